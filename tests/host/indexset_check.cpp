// Host-side index-set logic of the engine, checked on the CPU (no GPU needed):
// kronecker(Iset, d) keeps the I index fastest (tensorci2.jl:315-320),
// kronecker(d, Jset) the local index fastest (:322-327), union keeps the first
// occurrence order (Base.union), select picks rows by pivot order, and
// pushunique! (util.jl:16-26) skips duplicates.
#include <cstdio>
#include <vector>

#include "engine.h"

using tci::IndexSet;

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAILED line %d: %s\n", __LINE__, #c);          \
      ++failures;                                                  \
    }                                                              \
  } while (0)

static IndexSet make(int len, std::vector<std::vector<int>> rows) {
  IndexSet s;
  s.len = len;
  for (auto& r : rows) {
    std::vector<uint8_t> b(r.begin(), r.end());
    if (len == 0)
      ++s.n;
    else
      s.push(b.data());
  }
  return s;
}

static std::vector<int> row(const IndexSet& s, size_t i) {
  std::vector<int> r;
  for (int q = 0; q < s.len; ++q) r.push_back(s.at(i)[q]);
  return r;
}

int main() {
  IndexSet I = make(2, {{0, 1}, {2, 0}});
  IndexSet K = tci::kron_right(I, 3);
  CHECK(K.len == 3 && K.n == 6);
  CHECK((row(K, 0) == std::vector<int>{0, 1, 0}));
  CHECK((row(K, 1) == std::vector<int>{2, 0, 0}));  // I index fastest
  CHECK((row(K, 2) == std::vector<int>{0, 1, 1}));
  CHECK((row(K, 5) == std::vector<int>{2, 0, 2}));

  IndexSet J = make(1, {{4}, {1}});
  IndexSet KL = tci::kron_left(2, J);
  CHECK(KL.len == 2 && KL.n == 4);
  CHECK((row(KL, 0) == std::vector<int>{0, 4}));
  CHECK((row(KL, 1) == std::vector<int>{1, 4}));  // local index fastest
  CHECK((row(KL, 2) == std::vector<int>{0, 1}));

  IndexSet A = make(2, {{1, 1}, {0, 3}, {2, 2}});
  IndexSet B = make(2, {{0, 3}, {5, 5}, {1, 1}, {7, 0}});
  IndexSet U = tci::set_union(A, B);
  CHECK(U.n == 5);
  CHECK((row(U, 0) == std::vector<int>{1, 1}));
  CHECK((row(U, 2) == std::vector<int>{2, 2}));
  CHECK((row(U, 3) == std::vector<int>{5, 5}));  // first-seen order
  CHECK((row(U, 4) == std::vector<int>{7, 0}));
  IndexSet E = make(0, {{}, {}});
  CHECK(tci::set_union(E, E).n == 1);  // all empty multi-indices are one

  const int32_t pick[3] = {2, 0, 4};
  IndexSet S = tci::select(U, pick, 3);
  CHECK(S.n == 3);
  CHECK((row(S, 0) == std::vector<int>{2, 2}));
  CHECK((row(S, 2) == std::vector<int>{7, 0}));

  IndexSet P = make(2, {{3, 3}});
  const uint8_t dup[2] = {3, 3}, fresh[2] = {1, 2};
  P.push_unique(dup);
  P.push_unique(fresh);
  CHECK(P.n == 2);

  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
