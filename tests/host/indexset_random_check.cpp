// The engine's index-set operations against direct restatements of their
// definitions, on randomized inputs that cover both union paths (multi-indices
// of up to 16 bytes as packed keys, longer ones byte-wise) and many duplicates:
//   kronecker(Iset, d): I index fastest (tensorci2.jl:315-320)
//   kronecker(d, Jset): local index fastest (:322-327)
//   union: first occurrences, in order (Base.union)
//   select: rows in pivot order
// Also the global-scratch sizes of the task layouts (tci_work_elems).
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "engine.h"

using tci::IndexSet;

namespace {
IndexSet naive_kron_right(const IndexSet& I, int d) {
  IndexSet o;
  o.len = I.len + 1;
  std::vector<uint8_t> b(o.len);
  for (int j = 0; j < d; ++j)
    for (size_t i = 0; i < I.n; ++i) {
      for (int q = 0; q < I.len; ++q) b[q] = I.at(i)[q];
      b[I.len] = (uint8_t)j;
      o.push(b.data());
    }
  return o;
}
IndexSet naive_kron_left(int d, const IndexSet& J) {
  IndexSet o;
  o.len = J.len + 1;
  std::vector<uint8_t> b(o.len);
  for (size_t j = 0; j < J.n; ++j)
    for (int i = 0; i < d; ++i) {
      b[0] = (uint8_t)i;
      for (int q = 0; q < J.len; ++q) b[1 + q] = J.at(j)[q];
      o.push(b.data());
    }
  return o;
}
IndexSet naive_union(const IndexSet& a, const IndexSet& b) {
  IndexSet o;
  o.len = a.len;
  if (a.len == 0) {
    if (a.n + b.n > 0) o.n = 1;
    return o;
  }
  for (const IndexSet* s : {&a, &b})
    for (size_t i = 0; i < s->n; ++i) {
      bool seen = false;
      for (size_t k = 0; k < o.n && !seen; ++k) seen = std::memcmp(o.at(k), s->at(i), (size_t)a.len) == 0;
      if (!seen) o.push(s->at(i));
    }
  return o;
}
IndexSet random_set(std::mt19937& g, int n, int len, int alphabet) {
  IndexSet s;
  s.len = len;
  std::vector<uint8_t> v((size_t)len + 1);
  for (int i = 0; i < n; ++i) {
    for (int q = 0; q < len; ++q) v[q] = (uint8_t)(g() % alphabet);
    if (len == 0)
      ++s.n;
    else
      s.push(v.data());
  }
  return s;
}
bool same(const IndexSet& x, const IndexSet& y) { return x.len == y.len && x.n == y.n && x.data == y.data; }
}  // namespace

int main() {
  std::mt19937 g(2024);
  int bad = 0;
  for (int t = 0; t < 4000; ++t) {
    const int len = (int)(g() % 21), d = 1 + (int)(g() % 12);
    const int alphabet = 1 + (int)(g() % 4);  // small alphabets: many duplicates
    IndexSet a = random_set(g, (int)(g() % 150), len, alphabet), b = random_set(g, (int)(g() % 80), len, alphabet);
    if (!same(tci::set_union(a, b), naive_union(a, b))) ++bad;
    if (!same(tci::kron_right(a, d), naive_kron_right(a, d))) ++bad;
    if (!same(tci::kron_left(d, a), naive_kron_left(d, a))) ++bad;
    if (a.n) {
      std::vector<int32_t> idx(1 + g() % 40);
      for (auto& x : idx) x = (int32_t)(g() % a.n);
      IndexSet sel = tci::select(a, idx.data(), (int)idx.size()), ref;
      ref.len = a.len;
      for (int32_t k : idx) {
        if (a.len == 0)
          ++ref.n;
        else
          ref.push(a.at((size_t)k));
      }
      if (!same(sel, ref)) ++bad;
    }
  }
  // global scratch of the task layouts: Π (m x n) or P (r x r), then the f
  // states when they live in global memory too
  tci_task t{};
  t.kind = TCI_TASK_RRLU;
  t.m = 300;
  t.n = 200;
  t.smem_mode = 1;
  if (tci_work_elems(&t) != 0) ++bad;
  t.smem_mode = 0;
  if (tci_work_elems(&t) != 300u * 200u) ++bad;
  t.smem_mode = 2;
  if (tci_work_elems(&t) != 300u * 200u + 2u * 500u) ++bad;
  t.kind = TCI_TASK_SITE;
  t.r = 40;
  t.m = 640;
  t.smem_mode = 0;
  if (tci_work_elems(&t) != 1600u) ++bad;
  t.smem_mode = 2;
  if (tci_work_elems(&t) != 1600u + 1280u) ++bad;
  t.kind = TCI_TASK_EVAL;
  if (tci_work_elems(&t) != 0) ++bad;
  if (bad) {
    std::printf("%d mismatches\n", bad);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
