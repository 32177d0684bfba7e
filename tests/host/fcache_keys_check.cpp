// Host-side key layout of the device value cache (fcache.h), checked on the CPU:
// mixed-radix weights with the first site fastest (CachedFunction's coeffs,
// cachedfunction.jl:16-19), split into two words where a word would pass 2^52,
// and the 2^104 limit.  FCache::init touches no device memory.
#include <cstdio>
#include <vector>

#include "fcache.h"

static int failures = 0;
#define CHECK(c)                                          \
  do {                                                    \
    if (!(c)) {                                           \
      std::printf("FAILED line %d: %s\n", __LINE__, #c); \
      ++failures;                                         \
    }                                                     \
  } while (0)

int main() {
  {  // 5 sites of 10: one word, weights 1, 10, 100, ...
    const int d[5] = {10, 10, 10, 10, 10};
    std::vector<double> params(4 + 5);
    tci::FCache c;
    CHECK(c.init(5, d, nullptr, nullptr, params.data()) == 0);
    CHECK(c.split == 5);
    CHECK(params[3] == 5.0);
    CHECK(params[4] == 1.0 && params[5] == 10.0 && params[8] == 10000.0);
    CHECK(params[2] == 0.0);  // no table yet: mask 0
  }
  {  // 60 sites of 2: 2^52 fits the first word (52 sites), the rest starts at 1
    std::vector<int> d(60, 2);
    std::vector<double> params(4 + 60);
    tci::FCache c;
    CHECK(c.init(60, d.data(), nullptr, nullptr, params.data()) == 0);
    CHECK(c.split == 52);
    CHECK(params[4 + 51] == 2251799813685248.0);  // 2^51
    CHECK(params[4 + 52] == 1.0 && params[4 + 59] == 128.0);
  }
  {  // 110 sites of 2 need more than two words: ArgumentError
    std::vector<int> d(110, 2);
    std::vector<double> params(4 + 110);
    tci::FCache c;
    CHECK(c.init(110, d.data(), nullptr, nullptr, params.data()) == TCI_ERR_ARG);
  }
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
