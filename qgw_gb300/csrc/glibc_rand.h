// glibc_rand.h -- the pseudo-random sequence of the C library's rand() as
// glibc implements it (random_r with the default TYPE_3 state: an additive
// lagged-Fibonacci generator of degree 31 and separation 3, seeded by the
// Park-Miller minimal-standard LCG, with 310 outputs discarded).  The
// reference draws its stochastic forcing from rand() (src/forcing.h:62-63,
// 184-186) without seeding it, i.e. from the seed-1 sequence; restating the
// published recurrence lets the GPU reproduce that noise exactly.
//   seeding:  s_0 = seed (0 -> 1),  s_i = 16807 s_{i-1} mod (2^31 - 1), i < 31
//   step:     s_f += s_r (mod 2^32), output s_f >> 1, f and r advance by one
//             (mod 31), starting at f = 3, r = 0
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define QGW_RAND_HD __host__ __device__ __forceinline__
#else
#define QGW_RAND_HD inline
#endif

namespace qgw {

struct GlibcRand {
  uint32_t s[31];
  int f, r;
};

QGW_RAND_HD uint32_t glibc_rand_next(GlibcRand* g) {
  const uint32_t v = g->s[g->f] + g->s[g->r];
  g->s[g->f] = v;
  g->f = g->f == 30 ? 0 : g->f + 1;
  g->r = g->r == 30 ? 0 : g->r + 1;
  return v >> 1;
}

QGW_RAND_HD void glibc_rand_seed(GlibcRand* g, uint32_t seed) {
  int32_t word = seed == 0 ? 1 : (int32_t)seed;
  g->s[0] = (uint32_t)word;
  for (int i = 1; i < 31; ++i) {
    // 16807 * word mod (2^31 - 1) without overflow (Schrage's method)
    const int32_t hi = word / 127773, lo = word % 127773;
    word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    g->s[i] = (uint32_t)word;
  }
  g->f = 3;
  g->r = 0;
  for (int k = 0; k < 310; ++k) (void)glibc_rand_next(g);
}

constexpr double GLIBC_RAND_MAX = 2147483647.0;

}  // namespace qgw
