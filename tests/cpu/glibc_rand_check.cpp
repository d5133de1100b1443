// Host check of the restated C-library generator used by the GPU stochastic
// forcing (qgw_gb300/csrc/glibc_rand.h) against this machine's rand().
#include <cstdlib>

#include "../../qgw_gb300/csrc/glibc_rand.h"

// number of mismatches in the first n outputs after srand(seed)
extern "C" int glibc_rand_mismatches(unsigned seed, int n) {
  srand(seed);
  qgw::GlibcRand g;
  qgw::glibc_rand_seed(&g, seed);
  int bad = 0;
  for (int i = 0; i < n; ++i) bad += (unsigned)rand() != qgw::glibc_rand_next(&g);
  return bad;
}
