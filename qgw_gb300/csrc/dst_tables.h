// dst_tables.h -- host construction of the DST-I tables of dst_core.h, in
// FP64 with exactly reduced angles (one libm rounding per entry).
#pragma once

#include <cmath>
#include <vector>

#include "dst_core.h"

namespace qgw {

// sin(pi * m / N) for integer m, reduced exactly to [0, pi/2]
inline double sinpi_frac(long m, long N) {
  long r = m % (2 * N);
  if (r < 0) r += 2 * N;
  double sg = 1.0;
  if (r >= N) { r -= N; sg = -1.0; }
  if (2 * r > N) r = N - r;
  return sg * std::sin(M_PI * (double)r / (double)N);
}
// cos(pi m / N) = sin(pi (2m + N) / (2N))
inline double cospi_frac(long m, long N) { return sinpi_frac(2 * m + N, 2 * N); }

struct DstTablesHost {
  std::vector<double> tw, pre, spl, twp;  // interleaved (x, y) pairs
  std::vector<double> sj;                 // sin(pi j / M), j = 0..H
  // the warp transform's tables (H = 256, 512; one dummy pair otherwise):
  std::vector<double> twd;  // DIF twiddles: w_H^(n1 k2) at (k2-1) S0 + n1, then w_H^(8 n1 k2) at 7 S0 + (k2-1) S1 + n1
  std::vector<double> sjp;  // (s_{2m}, s_{2m+1}), m < H
};

// tw: H entries, twp: H - R0 entries, pre: H+1 entries, spl: H/2+1 entries
inline DstTablesHost build_dst_tables(int M) {
  const int H = M / 2;
  DstTablesHost t;
  t.tw.resize(2 * (size_t)H);
  for (int m = 0; m < H; ++m) {
    // 2 pi m / H = pi (2m) / H
    t.tw[2 * m] = cospi_frac(2L * m, H);
    t.tw[2 * m + 1] = -sinpi_frac(2L * m, H);
  }
  const DstGeom g = make_geom(M);
  t.twp.assign(2 * (size_t)(g.npass ? H - g.radix[0] : 0) + 2, 0.0);
  fill_pass_twiddles(g, t.tw.data(), t.twp.data());
  t.pre.resize(2 * (size_t)(H + 1));
  t.sj.resize((size_t)H + 1);
  for (int j = 0; j <= H; ++j) {
    const double s = sinpi_frac(j, M);
    t.pre[2 * j] = s + 0.5;
    t.pre[2 * j + 1] = s - 0.5;
    t.sj[j] = s;
  }
  t.spl.resize(2 * (size_t)(H / 2 + 1));
  for (int k = 0; k <= H / 2; ++k) {
    t.spl[2 * k] = cospi_frac(2L * k, M);
    t.spl[2 * k + 1] = sinpi_frac(2L * k, M);
  }
  t.twd.assign(2, 0.0);
  t.sjp.assign(2, 0.0);
  if (H == 256 || H == 512) {
    const int S0 = H / 8, S1 = H / 64;
    t.twd.assign(2 * (size_t)7 * (S0 + S1), 0.0);
    for (int k2 = 1; k2 < 8; ++k2) {
      for (int n1 = 0; n1 < S0; ++n1) {
        const int e = (k2 - 1) * S0 + n1, m = (n1 * k2) % H;
        t.twd[2 * e] = t.tw[2 * m];
        t.twd[2 * e + 1] = t.tw[2 * m + 1];
      }
      for (int n1 = 0; n1 < S1; ++n1) {
        const int e = 7 * S0 + (k2 - 1) * S1 + n1, m = (8 * n1 * k2) % H;
        t.twd[2 * e] = t.tw[2 * m];
        t.twd[2 * e + 1] = t.tw[2 * m + 1];
      }
    }
    t.sjp.resize(2 * (size_t)H);
    for (int m = 0; m < H; ++m) {
      const int j0 = 2 * m, j1 = 2 * m + 1;
      t.sjp[2 * m] = t.sj[j0 <= H ? j0 : M - j0];
      t.sjp[2 * m + 1] = t.sj[j1 <= H ? j1 : M - j1];
    }
  }
  return t;
}

}  // namespace qgw
