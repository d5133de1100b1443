// dst_blue.h -- the DST-I of the lengths the half-length FFT cannot take
// (M odd, or M/2 with a prime factor above 7), as a chirp-z transform
// (Bluestein's algorithm, the published identity jk = (j^2 + k^2 - (k-j)^2)/2).
//
//   S_k = sum_{j<M} x_j exp(i pi j k / M),     Y_k = 2 Im S_k = RODFT00(x)_k,
//   S_k = c_k sum_j (x_j c_j) conj(c_{k-j}),    c_m = exp(i pi m^2 / 2M),
//
// the sum a cyclic convolution of length L (a power of two >= 2M - 1) done
// with two L-point FFTs: A = FFT(a), a_j = x_j c_j (zero for j = 0 and
// j >= M); D = FFT(conj(A * Bz)) with Bz = FFT(b), b_d = conj(c_|d|) at
// d mod L for |d| < M; conv = conj(D) / L.  Input x_j at real index j,
// output Y_k at real index k (dst_core.h's formats); the work buffers hold
// L complex values per row.  Each function is one work item (one (row,
// index) pair) that the device code spreads over a block and a CPU check
// runs in loops.  The chirp angles are reduced exactly (m^2 mod 4M) on the
// host, where the tables are made in FP64.
#pragma once

#include <cstddef>
#include <utility>
#include <vector>

#include "dst_tables.h"

namespace qgw {

// phase 1: a_m = x_m c_m, m < L (zero outside 1 <= m < M)
template <typename T>
QGW_HD void blue_chirp_item(const T* __restrict__ x, C2<T>* __restrict__ a, int m, int M,
                            const C2<T>* __restrict__ bc) {
  C2<T> v;
  v.x = T(0);
  v.y = T(0);
  if (m >= 1 && m < M) {
    const T xm = x[pr<T>(m)];
    const C2<T> c = bc[m];
    v.x = xm * c.x;
    v.y = xm * c.y;
  }
  a[pc<T>(m)] = v;
}
// phase 3 (after the first FFT): conj(A_k Bz_k), in place
template <typename T>
QGW_HD void blue_mul_item(C2<T>* z, int k, const C2<T>* __restrict__ bz) {
  C2<T> p = cmul(z[pc<T>(k)], bz[k]);
  p.y = -p.y;
  z[pc<T>(k)] = p;
}
// phase 5 (after the second FFT D): Y_k = 2 Im(c_k conj(D_k) / L), k < M
// (Y_0 = 0 at index 0)
template <typename T>
QGW_HD void blue_out_item(const C2<T>* __restrict__ d, T* __restrict__ y, int k, T invL,
                          const C2<T>* __restrict__ bc) {
  if (k == 0) {
    y[pr<T>(0)] = T(0);
    return;
  }
  const C2<T> dk = d[pc<T>(k)];
  const C2<T> c = bc[k];
  const T vx = dk.x * invL, vy = -dk.y * invL;
  y[pr<T>(k)] = T(2) * fmaT(c.y, vx, c.x * vy);
}

// Host tables of a chirp-z length (g = make_geom_any(M), g.blue): the chirp
// c_m (M pairs) and Bz (L pairs), interleaved (re, im), FP64.
inline void build_blue_tables(const DstGeom& g, std::vector<double>& bc, std::vector<double>& bz) {
  const int M = g.M, L = g.H;
  const long four_m = 4L * M;
  bc.assign(2 * (size_t)M, 0.0);
  for (int m = 0; m < M; ++m) {
    const long e = ((long)m * m) % four_m;  // exp(i pi e / 2M)
    bc[2 * m] = cospi_frac(e, 2L * M);
    bc[2 * m + 1] = sinpi_frac(e, 2L * M);
  }
  // b at d mod L, d in (-M, M): conj(c_|d|)
  std::vector<double> re((size_t)L, 0.0), im((size_t)L, 0.0);
  for (int d = -(M - 1); d < M; ++d) {
    const int ad = d < 0 ? -d : d;
    const int idx = ((d % L) + L) % L;
    re[idx] = bc[2 * ad];
    im[idx] = -bc[2 * ad + 1];
  }
  // forward FFT of length L (radix 2, decimation in time after a bit
  // reversal), twiddles exp(-2 pi i t / L) with exactly reduced angles
  for (int i = 1, j = 0; i < L; ++i) {
    int bit = L >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  for (int len = 2; len <= L; len <<= 1) {
    const int half = len / 2, stride = L / len;
    for (int i = 0; i < L; i += len)
      for (int t = 0; t < half; ++t) {
        const long e = 2L * t * stride;  // 2 pi t / len = pi e / L
        const double wr = cospi_frac(e, L), wi = -sinpi_frac(e, L);
        const size_t u = (size_t)(i + t), v = u + half;
        const double xr = re[v] * wr - im[v] * wi, xi = re[v] * wi + im[v] * wr;
        re[v] = re[u] - xr;
        im[v] = im[u] - xi;
        re[u] += xr;
        im[u] += xi;
      }
  }
  bz.assign(2 * (size_t)L, 0.0);
  for (int k = 0; k < L; ++k) {
    bz[2 * k] = re[k];
    bz[2 * k + 1] = im[k];
  }
}

}  // namespace qgw
