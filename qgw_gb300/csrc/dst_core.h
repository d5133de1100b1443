// dst_core.h -- building blocks of the batched DST-I used by the PV
// inversion (the reference takes it from FFTW's RODFT00 plans,
// src/elliptic.h:63-66, executed at :101 and :131).
//
// Definition (FFTW RODFT00, unnormalised), length n = M-1, M = 2H, H a
// product of 2, 3, 5 and 7:
//     Y_k = 2 sum_{j=1}^{M-1} x_j sin(pi j k / M),   k = 1..M-1.
// Method (published: the sine transform through a half-length complex FFT,
// e.g. Press et al., Numerical Recipes, section 12.3):
//   1. y_0 = 0, y_j = (s_j + 1/2) x_j + (s_j - 1/2) x_{M-j},  s_j = sin(pi j/M)
//   2. Z = FFT_H(z),  z_m = y_{2m} + i y_{2m+1}          (Stockham autosort)
//   3. with A = Z_k, B = conj Z_{H-k}, (c, s) = (cos, sin)(2 pi k / M):
//        2R_k = (A+B).re + (c (A-B).im - s (A-B).re)
//        -2I_k = (c (A-B).re + s (A-B).im) - (A+B).im
//      Y_{2k} = -2 I_k,  Y_{2k+1} = R_0 + sum_{k'=1..k} 2 R_{k'} (prefix sum)
//
// Every function below is one independent work item of one phase; a phase
// may run its items in any order or in parallel (the CUDA kernels spread
// them over a thread block, the CPU unit test runs them in a loop).  Rows
// are stored contiguously: row r of a buffer starts at r * ld reals.
//
// Buffer formats (reals, every access through the padded index pr/pc):
//   input   x_j at index j (j = 1..M-1); index 0 is not read
//   work    H complex values = M reals (y_j at index j)
//   output  Y_k at index k (k = 1..M-1), index 0 = 0 -- the input format,
//           so a DST output can feed the next DST directly; the split
//           writes (Y_{2k}, 2 R_k) as one complex pair at complex index k.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define QGW_HD __host__ __device__ __forceinline__
#define QGW_HD_NOINLINE __host__ __device__ __noinline__
#define QGW_ALIGN(n) __align__(n)
#else
#define QGW_HD inline
#define QGW_HD_NOINLINE __attribute__((noinline))
#define QGW_ALIGN(n) alignas(n)
#endif

namespace qgw {

template <typename T> struct C2;
template <> struct QGW_ALIGN(16) C2<double> { double x, y; };
template <> struct QGW_ALIGN(8) C2<float> { float x, y; };

// fused multiply-add on both host and device
QGW_HD double fmaT(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}
QGW_HD float fmaT(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return __builtin_fmaf(a, b, c);
#endif
}

// Padded layout of a row buffer in shared memory: after every 128 bytes of
// data (2^LG complex values) come W complex pad slots -- one 16-byte slot
// for doubles (8 complex values per period), two 8-byte slots for floats
// (16 per period).  A warp's contiguous access then starts and ends inside
// whole 128-byte periods (one wavefront per 128 bytes), the stride-R stores
// of the first Stockham pass spread over all banks, and every 16-byte
// aligned group of reals stays contiguous and 16-byte aligned.
// Complex index e lives at pc<T>(e), real index i at pr<T>(i).
template <typename T> struct Pad {
  static constexpr int LG = sizeof(T) == 8 ? 3 : 4;  // log2 complex values per period
  static constexpr int W = sizeof(T) == 8 ? 1 : 2;   // pad slots (complex) per period
  static constexpr int P = 1 << LG;
};
template <typename T> QGW_HD int pc(int e) { return e + Pad<T>::W * (e >> Pad<T>::LG); }
template <typename T> QGW_HD int pr(int i) { return i + 2 * Pad<T>::W * (i >> (Pad<T>::LG + 1)); }
// reals occupied by a padded row of M reals (room for reals M and M+1, the
// last complex value of a real FFT), rounded up to whole 16-byte vectors so
// that every row of a buffer starts 16-byte aligned
template <typename T> QGW_HD int padded_len(int M) {
  const int n = pr<T>(M + 1) + 1;
  constexpr int V = 16 / (int)sizeof(T);
  return (n + V - 1) / V * V;
}

// Static shape of one DST length.
struct DstGeom {
  int M;          // DST length + 1 (>= 4; even unless blue)
  int H;          // complex FFT length: M / 2, or (blue) the chirp-z transform's L
  int npass;      // Stockham passes
  int radix[12];  // radix of each pass: 8s, then 4 or 2, then 3s, 5s, 7s; first pass has Ns = 1
  int chunk;      // prefix-sum chunk length (values per work item)
  int nchunk;     // ceil(H / chunk) (<= 32)
  int ok;         // 1 when H factors into 2, 3, 5 and 7
  int blue;       // 1: a length the half-length FFT cannot take (M odd, or M/2 with a
                  // prime factor above 7), run as a chirp-z (Bluestein) transform of
                  // power-of-two length L = H (dst_blue.h)
};

inline DstGeom make_geom(int M) {
  DstGeom g{};
  g.M = M;
  g.H = M / 2;
  int rem = g.H, p = 0;
  while (rem % 8 == 0 && rem >= 8) { g.radix[p++] = 8; rem /= 8; }
  if (rem % 4 == 0) { g.radix[p++] = 4; rem /= 4; }
  else if (rem % 2 == 0) { g.radix[p++] = 2; rem /= 2; }
  for (int f : {3, 5, 7})
    while (rem % f == 0 && p < 12) { g.radix[p++] = f; rem /= f; }
  g.npass = p;
  g.ok = (rem == 1 && M % 2 == 0 && M >= 4) ? 1 : 0;
  g.chunk = g.H < 8 ? g.H : (g.H >= 256 ? (g.H + 31) / 32 : 8);
  g.nchunk = g.chunk > 0 ? (g.H + g.chunk - 1) / g.chunk : 0;
  return g;
}

// Lengths the half-length transforms take: even, half-length a product of
// 2, 3, 5, 7
inline bool transform_length_ok(int M) { return M >= 4 && make_geom(M).ok == 1; }

// Geometry of the chirp-z form of DST length M >= 4: L the smallest power of
// two >= 2M - 1 (the cyclic convolution of M values with a chirp of 2M - 1
// values); make_geom_any: the half-length form where it applies, else this
inline DstGeom make_geom_blue(int M) {
  int L = 1;
  while (L < 2 * M - 1) L *= 2;
  DstGeom g = make_geom(2 * L);  // the radices of an L-point FFT
  g.M = M;
  g.blue = 1;
  g.chunk = 0;
  g.nchunk = 0;
  return g;
}
inline DstGeom make_geom_any(int M) { return transform_length_ok(M) ? make_geom(M) : make_geom_blue(M); }
// reals of one row buffer of a transform: M (padded) for the half-length
// form, L complex values for the chirp-z form
template <typename T> QGW_HD int row_len(const DstGeom& g) {
  return g.blue ? padded_len<T>(2 * g.H) : padded_len<T>(g.M);
}

// Twiddles of the Stockham passes with Ns > 1 in the order the passes read
// them: pass (R, Ns) holds w_H^(q k H/(Ns R)) at (Ns - R0) + (q-1) Ns + k for
// q = 1..R-1, k = 0..Ns-1 (R0 = the first radix; the pass sizes telescope,
// sum (R-1) Ns = H - R0), so the consecutive items k of a warp read
// consecutive entries.  tw holds the H values w_H^m in FP64 pairs; twp gets
// 2 (H - R0) values.
inline void fill_pass_twiddles(const DstGeom& g, const double* tw, double* twp) {
  if (g.npass == 0) return;
  const int R0 = g.radix[0];
  int Ns = R0;
  for (int p = 1; p < g.npass; ++p) {
    const int R = g.radix[p];
    for (int q = 1; q < R; ++q)
      for (int k = 0; k < Ns; ++k) {
        const int e = (Ns - R0) + (q - 1) * Ns + k;
        const int m = q * k * (g.H / (Ns * R));
        twp[2 * e] = tw[2 * m];
        twp[2 * e + 1] = tw[2 * m + 1];
      }
    Ns *= R;
  }
}

// Tables (host-computed in FP64, stored per real type):
//   tw[m]  = (cos, -sin)(2 pi m / H),            m < H     (FFT twiddles)
//   twp    = tw reordered per Stockham pass (fill_pass_twiddles)
//   pre[j] = (s_j + 1/2, s_j - 1/2), s_j = sin(pi j/M), j <= H
//   spl[k] = (cos, sin)(2 pi k / M),             k <= H/2
//   sj[j]  = s_j,                                j <= H
template <typename T> struct DstTables {
  const C2<T>* tw;
  const C2<T>* pre;
  const C2<T>* spl;
  const C2<T>* twp;
  const T* sj;  // s_j = sin(pi j/M), j <= H (the merged pre-processing pass)
  const C2<T>* twd;  // the one-warp transform (dst_warp.h, H = 256, 512): DIF twiddles
  const C2<T>* sjp;  // and (s_{2m}, s_{2m+1}), m < H
  const C2<T>* bc;   // chirp-z form (dst_blue.h): c_m = exp(i pi m^2 / 2M), m < M
  const C2<T>* bz;   // and the L-point FFT of the conjugate chirp
};

// Work-item loop of a block over nrows rows of n items each: f(r, i) for
// every row r and item i, spread over the block's threads; shifts when n is
// a power of two (the common case), one division per item otherwise.
#ifdef __CUDACC__
template <typename F>
__device__ __forceinline__ void block_items(int nrows, int n, F f) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  if ((n & (n - 1)) == 0) {
    const int lg = __ffs(n) - 1;
    for (int w = tid; w < (nrows << lg); w += nth) f(w >> lg, w & (n - 1));
  } else {
    for (int w = tid; w < nrows * n; w += nth) {
      const int r = w / n;
      f(r, w - r * n);
    }
  }
}
#endif

// ---- phase 1: pre-processing, items j = 1..H per row -------------------
// reads x (input format) of row r, writes y (work format) of row r.
template <typename T>
QGW_HD void dst_pre_item(const T* __restrict__ x, T* __restrict__ y, int j, const DstGeom& g,
                         const C2<T>* __restrict__ pre) {
  const T a = x[pr<T>(j)];
  const T b = x[pr<T>(g.M - j)];
  const C2<T> w = pre[j];
  y[pr<T>(j)] = fmaT(w.x, a, w.y * b);
  y[pr<T>(g.M - j)] = fmaT(w.y, a, w.x * b);
  if (j == 1) y[0] = T(0);
}

// ---- phase 2: Stockham radix-R pass, items b = 0..H/R-1 per row ---------
template <typename T> QGW_HD C2<T> cmul(C2<T> a, C2<T> w) {
  C2<T> r;
  r.x = fmaT(a.x, w.x, -(a.y * w.y));
  r.y = fmaT(a.x, w.y, a.y * w.x);
  return r;
}
template <typename T> QGW_HD C2<T> cadd(C2<T> a, C2<T> b) { C2<T> r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename T> QGW_HD C2<T> csub(C2<T> a, C2<T> b) { C2<T> r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// -i * a
template <typename T> QGW_HD C2<T> cmi(C2<T> a) { C2<T> r; r.x = a.y; r.y = -a.x; return r; }

template <typename T> QGW_HD void dft2(C2<T>* v) {
  const C2<T> a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <typename T> QGW_HD void dft4(C2<T>* v) {
  const C2<T> c0 = cadd(v[0], v[2]), c1 = csub(v[0], v[2]);
  const C2<T> d0 = cadd(v[1], v[3]), d1 = cmi(csub(v[1], v[3]));
  v[0] = cadd(c0, d0);
  v[2] = csub(c0, d0);
  v[1] = cadd(c1, d1);
  v[3] = csub(c1, d1);
}

// forward DFT of length 8 (52 real operations with FMA)
template <typename T> QGW_HD void dft8(C2<T>* v) {
  const T s = T(0.70710678118654752440);
  C2<T> a[4], b[4];
  for (int r = 0; r < 4; ++r) { a[r] = cadd(v[r], v[r + 4]); b[r] = csub(v[r], v[r + 4]); }
  // even outputs: DFT4(a)
  {
    const C2<T> c0 = cadd(a[0], a[2]), c1 = csub(a[0], a[2]);
    const C2<T> d0 = cadd(a[1], a[3]), d1 = cmi(csub(a[1], a[3]));
    v[0] = cadd(c0, d0);
    v[4] = csub(c0, d0);
    v[2] = cadd(c1, d1);
    v[6] = csub(c1, d1);
  }
  // odd outputs: DFT4(b0, W b1, W^2 b2, W^3 b3), W = (1 - i)/sqrt 2,
  // with the 1/sqrt 2 folded into the final FMAs
  {
    C2<T> p1, p3;
    p1.x = b[1].x + b[1].y; p1.y = b[1].y - b[1].x;     // sqrt2 * W b1
    p3.x = b[3].y - b[3].x; p3.y = -(b[3].x + b[3].y);  // sqrt2 * W^3 b3
    const C2<T> u2 = cmi(b[2]);
    const C2<T> c0 = cadd(b[0], u2), c1 = csub(b[0], u2);
    const C2<T> P = cadd(p1, p3), D = csub(p1, p3);
    // X1 = c0 + s P, X5 = c0 - s P, X3 = c1 - i s D, X7 = c1 + i s D
    v[1].x = fmaT(s, P.x, c0.x);  v[1].y = fmaT(s, P.y, c0.y);
    v[5].x = fmaT(-s, P.x, c0.x); v[5].y = fmaT(-s, P.y, c0.y);
    v[3].x = fmaT(s, D.y, c1.x);  v[3].y = fmaT(-s, D.x, c1.y);
    v[7].x = fmaT(-s, D.y, c1.x); v[7].y = fmaT(s, D.x, c1.y);
  }
}

// Radix-8 butterfly whose inputs 1..7 carry twiddles w[1..7]: the products
// are folded into the first butterfly layer with FMAs, using
// x_r - w y = 2 x_r - (x_r + w y) for the difference outputs.
template <typename T> QGW_HD void dft8_tw(C2<T>* v, const C2<T>* w) {
  C2<T> a[4], b[4];
  {
    // r = 0: x_0 has no twiddle
    const C2<T> y = v[4], t = w[4];
    a[0].x = fmaT(y.x, t.x, fmaT(-y.y, t.y, v[0].x));
    a[0].y = fmaT(y.x, t.y, fmaT(y.y, t.x, v[0].y));
    b[0].x = fmaT(T(2), v[0].x, -a[0].x);
    b[0].y = fmaT(T(2), v[0].y, -a[0].y);
  }
#pragma unroll
  for (int r = 1; r < 4; ++r) {
    const C2<T> xr = cmul(v[r], w[r]);
    const C2<T> y = v[r + 4], t = w[r + 4];
    a[r].x = fmaT(y.x, t.x, fmaT(-y.y, t.y, xr.x));
    a[r].y = fmaT(y.x, t.y, fmaT(y.y, t.x, xr.y));
    b[r].x = fmaT(T(2), xr.x, -a[r].x);
    b[r].y = fmaT(T(2), xr.y, -a[r].y);
  }
  const T s = T(0.70710678118654752440);
  {
    const C2<T> c0 = cadd(a[0], a[2]), c1 = csub(a[0], a[2]);
    const C2<T> d0 = cadd(a[1], a[3]), d1 = cmi(csub(a[1], a[3]));
    v[0] = cadd(c0, d0);
    v[4] = csub(c0, d0);
    v[2] = cadd(c1, d1);
    v[6] = csub(c1, d1);
  }
  {
    C2<T> p1, p3;
    p1.x = b[1].x + b[1].y; p1.y = b[1].y - b[1].x;
    p3.x = b[3].y - b[3].x; p3.y = -(b[3].x + b[3].y);
    const C2<T> u2 = cmi(b[2]);
    const C2<T> c0 = cadd(b[0], u2), c1 = csub(b[0], u2);
    const C2<T> P = cadd(p1, p3), D = csub(p1, p3);
    v[1].x = fmaT(s, P.x, c0.x);  v[1].y = fmaT(s, P.y, c0.y);
    v[5].x = fmaT(-s, P.x, c0.x); v[5].y = fmaT(-s, P.y, c0.y);
    v[3].x = fmaT(s, D.y, c1.x);  v[3].y = fmaT(-s, D.x, c1.y);
    v[7].x = fmaT(-s, D.y, c1.x); v[7].y = fmaT(s, D.x, c1.y);
  }
}

// forward DFTs of odd length (the published symmetric forms: outputs k and
// R-k share the sums over x_n + x_{R-n} and the differences x_n - x_{R-n})
template <typename T> QGW_HD void dft3(C2<T>* v) {
  const T s = T(0.86602540378443864676);  // sin(2 pi / 3)
  const C2<T> t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
  C2<T> m;
  m.x = fmaT(T(-0.5), t.x, v[0].x);
  m.y = fmaT(T(-0.5), t.y, v[0].y);
  v[0] = cadd(v[0], t);
  // y1 = m - i s d, y2 = m + i s d
  v[1].x = fmaT(s, d.y, m.x);  v[1].y = fmaT(-s, d.x, m.y);
  v[2].x = fmaT(-s, d.y, m.x); v[2].y = fmaT(s, d.x, m.y);
}
template <typename T> QGW_HD void dft5(C2<T>* v) {
  const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);  // cos(2 pi/5), cos(4 pi/5)
  const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);   // sin(2 pi/5), sin(4 pi/5)
  const C2<T> t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const C2<T> d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  C2<T> a, b, p, q;
  a.x = fmaT(c2, t2.x, fmaT(c1, t1.x, v[0].x)); a.y = fmaT(c2, t2.y, fmaT(c1, t1.y, v[0].y));
  b.x = fmaT(c1, t2.x, fmaT(c2, t1.x, v[0].x)); b.y = fmaT(c1, t2.y, fmaT(c2, t1.y, v[0].y));
  p.x = fmaT(s2, d2.x, s1 * d1.x); p.y = fmaT(s2, d2.y, s1 * d1.y);     // s1 d1 + s2 d2
  q.x = fmaT(-s1, d2.x, s2 * d1.x); q.y = fmaT(-s1, d2.y, s2 * d1.y);   // s2 d1 - s1 d2
  v[0] = cadd(v[0], cadd(t1, t2));
  // y1 = a - i p, y4 = a + i p, y2 = b - i q, y3 = b + i q
  v[1].x = a.x + p.y; v[1].y = a.y - p.x;
  v[4].x = a.x - p.y; v[4].y = a.y + p.x;
  v[2].x = b.x + q.y; v[2].y = b.y - q.x;
  v[3].x = b.x - q.y; v[3].y = b.y + q.x;
}
template <typename T> QGW_HD void dft7(C2<T>* v) {
  // cos and sin of 2 pi n / 7, n = 1, 2, 3
  const T c[3] = {T(0.62348980185873353053), T(-0.22252093395631440429), T(-0.90096886790241912624)};
  const T s[3] = {T(0.78183148246802980871), T(0.97492791218182360702), T(0.43388373911755812048)};
  C2<T> t[3], d[3];
  for (int n = 0; n < 3; ++n) { t[n] = cadd(v[n + 1], v[6 - n]); d[n] = csub(v[n + 1], v[6 - n]); }
  C2<T> y[7];
  y[0] = cadd(v[0], cadd(t[0], cadd(t[1], t[2])));
  for (int k = 1; k <= 3; ++k) {
    C2<T> a = v[0], p;
    p.x = T(0); p.y = T(0);
    for (int n = 1; n <= 3; ++n) {
      const int e = (n * k) % 7;                 // angle index of w^(n k)
      const T cn = e <= 3 ? c[e - 1] : c[7 - e - 1];
      const T sn = e <= 3 ? s[e - 1] : -s[7 - e - 1];
      a.x = fmaT(cn, t[n - 1].x, a.x); a.y = fmaT(cn, t[n - 1].y, a.y);
      p.x = fmaT(sn, d[n - 1].x, p.x); p.y = fmaT(sn, d[n - 1].y, p.y);
    }
    // y_k = a - i p, y_{7-k} = a + i p
    y[k].x = a.x + p.y; y[k].y = a.y - p.x;
    y[7 - k].x = a.x - p.y; y[7 - k].y = a.y + p.x;
  }
  for (int k = 0; k < 7; ++k) v[k] = y[k];
}

// One Stockham autosort pass of radix R over a row (Govindaraju et al.'s
// formulation, any mix of radices): item b reads b + q H/R, k = b mod Ns,
// multiplies by w_H^(q k H/(Ns R)) and writes (b - k) R + k + q Ns.
// k = b mod Ns and hs = H / (Ns R) come from the caller (uniform per pass).
template <int R, typename T>
QGW_HD void stockham_item_k(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst, int b, int k, int Ns, int H,
                            int hs, const C2<T>* __restrict__ tw) {
  const int stride = H / R;
  C2<T> v[R];
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = src[pc<T>(b + q * stride)];
  if (Ns > 1) {
    const int step = k * hs;
    if (R == 8) {
      C2<T> w[8];
#pragma unroll
      for (int q = 1; q < 8; ++q) w[q] = tw[q * step];
      dft8_tw(v, w);
    } else {
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tw[q * step]);
      if (R == 4) dft4(v);
      else if (R == 2) dft2(v);
      else if (R == 3) dft3(v);
      else if (R == 5) dft5(v);
      else dft7(v);
    }
  } else {
    if (R == 8) dft8(v);
    else if (R == 4) dft4(v);
    else if (R == 2) dft2(v);
    else if (R == 3) dft3(v);
    else if (R == 5) dft5(v);
    else dft7(v);
  }
  const int base = (b - k) * R + k;
#pragma unroll
  for (int q = 0; q < R; ++q) dst[pc<T>(base + q * Ns)] = v[q];
}

// the odd radices as separate functions: their registers do not weigh on
// the power-of-two paths the kernels inline
template <int R, typename T>
QGW_HD_NOINLINE void stockham_item_odd(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst, int b, int k, int Ns,
                                       int H, int hs, const C2<T>* __restrict__ tw) {
  stockham_item_k<R, T>(src, dst, b, k, Ns, H, hs, tw);
}
template <typename T>
QGW_HD void stockham_dispatch_k(int R, const C2<T>* src, C2<T>* dst, int b, int k, int Ns, int H, int hs,
                                const C2<T>* tw) {
  switch (R) {
    case 8: stockham_item_k<8, T>(src, dst, b, k, Ns, H, hs, tw); break;
    case 4: stockham_item_k<4, T>(src, dst, b, k, Ns, H, hs, tw); break;
    case 2: stockham_item_k<2, T>(src, dst, b, k, Ns, H, hs, tw); break;
    case 3: stockham_item_odd<3, T>(src, dst, b, k, Ns, H, hs, tw); break;
    case 5: stockham_item_odd<5, T>(src, dst, b, k, Ns, H, hs, tw); break;
    default: stockham_item_odd<7, T>(src, dst, b, k, Ns, H, hs, tw); break;
  }
}
template <typename T>
QGW_HD void stockham_dispatch(int R, const C2<T>* src, C2<T>* dst, int b, int Ns, int H, const C2<T>* tw) {
  stockham_dispatch_k<T>(R, src, dst, b, b % Ns, Ns, H, H / (Ns * R), tw);
}

#ifdef __CUDACC__
// one Stockham pass of radix R over nrows rows by the whole block
template <typename T>
__device__ __forceinline__ void stockham_pass_block(int R, const T* src, T* dst, int nrows, int ld, int Ns, int H,
                                                    const C2<T>* tw) {
  const int hs = H / (Ns * R);
  if ((Ns & (Ns - 1)) == 0) {
    block_items(nrows, H / R, [&](int r, int b) {
      stockham_dispatch_k<T>(R, (const C2<T>*)(src + r * ld), (C2<T>*)(dst + r * ld), b, b & (Ns - 1), Ns, H, hs,
                             tw);
    });
  } else {
    block_items(nrows, H / R, [&](int r, int b) {
      stockham_dispatch_k<T>(R, (const C2<T>*)(src + r * ld), (C2<T>*)(dst + r * ld), b, b % Ns, Ns, H, hs, tw);
    });
  }
}
#endif

// ---- phase 3: split, items k = 0..H/2 per row --------------------------
// reads the FFT result Z (work format) and writes the output format, with
// the odd outputs still as increments (2R_k at index 2k+1; R_0 at index 1),
// each (Y_{2k}, 2R_k) pair as one complex value at complex index k.
template <typename T>
QGW_HD void dst_split_item(const C2<T>* __restrict__ Z, T* __restrict__ out, int k, const DstGeom& g,
                           const C2<T>* __restrict__ spl) {
  const int H = g.H;
  C2<T>* o = (C2<T>*)out;
  if (k == 0) {
    const C2<T> a = Z[0];
    C2<T> z0;
    z0.x = T(0);       // index 0 (no output)
    z0.y = a.x + a.y;  // R_0
    o[0] = z0;
    return;
  }
  const C2<T> A = Z[pc<T>(k)];
  const C2<T> Bc = Z[pc<T>(H - k)];
  const T br = Bc.x, bi = -Bc.y;
  const C2<T> cs = spl[k];
  const T sr = A.x + br, si = A.y + bi, dr = A.x - br, di = A.y - bi;
  const T P = fmaT(cs.x, di, -(cs.y * dr));
  const T Q = fmaT(cs.x, dr, cs.y * di);
  C2<T> lo;
  lo.x = Q - si;  // Y_{2k} = -2 I_k
  lo.y = sr + P;  // 2 R_k
  o[pc<T>(k)] = lo;
  if (2 * k != H) {
    C2<T> hi;
    hi.x = Q + si;  // Y_{2(H-k)}
    hi.y = sr - P;  // 2 R_{H-k}
    o[pc<T>(H - k)] = hi;
  }
}

// ---- phase 4: prefix sum of the odd outputs (indices 1, 3, 5, ...) ------
// 4a: items c = 0..nchunk-1: inclusive scan inside chunk c, returns total
template <typename T>
QGW_HD T dst_scan_chunk(T* out, int c, const DstGeom& g) {
  T acc = T(0);
  const int k0 = c * g.chunk;
  const int n = g.H - k0 < g.chunk ? g.H - k0 : g.chunk;  // the last chunk may be short
  acc = out[pr<T>(2 * k0 + 1)];
  for (int t = 1; t < n; ++t) {
    acc = acc + out[pr<T>(2 * (k0 + t) + 1)];
    out[pr<T>(2 * (k0 + t) + 1)] = acc;
  }
  return acc;
}
// 4c: items c = 1..nchunk-1: add the exclusive prefix of chunk totals
template <typename T>
QGW_HD void dst_scan_fix(T* out, int c, T prefix, const DstGeom& g) {
  const int k0 = c * g.chunk;
  const int n = g.H - k0 < g.chunk ? g.H - k0 : g.chunk;
  for (int t = 0; t < n; ++t) out[pr<T>(2 * (k0 + t) + 1)] += prefix;
}

}  // namespace qgw
