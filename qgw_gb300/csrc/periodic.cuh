// periodic.cuh -- the step kernels' transforms for the doubly periodic basin
// (bc_fac = -1).  The reference inverts with FFTW's in-place 2-D r2c / c2r
// (src/elliptic.h:32-47,103-118); here, with rows along y and x contiguous:
//   K1p: real FFT of each row (x) after the layer -> mode projection
//   K2p: complex FFT of each complex column (y), Helmholtz divide, inverse
//   K3p: spectral mode -> layer projection, inverse real FFT of each row
// The real FFT of length N = 2H runs as a complex FFT of length H on
// z_m = x_{2m} + i x_{2m+1} followed by the split
//   X_k = (P - i w^k Q) / 2,  X_{H-k} = conj((P + i w^k Q) / 2),
//   P = Z_k + conj Z_{H-k},  Q = Z_k - conj Z_{H-k},  w = exp(-2 pi i / N);
// the inverse (FFTW's unnormalised c2r) forms
//   Z'_k = P' + U,  Z'_{H-k} = conj(P' - U),  U = i Q' conj(w^k),
//   P' = X_k + conj X_{H-k},  Q' = X_k - conj X_{H-k},
// takes the backward FFT of Z' as conj(FFT(conj Z')) and reads
// x_{2m} = Re, x_{2m+1} = Im of the result.  The Stockham passes are the
// runtime-geometry ones of dst_core.h (mixed radix 2, 3, 5, 7).
#pragma once

#include "dst_core.h"
#include "dst_fixed.cuh"
#include "qgw_device.cuh"

namespace qgw {

// forward complex FFT of length g.H on nrows rows (complex values at pc<T>(e)
// of row r at A + r*ld); B is the work buffer; returns the output buffer.
// With the pass-ordered table twp, the lengths 256, 512 and 1024 (grids of
// 512^2 to 2048^2) run the compile-time passes of dst_fixed.cuh (the same
// arithmetic).
template <typename T>
__device__ __forceinline__ T* cfft_block(T* A, T* B, int nrows, int ld, const DstGeom& g, const C2<T>* tw,
                                         const C2<T>* twp = nullptr) {
  if (twp) {
    switch (g.H) {
      case 256: return cfft_block_fixed<T, 8>(A, B, nrows, ld, twp);
      case 512: return cfft_block_fixed<T, 9>(A, B, nrows, ld, twp);
      case 1024: return cfft_block_fixed<T, 10>(A, B, nrows, ld, twp);
      default: break;
    }
  }
  const int H = g.H;
  T* src = A;
  T* dst = B;
  int Ns = 1;
  for (int p = 0; p < g.npass; ++p) {
    const int R = g.radix[p];
    stockham_pass_block<T>(R, src, dst, nrows, ld, Ns, H, tw);
    __syncthreads();
    Ns *= R;
    T* t = src; src = dst; dst = t;
  }
  return src;
}

// Real FFT of rows of N = 2 g.H reals (x_i at pr<T>(i) of A), unnormalised:
// X_k, k = 0..H, at pc<T>(k) of the returned buffer.
template <typename T>
__device__ __forceinline__ T* rfft_block(T* A, T* B, int nrows, int ld, const DstGeom& g, const DstTables<T>& tb) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  const int H = g.H;
  T* Zb = cfft_block<T>(A, B, nrows, ld, g, tb.tw, tb.twp);
  T* Xb = (Zb == A) ? B : A;
  const int nk = H / 2 + 1;  // k = 0..H/2 pairs with H-k
  for (int w = tid; w < nrows * nk; w += nth) {
    const int r = w / nk, k = w - r * nk;
    const C2<T>* Z = (const C2<T>*)(Zb + r * ld);
    C2<T>* X = (C2<T>*)(Xb + r * ld);
    const C2<T> A1 = Z[pc<T>(k)];
    const C2<T> B1 = Z[pc<T>(k == 0 ? 0 : H - k)];  // Z_H = Z_0
    const T Pr = A1.x + B1.x, Pi = A1.y - B1.y;  // P = Z_k + conj Z_{H-k}
    const T Qr = A1.x - B1.x, Qi = A1.y + B1.y;  // Q = Z_k - conj Z_{H-k}
    const C2<T> cs = tb.spl[k];                  // (cos, sin)(2 pi k / N)
    // V = -i w^k Q with w^k = (c, -s)
    const T Vr = fmaT(cs.x, Qi, -(cs.y * Qr));
    const T Vi = -fmaT(cs.x, Qr, cs.y * Qi);
    C2<T> xk, xh;
    xk.x = T(0.5) * (Pr + Vr);
    xk.y = T(0.5) * (Pi + Vi);
    xh.x = T(0.5) * (Pr - Vr);
    xh.y = -(T(0.5) * (Pi - Vi));
    X[pc<T>(k)] = xk;
    if (k != H - k) X[pc<T>(H - k)] = xh;
  }
  __syncthreads();
  return Xb;
}

// Inverse real FFT (FFTW c2r, unnormalised) of rows holding X_k, k = 0..H,
// at pc<T>(k) of A; returns the buffer F with x_{2m} = F[pc<T>(m)].x and
// x_{2m+1} = -F[pc<T>(m)].y.  The imaginary parts of X_0 and X_H are ignored.
template <typename T>
__device__ __forceinline__ T* irfft_block(T* A, T* B, int nrows, int ld, const DstGeom& g, const DstTables<T>& tb) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  const int H = g.H;
  const int nk = H / 2 + 1;
  for (int w = tid; w < nrows * nk; w += nth) {
    const int r = w / nk, k = w - r * nk;
    const C2<T>* X = (const C2<T>*)(A + r * ld);
    C2<T>* Zc = (C2<T>*)(B + r * ld);
    C2<T> a = X[pc<T>(k)], b = X[pc<T>(H - k)];
    if (k == 0) { a.y = T(0); b.y = T(0); }
    const T Pr = a.x + b.x, Pi = a.y - b.y;  // P' = X_k + conj X_{H-k}
    const T Qr = a.x - b.x, Qi = a.y + b.y;  // Q' = X_k - conj X_{H-k}
    const C2<T> cs = tb.spl[k];
    // U = i Q' conj(w^k), conj(w^k) = (c, s): Q' (c, s) = (c Qr - s Qi, c Qi + s Qr)
    const T Wr = fmaT(cs.x, Qr, -(cs.y * Qi));
    const T Wi = fmaT(cs.x, Qi, cs.y * Qr);
    const T Ur = -Wi, Ui = Wr;
    // store conj(Z'_k) and conj(Z'_{H-k}) = P' - U (forward FFT of conj Z')
    C2<T> zk, zh;
    zk.x = Pr + Ur;
    zk.y = -(Pi + Ui);
    zh.x = Pr - Ur;
    zh.y = Pi - Ui;
    if (k < H) Zc[pc<T>(k)] = zk;
    if (k != H - k && k > 0) Zc[pc<T>(H - k)] = zh;
  }
  __syncthreads();
  return cfft_block<T>(B, A, nrows, ld, g, tb.tw, tb.twp);
}

}  // namespace qgw
