// dst_fixed.cuh -- the batched DST-I of dst_core.h specialised at compile
// time for one transform length (M = 2H = 2^(LGH+1)), used by the step
// kernels for the common lengths.  Same phases, same arithmetic as the
// generic block DST (kernels.cu), so results agree bit for bit with it:
//   pre-processing -> Stockham radix-8 passes (+ one radix-4/2 pass)
//   -> split -> prefix sum of the odd outputs.
// With the geometry fixed, every padded shared-memory index is one base
// computation plus immediate offsets (strides that are multiples of 8
// complex values keep the pad pattern: pc(e + 8m) = pc(e) + 9m), and the
// prefix sum runs one warp per row without block barriers.
#pragma once

#include "dst_core.h"

namespace qgw {

template <int LGH> struct DstShape {
  static constexpr int H = 1 << LGH, M = 2 * H;
  static constexpr int NP8 = LGH / 3;                 // radix-8 passes
  static constexpr int RLAST = 1 << (LGH % 3);        // 1: none, 2 or 4
  static constexpr int CHUNK = H >= 256 ? H / 32 : 8; // prefix-sum chunk
  static constexpr int NCHUNK = H / CHUNK;
  static_assert(LGH >= 6, "fixed DST needs H >= 64");
};

// one Stockham item: inputs b + q*(H/R), outputs base + q*NS
template <typename T, int R, int NS, int H>
__device__ __forceinline__ void stockham_fixed(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst, int b,
                                               const C2<T>* __restrict__ tw) {
  constexpr int S = H / R;
  static_assert(S % 8 == 0, "input stride must keep the pad pattern");
  static_assert(NS == 1 || NS % 8 == 0, "output stride must keep the pad pattern");
  C2<T> v[R];
  const C2<T>* s0 = src + pc(b);
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = s0[q * (S + S / 8)];
  const int k = b & (NS - 1);
  if constexpr (NS > 1) {
    const int step = k * (H / (NS * R));
    if constexpr (R == 8) {
      C2<T> w[8];
#pragma unroll
      for (int q = 1; q < 8; ++q) w[q] = tw[q * step];
      dft8_tw(v, w);
    } else {
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tw[q * step]);
      if constexpr (R == 4) dft4(v);
      else dft2(v);
    }
  } else {
    if constexpr (R == 8) dft8(v);
    else if constexpr (R == 4) dft4(v);
    else dft2(v);
  }
  const int base = (b - k) * R + k;
  C2<T>* d0 = dst + pc(base);
  constexpr int OS = NS == 1 ? 1 : NS + NS / 8;
#pragma unroll
  for (int q = 0; q < R; ++q) d0[q * OS] = v[q];
}

template <typename T, int R, int NS, int H>
__device__ __forceinline__ void stockham_pass_fixed(const T* src, T* dst, int nrows, int ld, const C2<T>* tw) {
  constexpr int NB = H / R;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  for (int w = tid; w < nrows * NB; w += nth) {
    const int r = w / NB, b = w & (NB - 1);
    stockham_fixed<T, R, NS, H>((const C2<T>*)(src + r * ld), (C2<T>*)(dst + r * ld), b, tw);
  }
}

template <typename T, int LGH>
__device__ T* dst_block_fixed(T* A, T* B, int nrows, int ld, const DstTables<T>& tb) {
  using S = DstShape<LGH>;
  constexpr int H = S::H, M = S::M;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  // phase 1: pre-processing, items j = 1..H per row (dst_pre_item)
  for (int w = tid; w < (nrows << LGH); w += nth) {
    const int r = w >> LGH, j = (w & (H - 1)) + 1;
    const T* x = A + r * ld;
    T* y = B + r * ld;
    const T a = x[pr(j - 1)];
    const T b = x[pr(M - j - 1)];
    const C2<T> wp = tb.pre[j];
    y[pr(j)] = fmaT(wp.x, a, wp.y * b);
    y[pr(M - j)] = fmaT(wp.y, a, wp.x * b);
    if (j == 1) y[0] = T(0);
  }
  __syncthreads();
  // phase 2: Stockham passes B -> A -> B ...
  T* src = B;
  T* dst = A;
  if constexpr (S::NP8 >= 1) {
    stockham_pass_fixed<T, 8, 1, H>(src, dst, nrows, ld, tb.tw);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::NP8 >= 2) {
    stockham_pass_fixed<T, 8, 8, H>(src, dst, nrows, ld, tb.tw);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::NP8 >= 3) {
    stockham_pass_fixed<T, 8, 64, H>(src, dst, nrows, ld, tb.tw);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  static_assert(S::NP8 <= 3, "fixed DST covers H <= 2048");
  if constexpr (S::RLAST > 1) {
    constexpr int NS = 1 << (3 * S::NP8);
    stockham_pass_fixed<T, S::RLAST, NS, H>(src, dst, nrows, ld, tb.tw);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  // phase 3: split (dst_split_item), items k = 0..H/2-1; item 0 also does H/2
  for (int w = tid; w < nrows * (H / 2); w += nth) {
    const int r = w / (H / 2), k = w & (H / 2 - 1);
    const C2<T>* Z = (const C2<T>*)(src + r * ld);
    T* out = dst + r * ld;
    if (k == 0) {
      const C2<T> a = Z[0];
      out[0] = a.x + a.y;
      const C2<T> A2 = Z[pc(H / 2)];
      const T br = A2.x, bi = -A2.y;
      const C2<T> cs = tb.spl[H / 2];
      const T sr = A2.x + br, si = A2.y + bi, dr = A2.x - br, di = A2.y - bi;
      const T P = fmaT(cs.x, di, -(cs.y * dr));
      const T Q = fmaT(cs.x, dr, cs.y * di);
      out[pr(H)] = sr + P;
      out[pr(H - 1)] = Q - si;
    } else {
      const C2<T> Av = Z[pc(k)];
      const C2<T> Bc = Z[pc(H - k)];
      const T br = Bc.x, bi = -Bc.y;
      const C2<T> cs = tb.spl[k];
      const T sr = Av.x + br, si = Av.y + bi, dr = Av.x - br, di = Av.y - bi;
      const T P = fmaT(cs.x, di, -(cs.y * dr));
      const T Q = fmaT(cs.x, dr, cs.y * di);
      out[pr(2 * k)] = sr + P;
      out[pr(2 * k - 1)] = Q - si;
      out[pr(2 * (H - k))] = sr - P;
      out[pr(2 * (H - k) - 1)] = Q + si;
    }
  }
  __syncthreads();
  // phase 4: prefix sum of the odd outputs (indices 0, 2, 4, ...): one warp
  // per row, lane c scans chunk c, the chunk totals are scanned by shuffles
  const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
  constexpr int CH = S::CHUNK, NC = S::NCHUNK;
  static_assert((2 * CH) % 16 == 0, "chunk start must be pad-aligned");
  for (int r = warp; r < nrows; r += nwarp) {
    T* o = dst + r * ld + pr(2 * CH * lane);
    T acc = T(0);
    if (lane < NC) {
      acc = o[0];
#pragma unroll
      for (int t = 1; t < CH; ++t) {
        acc = acc + o[2 * t + ((2 * t) >> 4) * 2];
        o[2 * t + ((2 * t) >> 4) * 2] = acc;
      }
    }
    T incl = acc;
#pragma unroll
    for (int of = 1; of < 32; of <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, incl, of);
      if (lane >= of) incl += u;
    }
    T ex = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane > 0 && lane < NC) {
#pragma unroll
      for (int t = 0; t < CH; ++t) o[2 * t + ((2 * t) >> 4) * 2] += ex;
    }
  }
  __syncthreads();
  return dst;
}

}  // namespace qgw
