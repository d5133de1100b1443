// dst_fixed.cuh -- the batched DST-I of dst_core.h specialised at compile
// time for one transform length (M = 2H = 2^(LGH+1)), used by the step
// kernels for the common lengths, and its complex FFT alone (the periodic
// transforms).  Same phases and arithmetic as the generic block DST
// (step_device.cuh); the FP32 prefix sum runs here as a vector scan per lane
// (so FP32 results agree with the generic DST to round-off, FP64 ones and
// the FFT bit for bit):
//   pre-processing -> Stockham radix-8 passes (+ one radix-4/2 pass)
//   -> split -> prefix sum of the odd outputs.
// With the geometry fixed, a padded shared-memory index is one base
// computation plus compile-time offsets (StockhamItem), and the prefix sum
// runs one warp per row without block barriers.  The blocks have DST_NT threads and
// every phase has a power-of-two item count per row, so a thread meets the
// same in-row items in every row: their indices, table values and twiddles
// are computed once per transform, outside the row loop.
#pragma once

#include "dst_core.h"

namespace qgw {

constexpr int DST_NT = 256;  // threads per block of every kernel that calls dst_block_fixed

template <int LGH> struct DstShape {
  static constexpr int H = 1 << LGH, M = 2 * H;
  static constexpr int NP8 = LGH / 3;                 // radix-8 passes
  static constexpr int RLAST = 1 << (LGH % 3);        // 1: none, 2 or 4
  static_assert(LGH >= 6, "fixed DST needs H >= 64");
};

// One Stockham pass over all rows: item b of a row reads inputs b + q*(H/R)
// and writes outputs base + q*NS; the twiddles of item b are loaded once,
// from the pass-ordered table (consecutive items, consecutive entries).
// With R, NS, H/R and the pad period P all powers of two, adding q*stride to
// the item's base never carries across a pad period beyond what q*stride
// itself crosses (the base's offset inside its period plus that of q*stride
// stays below P), so pc(base + q*stride) = pc(base) + pc(q*stride): one
// padded base per item, compile-time offsets per q.
template <typename T, int R, int NS, int H>
struct StockhamItem {
  static constexpr int S = H / R;
  static constexpr int LG = Pad<T>::LG, W = Pad<T>::W;
  static constexpr int pco(int e) { return e + W * (e >> LG); }
  int in0, out0;
  C2<T> w[R];
  // twp: the pass-ordered twiddles (fill_pass_twiddles; first radix 8)
  __device__ __forceinline__ void init(int b, const C2<T>* __restrict__ twp) {
    in0 = pc<T>(b);
    const int k = b & (NS - 1);
    out0 = pc<T>((b - k) * R + k);
    if constexpr (NS > 1) {
#pragma unroll
      for (int q = 1; q < R; ++q) w[q] = twp[(NS - 8) + (q - 1) * NS + k];
    }
  }
  __device__ __forceinline__ void run(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst) const {
    C2<T> v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = src[in0 + pco(q * S)];
    if constexpr (NS > 1) {
      if constexpr (R == 8) {
        dft8_tw(v, w);
      } else {
#pragma unroll
        for (int q = 1; q < R; ++q) v[q] = cmul(v[q], w[q]);
        if constexpr (R == 4) dft4(v);
        else dft2(v);
      }
    } else {
      if constexpr (R == 8) dft8(v);
      else if constexpr (R == 4) dft4(v);
      else dft2(v);
    }
#pragma unroll
    for (int q = 0; q < R; ++q) dst[out0 + pco(q * NS)] = v[q];
  }
};

template <typename T, int R, int NS, int H>
__device__ __forceinline__ void stockham_pass_fixed(const T* src, T* dst, int nrows, int ld, const C2<T>* tw) {
  constexpr int NB = H / R;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  if constexpr (NB < DST_NT) {
    StockhamItem<T, R, NS, H> it;
    it.init(tid & (NB - 1), tw);
    for (int r = tid / NB; r < nrows; r += DST_NT / NB)
      it.run((const C2<T>*)(src + r * ld), (C2<T>*)(dst + r * ld));
  } else {
    constexpr int C = NB / DST_NT;
    StockhamItem<T, R, NS, H> it[C];
#pragma unroll
    for (int c = 0; c < C; ++c) it[c].init(tid + c * DST_NT, tw);
    for (int r = 0; r < nrows; ++r)
#pragma unroll
      for (int c = 0; c < C; ++c) it[c].run((const C2<T>*)(src + r * ld), (C2<T>*)(dst + r * ld));
  }
}

// The complex FFT of H = 2^LGH points (the Stockham passes alone) on nrows
// rows by the whole block: input in X, Y the second buffer; returns the
// buffer that holds the output.  The same passes and arithmetic as the
// runtime-geometry loops of dst_core.h (bit-identical results).
template <typename T, int LGH>
__device__ T* cfft_block_fixed(T* X, T* Y, int nrows, int ld, const C2<T>* __restrict__ twp) {
  using S = DstShape<LGH>;
  constexpr int H = S::H;
  static_assert(S::NP8 <= 3, "fixed passes cover H <= 4096");
  T* src = X;
  T* dst = Y;
  if constexpr (S::NP8 >= 1) {
    stockham_pass_fixed<T, 8, 1, H>(src, dst, nrows, ld, twp);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::NP8 >= 2) {
    stockham_pass_fixed<T, 8, 8, H>(src, dst, nrows, ld, twp);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::NP8 >= 3) {
    stockham_pass_fixed<T, 8, 64, H>(src, dst, nrows, ld, twp);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::RLAST > 1) {
    constexpr int NS = 1 << (3 * S::NP8);
    stockham_pass_fixed<T, S::RLAST, NS, H>(src, dst, nrows, ld, twp);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  return src;
}

template <typename T, int LGH>
__device__ T* dst_block_fixed(T* A, T* B, int nrows, int ld, const DstTables<T>& tb) {
  using S = DstShape<LGH>;
  constexpr int H = S::H, M = S::M;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  // phase 1: pre-processing, items j = 1..H per row (dst_pre_item); thread
  // tid handles j = tid + 1 + c * DST_NT of every row
  static_assert(H % DST_NT == 0 || DST_NT % H == 0, "power-of-two shapes");
  if constexpr (H >= DST_NT) {
    constexpr int C = H / DST_NT;
    int ia[C], ib[C], oa[C], ob[C];
    C2<T> wp[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int j = tid + 1 + c * DST_NT;
      ia[c] = pr<T>(j - 1);
      ib[c] = pr<T>(M - j - 1);
      oa[c] = pr<T>(j);
      ob[c] = pr<T>(M - j);
      wp[c] = tb.pre[j];
    }
    for (int r = 0; r < nrows; ++r) {
      const T* x = A + r * ld;
      T* y = B + r * ld;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const T a = x[ia[c]], b = x[ib[c]];
        y[oa[c]] = fmaT(wp[c].x, a, wp[c].y * b);
        y[ob[c]] = fmaT(wp[c].y, a, wp[c].x * b);
      }
      if (tid == 0) y[0] = T(0);
    }
  } else {
    const int j = (tid & (H - 1)) + 1;
    const int ia = pr<T>(j - 1), ib = pr<T>(M - j - 1), oa = pr<T>(j), ob = pr<T>(M - j);
    const C2<T> wp = tb.pre[j];
    for (int r = tid >> LGH; r < nrows; r += DST_NT / H) {
      const T* x = A + r * ld;
      T* y = B + r * ld;
      const T a = x[ia], b = x[ib];
      y[oa] = fmaT(wp.x, a, wp.y * b);
      y[ob] = fmaT(wp.y, a, wp.x * b);
      if (j == 1) y[0] = T(0);
    }
  }
  __syncthreads();
  // phase 2: Stockham passes B -> A -> B ...
  T* src = cfft_block_fixed<T, LGH>(B, A, nrows, ld, tb.twp);
  T* dst = src == A ? B : A;
  // phase 3: split (dst_split_item), items k = 0..H/2-1; item 0 also does
  // k = H/2 (and R_0); thread tid handles k = tid + c * DST_NT of every row
  {
    constexpr int KI = H / 2;
    constexpr int C = KI >= DST_NT ? KI / DST_NT : 1;
    constexpr int RS = KI >= DST_NT ? 1 : DST_NT / KI;
    const int kb = KI >= DST_NT ? tid : (tid & (KI - 1));
    int za[C], zb[C], o0[C], o1[C], o2[C], o3[C];
    C2<T> cs[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int k = kb + c * DST_NT;
      const int kk = k == 0 ? H / 2 : k;  // item 0 runs the k = H/2 butterfly
      za[c] = pc<T>(kk);
      zb[c] = pc<T>(H - kk);
      o0[c] = pr<T>(2 * kk);
      o1[c] = pr<T>(2 * kk - 1);
      o2[c] = pr<T>(2 * (H - kk));
      o3[c] = pr<T>(2 * (H - kk) - 1);
      cs[c] = tb.spl[kk];
    }
    for (int r = KI >= DST_NT ? 0 : tid / KI; r < nrows; r += RS) {
      const C2<T>* Z = (const C2<T>*)(src + r * ld);
      T* out = dst + r * ld;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const C2<T> Av = Z[za[c]];
        const C2<T> Bc = Z[zb[c]];
        const T br = Bc.x, bi = -Bc.y;
        const T sr = Av.x + br, si = Av.y + bi, dr = Av.x - br, di = Av.y - bi;
        const T P = fmaT(cs[c].x, di, -(cs[c].y * dr));
        const T Q = fmaT(cs[c].x, dr, cs[c].y * di);
        out[o0[c]] = sr + P;
        out[o1[c]] = Q - si;
        if (kb + c * DST_NT != 0) {
          out[o2[c]] = sr - P;
          out[o3[c]] = Q + si;
        } else {
          const C2<T> a = Z[0];
          out[0] = a.x + a.y;  // R_0
        }
      }
    }
  }
  __syncthreads();
  // phase 4: prefix sum of the odd outputs (indices 0, 2, 4, ...), one warp
  // per row.
  if constexpr (sizeof(T) == 8) {
    // FP64 (the FP64 pipe bounds these kernels, so the fewest additions):
    // lane c scans chunk c sequentially, the chunk totals are scanned by
    // shuffles and added back -- two additions per value
    constexpr int CH = H >= 256 ? H / 32 : 8, NC = H / CH;
    static_assert((2 * CH) % (2 * Pad<T>::P) == 0, "chunk start must be pad-aligned");
    const int warp = tid >> 5, lane = tid & 31, nwarp = DST_NT >> 5;
    for (int r = warp; r < nrows; r += nwarp) {
      T* o = dst + r * ld + pr<T>(2 * CH * lane);
      T acc = T(0);
      if (lane < NC) {
        acc = o[0];
#pragma unroll
        for (int t = 1; t < CH; ++t) {
          acc = acc + o[pr<T>(2 * t)];
          o[pr<T>(2 * t)] = acc;
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
        for (int t = 0; t < CH; ++t) o[pr<T>(2 * t)] += ex;
      }
    }
  } else {
    // FP32: each lane scans NV consecutive 16-byte vectors (4 NV reals,
    // 2 NV odd outputs) in registers, the lane totals are scanned by
    // shuffles, and a running carry joins the 128 NV reals of one round to
    // the next:  out = (carry + exclusive lane prefix) + in-lane prefix.
    // A lane's vectors start 4 NV reals (plus the pads) after its
    // neighbour's, which spreads the 8 lanes of each 128-byte wavefront
    // over all banks (the pad layout of 16 complex floats per 128 bytes).
    constexpr int NV = M >= 512 ? 4 : M / 128, SPAN = 128 * NV;
    static_assert(NV >= 1 && M % SPAN == 0, "whole rounds (M >= 128)");
    static_assert((2 * Pad<T>::P) % 4 == 0, "vectors stay inside one pad period");
    const int warp = tid >> 5, lane = tid & 31, nwarp = DST_NT >> 5;
    for (int r = warp; r < nrows; r += nwarp) {
      T* row = dst + r * ld;
      T carry = T(0);
#pragma unroll 1
      for (int it = 0; it < M / SPAN; ++it) {
        const int i0 = it * SPAN + lane * 4 * NV;
        float4 u[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) u[v] = *reinterpret_cast<const float4*>(row + pr<T>(i0 + 4 * v));
        T pre[2 * NV];
        T run = u[0].x;
        pre[0] = run;
        run = run + u[0].z;
        pre[1] = run;
#pragma unroll
        for (int v = 1; v < NV; ++v) {
          run = run + u[v].x;
          pre[2 * v] = run;
          run = run + u[v].z;
          pre[2 * v + 1] = run;
        }
        T incl = run;
#pragma unroll
        for (int of = 1; of < 32; of <<= 1) {
          const T t = __shfl_up_sync(0xffffffffu, incl, of);
          if (lane >= of) incl += t;
        }
        T ex = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) ex = T(0);
        const T base = carry + ex;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          u[v].x = base + pre[2 * v];
          u[v].z = base + pre[2 * v + 1];
          *reinterpret_cast<float4*>(row + pr<T>(i0 + 4 * v)) = u[v];
        }
        carry = carry + __shfl_sync(0xffffffffu, incl, 31);
      }
    }
  }
  __syncthreads();
  return dst;
}

}  // namespace qgw
