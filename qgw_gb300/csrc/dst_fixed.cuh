// dst_fixed.cuh -- the batched DST-I of dst_core.h specialised at compile
// time for one transform length (M = 2H = 2^(LGH+1)), used by the step
// kernels for the common lengths.  Same phases, same arithmetic as the
// generic block DST (kernels.cu), so results agree bit for bit with it:
//   pre-processing -> Stockham radix-8 passes (+ one radix-4/2 pass)
//   -> split -> prefix sum of the odd outputs.
// With the geometry fixed, every padded shared-memory index is one base
// computation plus immediate offsets (strides that are multiples of 8
// complex values keep the pad pattern: pc(e + 8m) = pc(e) + 9m), and the
// prefix sum runs one warp per row without block barriers.  The blocks have
// DST_NT threads and every phase has a power-of-two item count per row, so a
// thread meets the same in-row items in every row: their indices, table
// values and twiddles are computed once per transform, outside the row loop.
#pragma once

#include "dst_core.h"

namespace qgw {

constexpr int DST_NT = 256;  // threads per block of every kernel that calls dst_block_fixed

template <int LGH> struct DstShape {
  static constexpr int H = 1 << LGH, M = 2 * H;
  static constexpr int NP8 = LGH / 3;                 // radix-8 passes
  static constexpr int RLAST = 1 << (LGH % 3);        // 1: none, 2 or 4
  static constexpr int CHUNK = H >= 256 ? H / 32 : 8; // prefix-sum chunk
  static constexpr int NCHUNK = H / CHUNK;
  static_assert(LGH >= 6, "fixed DST needs H >= 64");
};

// One Stockham pass over all rows: item b of a row reads inputs b + q*(H/R)
// and writes outputs base + q*NS; the twiddles of item b are loaded once.
template <typename T, int R, int NS, int H>
struct StockhamItem {
  static constexpr int S = H / R;
  static constexpr int OS = NS == 1 ? 1 : NS + NS / 8;
  static_assert(S % 8 == 0, "input stride must keep the pad pattern");
  static_assert(NS == 1 || NS % 8 == 0, "output stride must keep the pad pattern");
  int in0, out0;
  C2<T> w[R];
  __device__ __forceinline__ void init(int b, const C2<T>* __restrict__ tw) {
    in0 = pc(b);
    const int k = b & (NS - 1);
    out0 = pc((b - k) * R + k);
    if constexpr (NS > 1) {
      const int step = k * (H / (NS * R));
#pragma unroll
      for (int q = 1; q < R; ++q) w[q] = tw[q * step];
    }
  }
  __device__ __forceinline__ void run(const C2<T>* __restrict__ src, C2<T>* __restrict__ dst) const {
    C2<T> v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = src[in0 + q * (S + S / 8)];
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
    for (int q = 0; q < R; ++q) dst[out0 + q * OS] = v[q];
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
      ia[c] = pr(j - 1);
      ib[c] = pr(M - j - 1);
      oa[c] = pr(j);
      ob[c] = pr(M - j);
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
    const int ia = pr(j - 1), ib = pr(M - j - 1), oa = pr(j), ob = pr(M - j);
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
      za[c] = pc(kk);
      zb[c] = pc(H - kk);
      o0[c] = pr(2 * kk);
      o1[c] = pr(2 * kk - 1);
      o2[c] = pr(2 * (H - kk));
      o3[c] = pr(2 * (H - kk) - 1);
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
  // phase 4: prefix sum of the odd outputs (indices 0, 2, 4, ...): one warp
  // per row, lane c scans chunk c, the chunk totals are scanned by shuffles
  const int warp = tid >> 5, lane = tid & 31, nwarp = DST_NT >> 5;
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
