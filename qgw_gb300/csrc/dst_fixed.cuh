// dst_fixed.cuh -- the batched DST-I of dst_core.h specialised at compile
// time for one transform length (M = 2H = 2^(LGH+1)), used by the step
// kernels for the common lengths, and its complex FFT alone (the periodic
// transforms).  Same arithmetic as the generic block DST (step_device.cuh),
// with phases merged where the data allow it:
//   [pre-processing + first radix-8 pass] -> later Stockham passes
//   -> [split + prefix sum of the odd outputs]
// (FP32; the FP64 kernels, bound by their FP64 pipe and short of registers
// for the merged phases, keep the pre-processing and the split and prefix
// sum as phases of their own).  The merged first pass reads the four raw
// values each complex input needs (x_{2m}, x_{2m+1}, x_{M-2m}, x_{M-2m-1}),
// so the pre-processed row is never stored.  With the geometry fixed, a
// padded shared-memory index is one base computation plus compile-time
// offsets (StockhamItem), and the prefix sum runs one warp per row without
// block barriers.  The blocks have DST_NT threads and every phase has a
// power-of-two item count per row, so a thread meets the same in-row items
// in every row: their indices, table values and twiddles are computed once
// per transform, outside the row loop.
// Buffer format (dst_core.h): x_j at index j, Y_k at index k, index 0 unused.
#pragma once

#include "dst_core.h"
#include "dst_warp.h"

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
    if constexpr (sizeof(T) == 4 && NS == 1) {
      // first pass: outputs R b .. R b + R - 1 lie in one pad period and
      // start 16-byte aligned -- 16-byte stores (8-byte ones at stride R
      // would meet bank conflicts)
#pragma unroll
      for (int q = 0; q < R; q += 2)
        *reinterpret_cast<float4*>(dst + out0 + q) = make_float4(v[q].x, v[q].y, v[q + 1].x, v[q + 1].y);
    } else {
#pragma unroll
      for (int q = 0; q < R; ++q) dst[out0 + pco(q * NS)] = v[q];
    }
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

// The Stockham passes of the complex FFT of H = 2^LGH points from pass FIRST
// on (0: the whole FFT) over nrows rows: input in X, Y the second buffer;
// returns the buffer that holds the output.  The same passes and arithmetic
// as the runtime-geometry loops of dst_core.h (bit-identical results).
template <typename T, int LGH, int FIRST>
__device__ T* cfft_passes_fixed(T* X, T* Y, int nrows, int ld, const C2<T>* __restrict__ twp) {
  using S = DstShape<LGH>;
  constexpr int H = S::H;
  static_assert(S::NP8 <= 3, "fixed passes cover H <= 4096");
  T* src = X;
  T* dst = Y;
  if constexpr (S::NP8 >= 1 && FIRST <= 0) {
    stockham_pass_fixed<T, 8, 1, H>(src, dst, nrows, ld, twp);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::NP8 >= 2 && FIRST <= 1) {
    stockham_pass_fixed<T, 8, 8, H>(src, dst, nrows, ld, twp);
    __syncthreads();
    T* t = src; src = dst; dst = t;
  }
  if constexpr (S::NP8 >= 3 && FIRST <= 2) {
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
__device__ T* cfft_block_fixed(T* X, T* Y, int nrows, int ld, const C2<T>* __restrict__ twp) {
  return cfft_passes_fixed<T, LGH, 0>(X, Y, nrows, ld, twp);
}

// Pre-processing merged into the first (radix-8, twiddle-free) Stockham
// pass: item b of a row forms z_m = y_{2m} + i y_{2m+1} for m = b + q H/8
// (q = 0..7) straight from the raw row, with y_j written symmetrically,
// y_j = s_j (x_j + x_{M-j}) + (x_j - x_{M-j}) / 2 (s_j = sin(pi j/M) =
// s_{M-j}, the same value as dst_pre_item's (s_j + 1/2) x_j + (s_j - 1/2)
// x_{M-j}), y_0 = 0; takes the radix-8 butterfly and writes outputs 8b + q.
// The item's sixteen s values stay in registers for all rows.  Every index
// is the item's padded base plus a compile-time offset: 2 q H/8 = q H/4 is a
// whole number of pad periods (H >= 128 for floats), so pr(i + q H/4) =
// pr(i) + pr(q H/4), and M - 2m = (M - 2b) - q H/4 likewise.
template <typename T, int H>
struct PrePassItem {
  static constexpr int M = 2 * H, S = H / 8, PR = 2 * (1 << Pad<T>::LG);
  static_assert((H / 4) % PR == 0, "offsets of whole pad periods");
  static constexpr int pro(int i) { return i + 2 * Pad<T>::W * (i >> (Pad<T>::LG + 1)); }
  int a0, m0, m1, out0;
  bool first;    // item 0: y_0 = 0
  T s[8][2];     // s_{2m}, s_{2m+1} of member q
  __device__ __forceinline__ void init(int b, const T* __restrict__ sj) {
    a0 = pr<T>(2 * b);           // x_{2m}, x_{2m+1} at a0 + pro(q H/4) (+1)
    m0 = pr<T>(M - 2 * b);       // x_{M-2m}
    m1 = pr<T>(M - 2 * b - 1);   // x_{M-2m-1}
    out0 = pc<T>(8 * b);
    first = b == 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int j0 = 2 * (b + q * S), j1 = j0 + 1;
      s[q][0] = sj[j0 <= H ? j0 : M - j0];
      s[q][1] = sj[j1 <= H ? j1 : M - j1];
    }
  }
  __device__ __forceinline__ void run(const T* __restrict__ x, C2<T>* __restrict__ dst) const {
    C2<T> v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int o = pro(q * (H / 4));
      // x_{2m}, x_{2m+1}: one aligned pair (2m is even, and an even index
      // and the next share a pad period)
      const C2<T> xp = *reinterpret_cast<const C2<T>*>(x + a0 + o);
      const T xa = xp.x, xb = xp.y;
      const T ya = x[m0 - o], yb = x[m1 - o];      // x_{M-2m}, x_{M-2m-1}
      const T y0 = fmaT(s[q][0], xa + ya, T(0.5) * (xa - ya));
      v[q].x = (q == 0 && first) ? T(0) : y0;
      v[q].y = fmaT(s[q][1], xb + yb, T(0.5) * (xb - yb));
    }
    dft8(v);
    // outputs 8b .. 8b+7 lie in one pad period and start 16-byte aligned:
    // four 16-byte stores (eight 8-byte ones at stride 8 would meet 2-way
    // bank conflicts in each half-warp)
#pragma unroll
    for (int q = 0; q < 8; q += 2) store_pair(dst + out0 + q, v[q], v[q + 1]);
  }
  __device__ __forceinline__ static void store_pair(C2<T>* p, C2<T> a, C2<T> b) {
    if constexpr (sizeof(T) == 4) {
      *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
    } else {
      p[0] = a;
      p[1] = b;
    }
  }
};

template <typename T, int H>
__device__ __forceinline__ void pre_pass1_fixed(const T* src, T* dst, int nrows, int ld, const T* sj) {
  constexpr int NB = H / 8;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  if constexpr (NB < DST_NT) {
    PrePassItem<T, H> it;
    it.init(tid & (NB - 1), sj);
    for (int r = tid / NB; r < nrows; r += DST_NT / NB) it.run(src + r * ld, (C2<T>*)(dst + r * ld));
  } else {
    constexpr int C = NB / DST_NT;
    PrePassItem<T, H> it[C];
#pragma unroll
    for (int c = 0; c < C; ++c) it[c].init(tid + c * DST_NT, sj);
    for (int r = 0; r < nrows; ++r)
#pragma unroll
      for (int c = 0; c < C; ++c) it[c].run(src + r * ld, (C2<T>*)(dst + r * ld));
  }
}

// FP32 split and prefix sum in one phase, one warp per row (rows r = warp,
// warp + 8, ...), for H = 64 KPL with KPL in {2, 4, 8}.  Lane L takes the
// split items k = k0 + t, k0 = KPL L, t = 0..KPL-1: each yields the pair
// (Y_{2k}, 2R_k) at complex index k ("lo") and its mirror (Y_{2(H-k)},
// 2R_{H-k}) at H-k ("hi"); lane 0's t = 0 yields R_0 and, in the hi slot,
// the self-mirrored item k = H/2.  The odd outputs Y_{2k+1} are the prefix
// sums of the increments over k = 0..H-1: the lo half (k < H/2) is a forward
// scan in (lane, t) order, the hi half (k' = H - k >= H/2) a suffix scan in
// the same order on top of the lo half's total.  Loads and stores move whole
// 16-byte complex pairs; the hi pairs start at even indices, so each lane
// stores its pairs H-k0-KPL .. H-k0-1, the first element taken from the next
// lane (lane 31 from lane 0's k = H/2 item).
// The split and prefix sum of one row by one warp from the lane's inputs
// Zl[t] = Z_{k0+t}, Zh[t] = Z_{H-k0-t} (k0 = KPL lane; lane 0's Zh[0] =
// Z_{H/2}) and split constants cs[t] = spl[k0 + t] (lane 0's cs[0] =
// spl[H/2]); writes Y_k at index k of orow.  The row's inputs have all been
// read (the caller synchronises the warp when orow is the input row).
template <int H>
__device__ __forceinline__ void split_scan_lane_f32(int lane, const C2<float>* Zl, const C2<float>* Zh,
                                                    const C2<float>* cs, float* orow) {
  constexpr int KPL = H / 64;
  const int k0 = KPL * lane;
  {
    C2<float> lo[KPL], hi[KPL];
#pragma unroll
    for (int t = 0; t < KPL; ++t) {
      const bool special = (lane == 0 && t == 0);
      // item k = k0 + t (the k = H/2 item in the special slot's hi)
      const C2<float> Av = special ? Zh[0] : Zl[t];
      const C2<float> Bc = Zh[t];
      const float br = Bc.x, bi = -Bc.y;
      const float sr = Av.x + br, si = Av.y + bi, dr = Av.x - br, di = Av.y - bi;
      const float P = fmaT(cs[t].x, di, -(cs[t].y * dr));
      const float Q = fmaT(cs[t].x, dr, cs[t].y * di);
      if (special) {
        lo[t].x = 0.f;                  // index 0 (no output)
        lo[t].y = Zl[0].x + Zl[0].y;    // R_0
        hi[t].x = Q - si;               // Y_H
        hi[t].y = sr + P;               // 2 R_{H/2}
      } else {
        lo[t].x = Q - si;  // Y_{2k}
        lo[t].y = sr + P;  // 2 R_k
        hi[t].x = Q + si;  // Y_{2(H-k)}
        hi[t].y = sr - P;  // 2 R_{H-k}
      }
    }
    // lo half: forward scan
    float run = 0.f, pre[KPL];
#pragma unroll
    for (int t = 0; t < KPL; ++t) { run = run + lo[t].y; pre[t] = run; }
    float incl = run;
#pragma unroll
    for (int of = 1; of < 32; of <<= 1) {
      const float u = __shfl_up_sync(0xffffffffu, incl, of);
      if (lane >= of) incl += u;
    }
    float ex = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) ex = 0.f;
#pragma unroll
    for (int t = 0; t < KPL; ++t) lo[t].y = ex + pre[t];
    const float T1 = __shfl_sync(0xffffffffu, incl, 31);
    const float incH2 = __shfl_sync(0xffffffffu, hi[0].y, 0);
    // hi half: suffix scan over k >= 1 (lane 0's t = 0 slot is the k = H/2 item)
    float suf[KPL];
    float srun = 0.f;
#pragma unroll
    for (int t = KPL - 1; t >= 0; --t) {
      srun = srun + ((lane == 0 && t == 0) ? 0.f : hi[t].y);
      suf[t] = srun;
    }
    float sincl = srun;
#pragma unroll
    for (int of = 1; of < 32; of <<= 1) {
      const float u = __shfl_down_sync(0xffffffffu, sincl, of);
      if (lane + of < 32) sincl += u;
    }
    float sx = __shfl_down_sync(0xffffffffu, sincl, 1);
    if (lane == 31) sx = 0.f;
    const float base = T1 + incH2;
#pragma unroll
    for (int t = 0; t < KPL; ++t) hi[t].y = (lane == 0 && t == 0) ? base : base + (sx + suf[t]);
    // stores: lo pairs at k0 + 2p; hi pairs at H - k0 - KPL + 2p, whose first
    // element (index H - k0 - KPL, t = KPL) is the next lane's t = 0
    C2<float> nb;
    nb.x = __shfl_sync(0xffffffffu, hi[0].x, (lane + 1) & 31);
    nb.y = __shfl_sync(0xffffffffu, hi[0].y, (lane + 1) & 31);
#pragma unroll
    for (int p = 0; p < KPL / 2; ++p) {
      *reinterpret_cast<float4*>(orow + 2 * pc<float>(k0 + 2 * p)) =
          make_float4(lo[2 * p].x, lo[2 * p].y, lo[2 * p + 1].x, lo[2 * p + 1].y);
      const C2<float> e0 = p == 0 ? nb : hi[KPL - 2 * p], e1 = hi[KPL - 2 * p - 1];
      *reinterpret_cast<float4*>(orow + 2 * pc<float>(H - k0 - KPL + 2 * p)) = make_float4(e0.x, e0.y, e1.x, e1.y);
    }
  }
}

template <int H>
__device__ __forceinline__ void split_scan_warp_f32(const float* src, float* dst, int nrows, int ld,
                                                    const C2<float>* __restrict__ spl) {
  constexpr int KPL = H / 64;
  static_assert(KPL == 2 || KPL == 4 || KPL == 8, "H = 128, 256 or 512");
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarp = DST_NT >> 5;
  const int k0 = KPL * lane;
  C2<float> cs[KPL];
#pragma unroll
  for (int t = 0; t < KPL; ++t) cs[t] = spl[(lane == 0 && t == 0) ? H / 2 : k0 + t];
  const int hs = lane == 0 ? pc<float>(H / 2) : pc<float>(H - k0);  // t = 0 mirror (or k = H/2)
  for (int r = warp; r < nrows; r += nwarp) {
    const C2<float>* Z = (const C2<float>*)(src + r * ld);
    C2<float> Zl[KPL], Zh[KPL];
#pragma unroll
    for (int p = 0; p < KPL / 2; ++p) {
      // an even index and the next share a pad period: one 16-byte pair
      const float4 u = *reinterpret_cast<const float4*>(Z + pc<float>(k0 + 2 * p));
      Zl[2 * p].x = u.x; Zl[2 * p].y = u.y; Zl[2 * p + 1].x = u.z; Zl[2 * p + 1].y = u.w;
    }
#pragma unroll
    for (int p = 0; p < KPL / 2; ++p) {
      const int e = H - k0 - KPL + 2 * p;
      const float4 u = *reinterpret_cast<const float4*>(Z + pc<float>(e));
      if (p > 0) { Zh[KPL - 2 * p].x = u.x; Zh[KPL - 2 * p].y = u.y; }
      Zh[KPL - 2 * p - 1].x = u.z; Zh[KPL - 2 * p - 1].y = u.w;
    }
    Zh[0] = Z[hs];
    split_scan_lane_f32<H>(lane, Zl, Zh, cs, dst + r * ld);
  }
}

// One row's DST-I by one warp, in place (dst_warp.h): pre-processing with
// the first DIF pass, two more passes, then the split with the prefix sum.
// x_{M-2m} of a pass-1 member comes from the previous member's mirror pair
// by one shuffle per member: from lane - 1, and for lane 0 from lane 31 at
// the previous member in (n2, u) order (the value the shuffle of the
// previous iteration delivered).
template <int LGH>
__device__ __forceinline__ void dst_row_warp_f32(float* row, const DstTables<float>& tb, int lane) {
  using W = WarpDst<LGH>;
  C2<float>* Z = reinterpret_cast<C2<float>*>(row);
  C2<float> v[W::IPL][8];
  {
    float prev = 0.f;
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2)
#pragma unroll
      for (int u = 0; u < W::IPL; ++u) {
        const int m = lane + 32 * u + W::S0 * n2;
        C2<float> own, mir;
        W::p1_read(m, Z, own, mir);
        const float got = __shfl_sync(0xffffffffu, mir.x, (lane + 31) & 31);
        const float xm = lane > 0 ? got : prev;  // (lane 0, m = 0): x_M, enters only y_0 = 0
        prev = got;
        v[u][n2] = W::p1_pre(m, own, xm, mir.y, tb.sjp[m]);
      }
  }
  __syncwarp();
#pragma unroll
  for (int u = 0; u < W::IPL; ++u) W::p1_fft(lane + 32 * u, v[u], tb.twd, Z);
  __syncwarp();
  {
    C2<float> w2[8];
    W::p2_twiddles(lane % W::S1, tb.twd, w2);
#pragma unroll
    for (int u = 0; u < W::IPL; ++u) W::p2(lane + 32 * u, w2, Z);
  }
  __syncwarp();
#pragma unroll
  for (int u = 0; u < 2; ++u) W::p3(lane + 32 * u, Z);
  __syncwarp();
  C2<float> Zl[W::KPL], Zh[W::KPL], cs[W::KPL];
  W::split_read(lane, Z, Zl, Zh);
  const int k0 = W::KPL * lane;
#pragma unroll
  for (int t = 0; t < W::KPL; ++t) cs[t] = tb.spl[(lane == 0 && t == 0) ? W::H / 2 : k0 + t];
  __syncwarp();
  split_scan_lane_f32<W::H>(lane, Zl, Zh, cs, row);
  __syncwarp();
}

// DST-I of nrows raw rows in A by one warp per row, in place; the caller
// has synchronised the block since the rows were written, and the block is
// synchronised again before the result (in A) is returned.
template <int LGH>
__device__ float* dst_block_warp_f32(float* A, int nrows, int ld, const DstTables<float>& tb) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarp = DST_NT >> 5;
  for (int r = warp; r < nrows; r += nwarp) dst_row_warp_f32<LGH>(A + r * ld, tb, lane);
  __syncthreads();
  return A;
}

// DST-I of nrows raw rows in A (x_j at index j), B the second buffer;
// returns the buffer that holds Y_k at index k.
template <typename T, int LGH>
__device__ T* dst_block_fixed(T* A, T* B, int nrows, int ld, const DstTables<T>& tb) {
  using S = DstShape<LGH>;
  constexpr int H = S::H, M = S::M;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  static_assert(H % DST_NT == 0 || DST_NT % H == 0, "power-of-two shapes");
  T* src;
  if constexpr (sizeof(T) == 4 && (H / 4) % (2 * (1 << Pad<T>::LG)) == 0) {
    // phases 1 + 2a: pre-processing and the first pass, A -> B
    pre_pass1_fixed<T, H>(A, B, nrows, ld, tb.sj);
    __syncthreads();
    src = cfft_passes_fixed<T, LGH, 1>(B, A, nrows, ld, tb.twp);
  } else {
    // pre-processing as its own phase, A -> B (dst_pre_item's arithmetic):
    // doubles (the merged phase's 16 live complex values and their table
    // entries exceed the FP64 kernels' register bound; those kernels are
    // bound by the FP64 pipe, not by barriers) and short float rows (H = 64)
    for (int w = tid; w < nrows * H; w += DST_NT) {
      const int r = w >> LGH, j = (w & (H - 1)) + 1;
      const T* x = A + r * ld;
      T* y = B + r * ld;
      const T a = x[pr<T>(j)], b = x[pr<T>(M - j)];
      const C2<T> wp = tb.pre[j];
      y[pr<T>(j)] = fmaT(wp.x, a, wp.y * b);
      y[pr<T>(M - j)] = fmaT(wp.y, a, wp.x * b);
      if (j == 1) y[0] = T(0);
    }
    __syncthreads();
    src = cfft_passes_fixed<T, LGH, 0>(B, A, nrows, ld, tb.twp);
  }
  T* dst = src == A ? B : A;
  if constexpr (sizeof(T) == 4 && H >= 128 && H <= 512) {
    // phases 3 + 4 in one, one warp per row
    split_scan_warp_f32<H>(src, dst, nrows, ld, tb.spl);
    __syncthreads();
    return dst;
  }
  // phase 3: split (dst_split_item), items k = 0..H/2-1; item 0 also does
  // k = H/2 (and R_0); thread tid handles k = tid + c * DST_NT of every row.
  // Outputs go out as (Y_{2k}, 2 R_k) pairs at complex index k.
  {
    constexpr int KI = H / 2;
    constexpr int C = KI >= DST_NT ? KI / DST_NT : 1;
    constexpr int RS = KI >= DST_NT ? 1 : DST_NT / KI;
    const int kb = KI >= DST_NT ? tid : (tid & (KI - 1));
    int za[C], zb[C];
    C2<T> cs[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int k = kb + c * DST_NT;
      const int kk = k == 0 ? H / 2 : k;  // item 0 runs the k = H/2 butterfly
      za[c] = pc<T>(kk);
      zb[c] = pc<T>(H - kk);
      cs[c] = tb.spl[kk];
    }
    for (int r = KI >= DST_NT ? 0 : tid / KI; r < nrows; r += RS) {
      const C2<T>* Z = (const C2<T>*)(src + r * ld);
      C2<T>* out = (C2<T>*)(dst + r * ld);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const C2<T> Av = Z[za[c]];
        const C2<T> Bc = Z[zb[c]];
        const T br = Bc.x, bi = -Bc.y;
        const T sr = Av.x + br, si = Av.y + bi, dr = Av.x - br, di = Av.y - bi;
        const T P = fmaT(cs[c].x, di, -(cs[c].y * dr));
        const T Q = fmaT(cs[c].x, dr, cs[c].y * di);
        C2<T> lo, hi;
        lo.x = Q - si;  // Y_{2k}
        lo.y = sr + P;  // 2 R_k
        out[za[c]] = lo;
        if (kb + c * DST_NT != 0) {
          hi.x = Q + si;  // Y_{2(H-k)}
          hi.y = sr - P;  // 2 R_{H-k}
          out[zb[c]] = hi;
        } else {
          const C2<T> a = Z[0];
          C2<T> z0;
          z0.x = T(0);         // index 0 (no output)
          z0.y = a.x + a.y;    // R_0
          out[0] = z0;
        }
      }
    }
  }
  __syncthreads();
  // phase 4: prefix sum of the odd outputs (indices 1, 3, 5, ...), one warp
  // per row.
  if constexpr (sizeof(T) == 8) {
    // FP64 (the FP64 pipe bounds these kernels, so the fewest additions):
    // lane c scans chunk c sequentially, the chunk totals are scanned by
    // shuffles and added back -- two additions per value
    constexpr int CH = H >= 256 ? H / 32 : 8, NC = H / CH;
    static_assert((2 * CH) % (2 * Pad<T>::P) == 0, "chunk start must be pad-aligned");
    const int warp = tid >> 5, lane = tid & 31, nwarp = DST_NT >> 5;
    for (int r = warp; r < nrows; r += nwarp) {
      // odd index 2k + 1 of the chunk: o[pr(2t)] (2t and 2t + 1 share a pad period)
      T* o = dst + r * ld + pr<T>(2 * CH * lane) + 1;
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
    // FP32 (rows of other lengths): each lane scans NV consecutive 16-byte
    // vectors (4 NV reals, 2 NV odd outputs, the .y and .w members) in
    // registers, the lane totals are scanned by shuffles, and a running
    // carry joins the 128 NV reals of one round to the next:  out = (carry +
    // exclusive lane prefix) + in-lane prefix.  A lane's vectors start 4 NV
    // reals (plus the pads) after its neighbour's, which spreads the 8 lanes
    // of each 128-byte wavefront over all banks (the pad layout of 16
    // complex floats per 128 bytes).
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
        T run = u[0].y;
        pre[0] = run;
        run = run + u[0].w;
        pre[1] = run;
#pragma unroll
        for (int v = 1; v < NV; ++v) {
          run = run + u[v].y;
          pre[2 * v] = run;
          run = run + u[v].w;
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
          u[v].y = base + pre[2 * v];
          u[v].w = base + pre[2 * v + 1];
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
