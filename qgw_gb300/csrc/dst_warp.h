// dst_warp.h -- work items of the FP32 DST-I that one warp runs on one row,
// in place, for M = 512 and 1024 (H = 256, 512).
//
// The transform is dst_core.h's (Y_k = 2 sum_j x_j sin(pi j k / M); input x_j
// at real index j, output Y_k at real index k, index 0 = 0) with the
// half-length complex FFT run as three in-place decimation-in-frequency
// passes of radix 8, 8 and R3 = H/64 (8 or 4):
//   pass 1  items n1 < S0 = H/8:   z at n1 + S0 n2 (n2 < 8) -> DFT_8 over n2,
//           output k2 times w_H^(n1 k2), back to n1 + S0 k2;
//   pass 2  items (block b < 8, n1 < S1 = H/64): the same on the block of
//           H/8 values at b H/8, stride S1, twiddles w_H^(8 n1 k2);
//   pass 3  items b < 64: DFT_R3 of the R3 values at R3 b, in place.
// The FFT's output Z_k then lies at pos(k) = d0 S0 + d1 S1 + d2 for
// k = d0 + 8 d1 + 64 d2 (its base-8 digits reversed), where the split reads
// it.  Each pass's items touch disjoint values; the pre-processing (merged
// into pass 1) and the split (merged with the prefix sum) read values that
// other lanes' items overwrite, so those phases read everything first.
// Every function is a work item of one lane (lane 0..31) that both the
// device code and a CPU check run; the lane-to-lane steps (one shuffle in
// pass 1, the scans of the split) are in the device code.
#pragma once

#include "dst_core.h"

namespace qgw {

// 16-byte vector of four floats (CUDA's float4 on the device)
#ifdef __CUDACC__
#define QGW_UNROLL _Pragma("unroll")
using F4 = float4;
QGW_HD F4 mk4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
#else
#define QGW_UNROLL
struct alignas(16) F4 { float x, y, z, w; };
inline F4 mk4(float a, float b, float c, float d) { return F4{a, b, c, d}; }
#endif

// the lengths the one-warp transform takes: FP32, H = 256 or 512 (its
// callers then need one buffer per row, the transform runs in place)
QGW_HD bool warp_dst_len(int H, int elem) { return elem == 4 && (H == 256 || H == 512); }

template <int LGH> struct WarpDst {
  static_assert(LGH == 8 || LGH == 9, "H = 256 or 512");
  static constexpr int H = 1 << LGH, M = 2 * H;
  static constexpr int S0 = H / 8, S1 = H / 64, R3 = H / 64;
  static constexpr int IPL = S0 / 32;  // pass-1 and pass-2 items per lane
  static constexpr int KPL = H / 64;   // split items per lane
  static constexpr int NTW = 7 * (S0 + S1);  // DIF twiddles (pass 1, then pass 2)
  QGW_HD static int pos(int k) { return (k & 7) * S0 + ((k >> 3) & 7) * S1 + (k >> 6); }

  // pass-1 member (u, n2) of a lane: complex index m = lane + 32 u + S0 n2.
  // Reads the pair (x_{2m}, x_{2m+1}) and the mirror pair (x_{M-2m-2},
  // x_{M-2m-1}); x_{M-2m} is the mirror pair's .x of member m - 1 (the
  // previous lane, or lane 31 at the previous member in (n2, u) order).
  QGW_HD static void p1_read(int m, const C2<float>* Z, C2<float>& own, C2<float>& mir) {
    own = Z[pc<float>(m)];
    mir = Z[pc<float>(H - 1 - m)];
  }
  // z_m = y_{2m} + i y_{2m+1}, y_j = s_j (x_j + x_{M-j}) + (x_j - x_{M-j}) / 2
  // (dst_pre_item's values, written symmetrically), y_0 = 0; s = (s_{2m},
  // s_{2m+1})
  QGW_HD static C2<float> p1_pre(int m, C2<float> own, float xM2m, float xM2m1, C2<float> s) {
    C2<float> z;
    const float y0 = fmaT(s.x, own.x + xM2m, 0.5f * (own.x - xM2m));
    z.x = m == 0 ? 0.f : y0;
    z.y = fmaT(s.y, own.y + xM2m1, 0.5f * (own.y - xM2m1));
    return z;
  }
  // pass-1 butterfly of item n1 on its eight z values v (n2 order)
  QGW_HD static void p1_fft(int n1, C2<float>* v, const C2<float>* __restrict__ twd, C2<float>* Z) {
    dft8(v);
    QGW_UNROLL
    for (int k2 = 1; k2 < 8; ++k2) v[k2] = cmul(v[k2], twd[(k2 - 1) * S0 + n1]);
    QGW_UNROLL
    for (int k2 = 0; k2 < 8; ++k2) Z[pc<float>(n1 + S0 * k2)] = v[k2];
  }
  // pass-2 twiddles of offset n1 < S1 (w[k2], k2 = 1..7): the items of a
  // lane (it = lane + 32 u) share their offset it % S1 = lane % S1
  QGW_HD static void p2_twiddles(int n1, const C2<float>* __restrict__ twd, C2<float>* w) {
    QGW_UNROLL
    for (int k2 = 1; k2 < 8; ++k2) w[k2] = twd[7 * S0 + (k2 - 1) * S1 + n1];
  }
  // pass-2 item it < S0: block it / S1, offset it % S1 (twiddles w)
  QGW_HD static void p2(int it, const C2<float>* w, C2<float>* Z) {
    const int b = it / S1, n1 = it - b * S1;
    const int base = b * (H / 8) + n1;
    C2<float> v[8];
    QGW_UNROLL
    for (int n2 = 0; n2 < 8; ++n2) v[n2] = Z[pc<float>(base + S1 * n2)];
    dft8(v);
    QGW_UNROLL
    for (int k2 = 1; k2 < 8; ++k2) v[k2] = cmul(v[k2], w[k2]);
    QGW_UNROLL
    for (int k2 = 0; k2 < 8; ++k2) Z[pc<float>(base + S1 * k2)] = v[k2];
  }
  // pass-3 item it < 64: the R3 values at R3 it (one pad period, 16-byte
  // aligned: moved as 16-byte pairs)
  QGW_HD static void p3(int it, C2<float>* Z) {
    C2<float> v[R3];
    const int b = pc<float>(R3 * it);
    QGW_UNROLL
    for (int q = 0; q < R3; q += 2) {
      const F4 u = *reinterpret_cast<const F4*>(Z + b + q);
      v[q].x = u.x; v[q].y = u.y; v[q + 1].x = u.z; v[q + 1].y = u.w;
    }
    if constexpr (R3 == 8) dft8(v);
    else dft4(v);
    QGW_UNROLL
    for (int q = 0; q < R3; q += 2)
      *reinterpret_cast<F4*>(Z + b + q) = mk4(v[q].x, v[q].y, v[q + 1].x, v[q + 1].y);
  }
  // the split's inputs of a lane: Zl[t] = Z_{k0+t}, Zh[t] = Z_{H-k0-t}
  // (k0 = KPL lane), except lane 0's Zh[0] = Z_{H/2}
  QGW_HD static void split_read(int lane, const C2<float>* Z, C2<float>* Zl, C2<float>* Zh) {
    const int k0 = KPL * lane;
    QGW_UNROLL
    for (int t = 0; t < KPL; ++t) {
      Zl[t] = Z[pc<float>(pos(k0 + t))];
      Zh[t] = Z[pc<float>(pos((lane == 0 && t == 0) ? H / 2 : H - k0 - t))];
    }
  }
};

}  // namespace qgw
