// CPU check of the device DST-I building blocks (qgw_gb300/csrc/dst_core.h):
// runs every phase's work items in a plain loop, exactly as the kernels
// spread them over threads, and exposes the result through a C function.
#include <cmath>
#include <vector>
#include <cstring>
#include "../../qgw_gb300/csrc/dst_tables.h"
#include "../../qgw_gb300/csrc/dst_warp.h"
#include "../../qgw_gb300/csrc/dst_blue.h"

using namespace qgw;

template <typename T>
static void run(int M, int howmany, T* data) {
  DstGeom g = make_geom(M);
  DstTablesHost th = build_dst_tables(M);
  std::vector<T> tw(th.tw.begin(), th.tw.end()), pre(th.pre.begin(), th.pre.end()),
      spl(th.spl.begin(), th.spl.end());
  const C2<T>* TW = (const C2<T>*)tw.data();
  const C2<T>* PRE = (const C2<T>*)pre.data();
  const C2<T>* SPL = (const C2<T>*)spl.data();
  std::vector<T> A(padded_len<T>(M)), B(padded_len<T>(M));
  for (int r = 0; r < howmany; ++r) {
    T* x = data + (size_t)r * (M - 1);
    for (size_t j = 0; j < A.size(); ++j) A[j] = B[j] = T(777);  // pad slots must never be read
    for (int j = 0; j < M - 1; ++j) A[pr<T>(j + 1)] = x[j];      // x_j at index j
    A[pr<T>(0)] = T(12345);  // index 0 must never be read
    for (int j = 1; j <= g.H; ++j) dst_pre_item<T>(A.data(), B.data(), j, g, PRE);
    T* src = B.data();
    T* dst = A.data();
    int Ns = 1;
    for (int p = 0; p < g.npass; ++p) {
      const int R = g.radix[p];
      for (int b = 0; b < g.H / R; ++b)
        stockham_dispatch<T>(R, (const C2<T>*)src, (C2<T>*)dst, b, Ns, g.H, TW);
      Ns *= R;
      T* t = src; src = dst; dst = t;
    }
    // result in src; split into dst
    for (int k = 0; k <= g.H / 2; ++k) dst_split_item<T>((const C2<T>*)src, dst, k, g, SPL);
    std::vector<T> tot(g.nchunk);
    for (int c = 0; c < g.nchunk; ++c) tot[c] = dst_scan_chunk<T>(dst, c, g);
    T pref = T(0);
    for (int c = 0; c < g.nchunk; ++c) {
      if (c > 0) dst_scan_fix<T>(dst, c, pref, g);
      pref += tot[c];
    }
    for (int j = 0; j < M - 1; ++j) x[j] = dst[pr<T>(j + 1)];  // Y_k at index k
  }
}

// The one-warp transform (dst_warp.h) with its 32 lanes run one after the
// other inside each phase, every phase's reads done before its writes where
// the device code synchronises the warp in between; the lane-to-lane value
// of pass 1 (x_{M-2m}) taken as the device's shuffle delivers it.  The
// split's inputs are read through WarpDst::split_read (the digit-reversed
// positions) into a natural-order row, which the split and scan items of
// dst_core.h finish.
template <int LGH>
static void run_warp(int howmany, float* data) {
  using W = WarpDst<LGH>;
  constexpr int H = W::H, M = W::M, IPL = W::IPL, KPL = W::KPL;
  DstGeom g = make_geom(M);
  DstTablesHost th = build_dst_tables(M);
  std::vector<float> twd(th.twd.begin(), th.twd.end()), sjp(th.sjp.begin(), th.sjp.end()),
      spl(th.spl.begin(), th.spl.end());
  const C2<float>* TWD = (const C2<float>*)twd.data();
  const C2<float>* SJP = (const C2<float>*)sjp.data();
  const C2<float>* SPL = (const C2<float>*)spl.data();
  const int L = padded_len<float>(M);
  std::vector<F4> Abuf((L + 3) / 4), Bbuf((L + 3) / 4), Cbuf((L + 3) / 4);
  float* A = (float*)Abuf.data();
  float* B = (float*)Bbuf.data();
  float* Cr = (float*)Cbuf.data();
  static C2<float> own[32][IPL][8], mir[32][IPL][8], v[32][IPL][8];
  for (int r = 0; r < howmany; ++r) {
    float* x = data + (size_t)r * (M - 1);
    for (int j = 0; j < L; ++j) A[j] = B[j] = Cr[j] = 777.f;  // pad slots must never be read
    for (int j = 0; j < M - 1; ++j) A[pr<float>(j + 1)] = x[j];
    A[pr<float>(0)] = 12345.f;  // index 0 must never be read
    C2<float>* Z = (C2<float>*)A;
    for (int lane = 0; lane < 32; ++lane)
      for (int n2 = 0; n2 < 8; ++n2)
        for (int u = 0; u < IPL; ++u) W::p1_read(lane + 32 * u + W::S0 * n2, Z, own[lane][u][n2], mir[lane][u][n2]);
    for (int lane = 0; lane < 32; ++lane) {
      float prev = 0.f;
      for (int n2 = 0; n2 < 8; ++n2)
        for (int u = 0; u < IPL; ++u) {
          const int m = lane + 32 * u + W::S0 * n2;
          const float got = mir[(lane + 31) & 31][u][n2].x;  // __shfl_sync(.., (lane + 31) & 31)
          const float xm = lane > 0 ? got : prev;
          prev = got;
          v[lane][u][n2] = W::p1_pre(m, own[lane][u][n2], xm, mir[lane][u][n2].y, SJP[m]);
        }
    }
    for (int lane = 0; lane < 32; ++lane)
      for (int u = 0; u < IPL; ++u) W::p1_fft(lane + 32 * u, v[lane][u], TWD, Z);
    for (int lane = 0; lane < 32; ++lane) {
      C2<float> w2[8];
      W::p2_twiddles(lane % W::S1, TWD, w2);
      for (int u = 0; u < IPL; ++u) W::p2(lane + 32 * u, w2, Z);
    }
    for (int lane = 0; lane < 32; ++lane)
      for (int u = 0; u < 2; ++u) W::p3(lane + 32 * u, Z);
    C2<float>* N = (C2<float>*)B;
    for (int lane = 0; lane < 32; ++lane) {
      C2<float> Zl[KPL], Zh[KPL];
      W::split_read(lane, Z, Zl, Zh);
      for (int t = 0; t < KPL; ++t) {
        N[pc<float>(KPL * lane + t)] = Zl[t];
        N[pc<float>((lane == 0 && t == 0) ? H / 2 : H - KPL * lane - t)] = Zh[t];
      }
    }
    for (int k = 0; k <= H / 2; ++k) dst_split_item<float>((const C2<float>*)B, Cr, k, g, SPL);
    std::vector<float> tot(g.nchunk);
    for (int c = 0; c < g.nchunk; ++c) tot[c] = dst_scan_chunk<float>(Cr, c, g);
    float pref = 0.f;
    for (int c = 0; c < g.nchunk; ++c) {
      if (c > 0) dst_scan_fix<float>(Cr, c, pref, g);
      pref += tot[c];
    }
    for (int j = 0; j < M - 1; ++j) x[j] = Cr[pr<float>(j + 1)];
  }
}

// the one-warp transform for M = 512 and 1024; returns 0 for other lengths
extern "C" int dst_warp_run_f32(int M, int howmany, float* data) {
  if (M == 512) run_warp<8>(howmany, data);
  else if (M == 1024) run_warp<9>(howmany, data);
  else return 0;
  return 1;
}

// The chirp-z form (dst_blue.h) of any length M >= 4, its phases as loops:
// chirp, L-point FFT (the Stockham items), multiply, FFT, output.
template <typename T>
static void run_blue(int M, int howmany, T* data) {
  const DstGeom g = make_geom_blue(M);
  const int L = g.H;
  DstTablesHost th = build_dst_tables(2 * L);  // twiddles of the L-point FFT
  std::vector<double> bcd, bzd;
  build_blue_tables(g, bcd, bzd);
  std::vector<T> tw(th.tw.begin(), th.tw.end()), bc(bcd.begin(), bcd.end()), bz(bzd.begin(), bzd.end());
  const C2<T>* TW = (const C2<T>*)tw.data();
  const C2<T>* BC = (const C2<T>*)bc.data();
  const C2<T>* BZ = (const C2<T>*)bz.data();
  const int ld = padded_len<T>(2 * L);
  std::vector<T> A(ld), B(ld);
  auto fft = [&](T* src, T* dst) -> T* {
    int Ns = 1;
    for (int p = 0; p < g.npass; ++p) {
      const int R = g.radix[p];
      for (int b = 0; b < L / R; ++b) stockham_dispatch<T>(R, (const C2<T>*)src, (C2<T>*)dst, b, Ns, L, TW);
      Ns *= R;
      T* t = src; src = dst; dst = t;
    }
    return src;
  };
  for (int r = 0; r < howmany; ++r) {
    T* x = data + (size_t)r * (M - 1);
    for (int j = 0; j < ld; ++j) A[j] = B[j] = T(777);
    for (int j = 0; j < M - 1; ++j) A[pr<T>(j + 1)] = x[j];
    A[pr<T>(0)] = T(12345);  // index 0 must never be read
    for (int m = 0; m < L; ++m) blue_chirp_item<T>(A.data(), (C2<T>*)B.data(), m, M, BC);
    T* O = fft(B.data(), A.data());
    for (int k = 0; k < L; ++k) blue_mul_item<T>((C2<T>*)O, k, BZ);
    T* D = fft(O, O == A.data() ? B.data() : A.data());
    T* out = D == A.data() ? B.data() : A.data();
    for (int k = 0; k < M; ++k) blue_out_item<T>((const C2<T>*)D, out, k, T(1) / T(L), BC);
    for (int j = 0; j < M - 1; ++j) x[j] = out[pr<T>(j + 1)];
  }
}
extern "C" void dst_blue_run_f64(int M, int howmany, double* data) { run_blue<double>(M, howmany, data); }
extern "C" void dst_blue_run_f32(int M, int howmany, float* data) { run_blue<float>(M, howmany, data); }

extern "C" void dst_core_run_f64(int M, int howmany, double* data) { run<double>(M, howmany, data); }
extern "C" void dst_core_run_f32(int M, int howmany, float* data) { run<float>(M, howmany, data); }

// pass-ordered twiddles (fill_pass_twiddles) against their definition:
// returns the number of mismatching entries, or -1 if the count is wrong
extern "C" int dst_core_check_twp(int M) {
  DstGeom g = make_geom(M);
  DstTablesHost th = build_dst_tables(M);
  const int H = g.H;
  int bad = 0, count = 0, Ns = g.radix[0];
  for (int p = 1; p < g.npass; ++p) {
    const int R = g.radix[p];
    for (int q = 1; q < R; ++q)
      for (int k = 0; k < Ns; ++k) {
        const int e = (Ns - g.radix[0]) + (q - 1) * Ns + k;
        const double ang = 2.0 * M_PI * ((double)q * k * (H / (Ns * R))) / H;
        if (std::fabs(th.twp[2 * e] - std::cos(ang)) > 1e-15 || std::fabs(th.twp[2 * e + 1] + std::sin(ang)) > 1e-15)
          ++bad;
        ++count;
      }
    Ns *= R;
  }
  if (count != (g.npass > 1 ? H - g.radix[0] : 0)) return -1;
  return bad;
}

// the transform lengths the library accepts (M even, M/2 a product of 2, 3, 5, 7)
extern "C" int dst_core_length_ok(int M) { return transform_length_ok(M) ? 1 : 0; }
