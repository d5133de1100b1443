// CPU check of the device DST-I building blocks (qgw_gb300/csrc/dst_core.h):
// runs every phase's work items in a plain loop, exactly as the kernels
// spread them over threads, and exposes the result through a C function.
#include <cmath>
#include <vector>
#include <cstring>
#include "../../qgw_gb300/csrc/dst_tables.h"

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
