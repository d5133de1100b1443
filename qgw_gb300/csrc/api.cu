// api.cu -- the C ABI of libqgw_gpu.so (include/qgw_gpu.h): run creation,
// boundary copies in the reference layout, the device-resident step loop
// and diagnostics.  All device memory of a run is allocated in qgw_create
// and released in qgw_destroy.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/qgw_gpu.h"
#include "dst_tables.h"
#include "dst_warp.h"
#include "dst_blue.h"
#include "host.h"
#include "kernels.h"
#include "qgw_device.cuh"

using qgw::DevState;
using qgw::DstGeom;
using qgw::StepArgs;

#include "run.h"

namespace {

int cuda_fail(cudaError_t e) {
  if (e == cudaSuccess) return QGW_OK;
  if (e == cudaErrorMemoryAllocation) return QGW_ERR_NOMEM;
  return QGW_ERR_CUDA;
}
#define CK(x)                                  \
  do {                                         \
    cudaError_t e_ = (x);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_); \
  } while (0)

// row pitch of a periodic run's fields (and of the forcing spectra): the
// NX/2 + 1 complex values of a spectral row, rounded up to 16-byte rows
int periodic_pitch(int NX) { return (NX + 2 + 3) & ~3; }

template <typename T>
int dalloc(qgw_run* r, T** out, size_t count) {
  void* ptr = nullptr;
  cudaError_t e = cudaMalloc(&ptr, count * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_fail(e);
  r->allocs.push_back(ptr);
  e = cudaMemsetAsync(ptr, 0, count * sizeof(T) + 16, r->stream);
  if (e != cudaSuccess) return cuda_fail(e);
  *out = (T*)ptr;
  return QGW_OK;
}

template <typename T>
int upload(qgw_run* r, T** out, const std::vector<double>& host) {
  std::vector<T> tmp(host.begin(), host.end());
  int rc = dalloc(r, out, tmp.size());
  if (rc) return rc;
  CK(cudaMemcpyAsync(*out, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, r->stream));
  return cudaStreamSynchronize(r->stream) == cudaSuccess ? QGW_OK : QGW_ERR_CUDA;
}

// choose the modes per row block and the columns per column block so that
// each block's two work buffers stay within the shared-memory budget
// Shared-memory budget of the row kernels' work buffers.  Measured at
// 1024^2 x 10 on GB300: 64 KiB (3 blocks/SM) is fastest for FP64 and 40 KiB
// (4-5 blocks/SM) for FP32; QGW_ROW_SMEM_KB overrides it (tuning knob).
// Shared-memory budget of the work buffers of the forward rows kernel (K1):
// 48 KiB (FP64) / 56 KiB (FP32), which keeps four blocks per SM, and 40 KiB
// for FP32 rows of 2048 and more or more than 10 layers; measured at 512^2,
// 1024^2 and 2048^2 with 10, 16 and 20 layers on GB300 (1024^2 x 16 FP32:
// 0.254 -> 0.197 ms).  QGW_ROW_SMEM_KB overrides it.
size_t row_budget(size_t elem, int M, int nl) {
  const char* e = std::getenv("QGW_ROW_SMEM_KB");
  const long v = e ? std::atol(e) : 0;
  if (v >= 16 && v <= 220) return (size_t)v * 1024;
  if (elem == 4 && (M >= 2048 || nl > 10)) return (size_t)40 * 1024;
  return (size_t)(elem == 8 ? 48 : 56) * 1024;
}

// Layers per block of the inverse rows kernel (K3): the measured optimum is
// a fixed group size rather than a byte budget (each group re-reads the
// row's spectral data, while larger groups cost occupancy).  With the zeta
// rows: 3 layers, 5 for rows of 512 and less or more than 10 layers
// (1024^2 x 20 FP32: 0.477 -> 0.430 ms), 4 where the rows transform in place
// (one buffer per row; 1024^2 x 10 FP32: 0.127 -> 0.114 ms); without: 2, 4
// for more than 10 layers on rows of 1024 and less; within 110 KiB of work
// buffers.  QGW_INV_GROUP overrides the size.
int inv_group(int zeta, int M, int nl, int bufs) {
  const char* e = std::getenv("QGW_INV_GROUP");
  const int v = e ? std::atoi(e) : 0;
  if (v >= 1 && v <= 16) return v;
  if (zeta) return (M <= 512 || nl > 10) ? 5 : bufs == 1 ? 4 : 3;
  return (nl > 10 && M <= 1024) ? 4 : 2;
}

// Modes (layers) per block of a row kernel: as many as the budget holds (each
// takes rows_per_mode rows in each of the bufs DST work buffers), at most
// gmax and at most want, then balanced over the resulting number of groups.
int mode_group(int nl, int M, size_t elem, size_t budget, int rows_per_mode, int gmax, int want, int bufs = 2) {
  int g = (int)(budget / (bufs * (size_t)rows_per_mode * (elem == 4 ? qgw::padded_len<float>(M) : qgw::padded_len<double>(M)) * elem));
  if (g > want) g = want;
  if (g > gmax) g = gmax;
  if (g < 1) g = 1;
  const int ngroups = (nl + g - 1) / g;
  return (nl + ngroups - 1) / ngroups;
}

// The same for a kernel bound by its projection FMAs (the FP64 forward rows
// kernel): each group's loop runs at the compile-time width GB = the power
// of two at or above its size, so a group of 5 costs 8 FMAs per layer and
// point, and each group costs about 1.5 such FMAs more in fixed work (its
// pass over the layers, its barriers).  Among the sizes the budget allows,
// take the one of least groups x (GB + 1.5), then the fewest groups
// (fitted to GB300 sweeps of 256^2 and 512^2 x 5, 10, 20 layers: groups of
// 4 for 10 and 20 layers, one group for 5; 512^2 x 20: 0.579 -> 0.461 ms).
int mode_group_fma(int nl, int M, size_t elem, size_t budget, int gmax) {
  const int gfit = mode_group(1 << 30, M, elem, budget, 1, gmax, gmax);  // largest size that fits
  int best = 1, best_cost = 1 << 30, best_ng = 1 << 30;
  for (int g = 1; g <= gfit; ++g) {
    const int ng = (nl + g - 1) / g, s = (nl + ng - 1) / ng;
    int gb = 1;
    while (gb < s) gb <<= 1;
    const int cost = ng * (2 * gb + 3);
    if (cost < best_cost || (cost == best_cost && ng < best_ng)) { best = s; best_cost = cost; best_ng = ng; }
  }
  return best;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// libcuda link dependency); null when the driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)ptr;
  }();
  return fn;
}

// 3-D map (x, y, layer) of a run field for the RHS kernel's tile boxes:
// rhs_box_width() columns x `rows` rows x 1 layer; out-of-range elements
// read as zero.  The driver checks the base alignment, strides and box.
template <typename T>
bool encode_tile_map(CUtensorMap* m, const T* base, const qgw_run* r, int rows) {
  const cuuint64_t dims[3] = {(cuuint64_t)r->nx, (cuuint64_t)r->ny, (cuuint64_t)r->nl};
  const cuuint64_t strides[2] = {(cuuint64_t)r->pitch * sizeof(T), (cuuint64_t)r->lstride * sizeof(T)};
  const cuuint32_t box[3] = {(cuuint32_t)qgw::rhs_box_width(), (cuuint32_t)rows, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  const CUresult e = tmap_encoder()(m, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                                    3, (void*)base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return e == CUDA_SUCCESS;
}

// The RHS kernel's tensor maps for the run's tile height (boxes of TY + 2R
// psi rows, TY + 2 q rows, TY + 2R - 2 zeta rows), or element-wise copies
// when the driver cannot encode them, or when QGW_RHS_TILE_LOADS=copies asks
// for that path.
template <typename T>
void encode_rhs_maps(const qgw_run* r, StepArgs<T>& a) {
  std::memset(a.tm, 0, sizeof(a.tm));
  a.use_tma = 0;
  const char* loads = std::getenv("QGW_RHS_TILE_LOADS");
  if (!tmap_encoder() || (loads && !std::strcmp(loads, "copies"))) return;
  int R, ty;
  if constexpr (sizeof(T) == 8) {
    R = qgw::rhs_halo_of_f64(a);
    ty = qgw::rhs_tile_y_f64(a);
  } else {
    R = qgw::rhs_halo_of_f32c(a);
    ty = qgw::rhs_tile_y_f32c(a);
  }
  const int HH = ty + 2 * R;
  bool ok = encode_tile_map<T>(&a.tm[0], a.psi, r, HH) && encode_tile_map<T>(&a.tm[1], a.q, r, ty + 2);
  if (ok && a.zeta_mode == 1 && a.nsweep >= 1) ok = encode_tile_map<T>(&a.tm[2], a.zeta, r, HH - 2);
  a.use_tma = ok ? 1 : 0;
}

template <typename T>
int setup_args(qgw_run* r, StepArgs<T>& a) {
  const qgw_params& p = r->p;
  a.nx = r->nx;
  a.ny = r->ny;
  a.nl = r->nl;
  a.pitch = r->pitch;
  a.lstride = (long long)r->lstride;
  const bool per = p.bc_fac == -1;
  a.periodic = per ? 1 : 0;
  a.qin = nullptr;
  a.qout = nullptr;
  // closed basin: DST-I of length n along x and y (M = n + 1); periodic:
  // real FFT of length NX along x (a complex FFT of NX/2: M = NX) and
  // complex FFT of length NY along y (M = 2 NY)
  const int Mx = per ? r->nx : r->nx + 1, My = per ? 2 * r->ny : r->ny + 1;
  a.gx = per ? qgw::make_geom(Mx) : qgw::make_geom_any(Mx);
  a.gy = per ? qgw::make_geom(My) : qgw::make_geom_any(My);
  int rc;
  // transform tables for x and y
  for (int dim = 0; dim < 2; ++dim) {
    const qgw::DstGeom& g = dim == 0 ? a.gx : a.gy;
    // the chirp-z form's FFT is L = g.H points: its tables are those of a
    // half-length FFT of L (the DST tables of 2L), plus the chirp tables
    qgw::DstTablesHost th = qgw::build_dst_tables(g.blue ? 2 * g.H : g.M);
    std::vector<double> bcv(2, 0.0), bzv(2, 0.0);
    if (g.blue) qgw::build_blue_tables(g, bcv, bzv);
    T *tw, *pre, *spl, *twp, *sj, *twd, *sjp, *bc, *bz;
    if ((rc = upload<T>(r, &bc, bcv))) return rc;
    if ((rc = upload<T>(r, &bz, bzv))) return rc;
    if ((rc = upload<T>(r, &tw, th.tw))) return rc;
    if ((rc = upload<T>(r, &pre, th.pre))) return rc;
    if ((rc = upload<T>(r, &spl, th.spl))) return rc;
    if ((rc = upload<T>(r, &twp, th.twp))) return rc;
    if ((rc = upload<T>(r, &sj, th.sj))) return rc;
    if ((rc = upload<T>(r, &twd, th.twd))) return rc;
    if ((rc = upload<T>(r, &sjp, th.sjp))) return rc;
    qgw::DstTables<T>& t = dim == 0 ? a.tx : a.ty;
    t.tw = (const qgw::C2<T>*)tw;
    t.pre = (const qgw::C2<T>*)pre;
    t.spl = (const qgw::C2<T>*)spl;
    t.twp = (const qgw::C2<T>*)twp;
    t.sj = sj;
    t.twd = (const qgw::C2<T>*)twd;
    t.sjp = (const qgw::C2<T>*)sjp;
    t.bc = (const qgw::C2<T>*)bc;
    t.bz = (const qgw::C2<T>*)bz;
  }
  T *cl, *cm;
  if ((rc = upload<T>(r, &cl, r->cl2m))) return rc;
  if ((rc = upload<T>(r, &cm, r->cm2l))) return rc;
  a.cl2m = cl;
  a.cm2l = cm;
  double* ird;
  if ((rc = upload<double>(r, &ird, r->iRd2))) return rc;
  a.iRd2 = ird;
  const size_t field = (size_t)r->nl * r->lstride;
  if ((rc = dalloc(r, &a.q, field))) return rc;
  a.qlo = nullptr;
  if (r->precision == QGW_FP32C && (rc = dalloc(r, &a.qlo, field))) return rc;
  if ((rc = dalloc(r, &a.psi, field))) return rc;
  if ((rc = dalloc(r, &a.spec, field))) return rc;
  if ((rc = dalloc(r, &a.fab, 3 * field))) return rc;
  // squared wavenumbers: closed basin L_{k+1}, K_{j+1} (src/domain.h:170-173);
  // periodic K_k = 2 pi k / Lx along x (k <= NX/2) and L_j = 2 pi f(j) / Lx
  // along y with the signed frequency f(j) (src/domain.h:163-168), both with
  // Lx as the reference has them
  std::vector<double> Lsq(r->nx, 0.0), Ksq(r->ny);
  if (per) {
    for (int k = 0; k <= r->nx / 2; ++k) { const double L = 2 * M_PI * k / p.Lx; Lsq[k] = L * L; }
    for (int j = 0; j < r->ny; ++j) {
      const double K = 2 * M_PI / p.Lx * (((j + r->ny / 2) % r->ny) - r->ny / 2);
      Ksq[j] = K * K;
    }
  } else {
    for (int k = 0; k < r->nx; ++k) { const double L = M_PI * (k + 1) / p.Lx; Lsq[k] = L * L; }
    for (int j = 0; j < r->ny; ++j) { const double K = M_PI * (j + 1) / p.Lx; Ksq[j] = K * K; }
  }
  double *dL, *dK;
  if ((rc = upload<double>(r, &dL, Lsq))) return rc;
  if ((rc = upload<double>(r, &dK, Ksq))) return rc;
  a.Lsq = dL;
  a.Ksq = dK;
  float *fL, *fK;
  if ((rc = upload<float>(r, &fL, Lsq))) return rc;
  if ((rc = upload<float>(r, &fK, Ksq))) return rc;
  a.Lsqf = fL;
  a.Ksqf = fK;
  a.hinv = nullptr;
  if (r->precision == QGW_FP64) {
    // 1 / (fact * norm), fact = -(sq(L[i]) + sq(K[j]) + iRd2[k]) as in
    // invert_pv, src/elliptic.h:122-127 and the /norm of :134-138
    // periodic: one factor per complex value k <= NX/2; the mean is removed
    // (src/elliptic.h:103-117), a zero factor elsewhere is never hit
    std::vector<double> h(field, 0.0);
    const int nk = per ? r->nx / 2 + 1 : r->nx;
    for (int m = 0; m < r->nl; ++m)
      for (int j = 0; j < r->ny; ++j)
        for (int k = 0; k < nk; ++k) {
          const double fact = -(Lsq[k] + Ksq[j] + r->iRd2[m]);
          const bool mean = per && j == 0 && k == 0;
          h[(size_t)m * r->lstride + (size_t)j * r->pitch + k] = (mean || fact == 0) ? 0.0 : 1.0 / (fact * r->norm);
        }
    double* dh;
    if ((rc = upload<double>(r, &dh, h))) return rc;
    a.hinv = dh;
  }
  std::vector<double> wind(r->ny);
  for (int j = 0; j < r->ny; ++j) wind[j] = qgw_host_wind(&p, j + 1);
  T* dw;
  if ((rc = upload<T>(r, &dw, wind))) return rc;
  a.wind = dw;
  a.topo = nullptr;
  a.state = r->d_state;
  a.Delta = r->Delta;
  a.norm = r->norm;
  a.cfl = p.cfl;
  a.inv12d2 = 1.0 / (12. * r->Delta * r->Delta);
  a.b2d = p.beta / (2 * r->Delta);
  a.nu_d2 = p.nu / (r->Delta * r->Delta);
  a.has_nu = p.nu != 0;
  const double nuh = qgw_host_nu_hyper(&p);
  // calc_diff runs n_hyper/2+1 Laplacian sweeps (src/dynamics.h:25); the
  // term is nu_hyper * lap_n_diff, identically zero when nu_hyper == 0
  int sweeps = p.n_hyper >= 0 ? p.n_hyper / 2 + 1 : 0;
  if (nuh == 0) sweeps = 0;
  if (sweeps > 7) return QGW_ERR_UNSUPPORTED;
  a.nsweep = sweeps;
  a.nuh_scaled = sweeps ? nuh / std::pow(r->Delta, 2.0 * sweeps) : 0.0;
  a.cbc = 2 * p.bc_fac / (r->Delta * r->Delta);
  for (int s = 0; s < 8; ++s) a.gh[s] = (s >= 1) ? 2 * p.bc_fac * std::pow(r->Delta, 2.0 * s - 2) : 0.0;
  const double dhb = p.dh[r->nl - 1];
  a.drag_d2 = -p.hEkb * p.f0 / (2 * dhb) / (r->Delta * r->Delta);
  a.has_drag = p.hEkb != 0;
  a.topo_fac = p.f0 / dhb;
  a.has_topo = 0;
  a.has_wind = p.tau0 != 0;
  // work buffers per row of the row kernels' transforms (one: in place)
  const int bufs_x = (!per && !a.gx.blue && qgw::warp_dst_len(a.gx.H, (int)sizeof(T))) ? 1 : 2;
  // reals per row buffer (the chirp-z form holds L complex values)
  const int Mrow = a.gx.blue ? 2 * a.gx.H : Mx;
  {
    // QGW_ROW_GROUP overrides the modes per forward-rows block (tuning knob)
    const char* e = std::getenv("QGW_ROW_GROUP");
    const int want = e ? std::atoi(e) : 0;
    const size_t budget = row_budget(sizeof(T), Mrow, r->nl);
    if (want >= 1 && want <= 16) a.G1 = mode_group(r->nl, Mrow, sizeof(T), budget, 1, 16, want, bufs_x);
    else if (sizeof(T) == 8) a.G1 = mode_group_fma(r->nl, Mrow, sizeof(T), budget, 16);
    else a.G1 = mode_group(r->nl, Mrow, sizeof(T), budget, 1, 16, 16, bufs_x);
  }
  a.G3 = mode_group(r->nl, Mrow, sizeof(T), 110 * 1024, 1, 16, inv_group(0, Mrow, r->nl, bufs_x), bufs_x);
  a.CT = 0;
  a.low_k64 = 8;
  // 16-byte column vectors: rows 16-byte aligned and a whole number of
  // column tiles per row, so a tile never crosses into the next row
  const int ct = sizeof(T) == 8 ? qgw::cols_per_tile_f64() : qgw::cols_per_tile_f32c();
  a.vec_cols = ((size_t)r->pitch * sizeof(T)) % 16 == 0 && r->pitch % ct == 0;
  // compensated path: psi's FP32 round-off is white in wavenumber while psi
  // itself is dominated by the largest scales, so Laplacians of psi taken
  // by stencils lose ~(k_max/k_min)^2 of relative accuracy at grid scale.
  // The Laplacians are therefore formed spectrally with the exact symbol of
  // the 5-point stencil.  Where every sweep of calc_diff (src/dynamics.h:13-44)
  // sees zero ghosts (free-slip walls: adjust_bc sets lap_n_diff's ghosts to
  // 2 bc_fac/Delta^2 psi = 0) or wrapped ones (periodic), the whole chain
  // L^nsweep psi is diagonal in the transform basis and is formed there
  // (zeta_mode 2) when there is no bottom drag; otherwise the spectral
  // zeta = L psi starts the chain and feeds the bottom drag (zeta_mode 1):
  // the drag's Laplacian taken by the stencil of an FP32 psi raised the
  // error against FP64 at 1024^2 x 10 from 8.6e-7 to 5.5e-6 (q, 100 steps),
  // while a third spectral field for it would cost the column kernel one
  // more inverse transform per column than the tile's sweeps cost.
  // QGW_FP32C_DISSIPATION=zeta keeps zeta_mode 1 everywhere (comparisons).
  a.zeta_mode = 0;
  a.spec2 = nullptr;
  a.zeta = nullptr;
  const char* dmode = std::getenv("QGW_FP32C_DISSIPATION");
  const bool chain_diag = (p.bc_fac == 0 || per) && !a.has_drag && !(dmode && !std::strcmp(dmode, "zeta"));
  if (r->precision == QGW_FP32C && (a.nsweep > 0 || a.has_drag)) {
    a.zeta_mode = (chain_diag && a.nsweep > 0) ? 2 : 1;
    if ((rc = dalloc(r, &a.spec2, field))) return rc;
    if ((rc = dalloc(r, &a.zeta, field))) return rc;
    // K3 transforms psi and zeta rows of each mode: two rows per mode
    a.G3 = mode_group(r->nl, Mrow, sizeof(T), 110 * 1024, 2, 8, inv_group(1, Mrow, r->nl, bufs_x), bufs_x);
    // symbol of the 5-point Laplacian: DST-I basis sin^2(pi k / 2(n+1));
    // periodic Fourier basis sin^2(pi k / N)
    std::vector<double> sx(r->nx, 0.0), sy(r->ny);
    if (per) {
      for (int k = 0; k <= r->nx / 2; ++k) { const double s = std::sin(M_PI * k / r->nx); sx[k] = s * s; }
      for (int j = 0; j < r->ny; ++j) { const double s = std::sin(M_PI * j / r->ny); sy[j] = s * s; }
    } else {
      for (int k = 0; k < r->nx; ++k) { const double s = std::sin(M_PI * (k + 1) / (2.0 * (r->nx + 1))); sx[k] = s * s; }
      for (int j = 0; j < r->ny; ++j) { const double s = std::sin(M_PI * (j + 1) / (2.0 * (r->ny + 1))); sy[j] = s * s; }
    }
    double *dsx, *dsy;
    if ((rc = upload<double>(r, &dsx, sx))) return rc;
    if ((rc = upload<double>(r, &dsy, sy))) return rc;
    a.sx2 = dsx;
    a.sy2 = dsy;
    float *fsx, *fsy;
    if ((rc = upload<float>(r, &fsx, sx))) return rc;
    if ((rc = upload<float>(r, &fsy, sy))) return rc;
    a.sx2f = fsx;
    a.sy2f = fsy;
    a.lx2 = -4.0 / (r->Delta * r->Delta);
    a.ly2 = a.lx2;
  }
  // stochastic ring forcing (src/forcing.h:67-201); the reference forces
  // only when the ring has more than one point (:172)
  std::memset(&a.fr, 0, sizeof(a.fr));
  {
    std::vector<int> ij;
    const int NP = qgw_host_forcing_ring(&p, &ij);
    if (NP > 1) {
      qgw::ForcArgs<T>& f = a.fr;
      f.on = 1;
      f.nring = NP;
      f.NF = p.NX;
      f.fpitch = periodic_pitch(p.NX);
      int imax = 0;
      for (size_t k = 0; k < ij.size(); k += 2) imax = std::max(imax, ij[k]);
      f.col_blocks = imax / 2 + 1;
      f.gx = qgw::make_geom(f.NF);
      f.gy = qgw::make_geom(2 * f.NF);
      for (int dim = 0; dim < 2; ++dim) {
        qgw::DstTablesHost th = qgw::build_dst_tables(dim == 0 ? f.NF : 2 * f.NF);
        T *tw, *pre, *spl;
        if ((rc = upload<T>(r, &tw, th.tw))) return rc;
        if ((rc = upload<T>(r, &pre, th.pre))) return rc;
        if ((rc = upload<T>(r, &spl, th.spl))) return rc;
        qgw::DstTables<T>& t = dim == 0 ? f.tx : f.ty;
        t.tw = (const qgw::C2<T>*)tw;
        t.pre = (const qgw::C2<T>*)pre;
        t.spl = (const qgw::C2<T>*)spl;
      }
      int* dring;
      if ((rc = dalloc(r, &dring, ij.size()))) return rc;
      CK(cudaMemcpyAsync(dring, ij.data(), sizeof(int) * ij.size(), cudaMemcpyHostToDevice, r->stream));
      f.ring = dring;
      const double kf = p.k_f / (2 * M_PI);
      f.env = std::sqrt((double)8 / ((NP - 1) * 2)) * M_PI * kf;
      f.sigma = p.sigma_f;
      qgw::GlibcRand g;
      qgw::glibc_rand_seed(&g, 1);  // rand() of a fresh process
      if ((rc = dalloc(r, &f.rng, 1))) return rc;
      CK(cudaMemcpyAsync(f.rng, &g, sizeof(g), cudaMemcpyHostToDevice, r->stream));
      if ((rc = dalloc(r, &f.spec, (size_t)f.NF * f.fpitch))) return rc;
      if ((rc = dalloc(r, &f.spec2, (size_t)f.NF * f.fpitch))) return rc;
      if ((rc = dalloc(r, &f.field, (size_t)r->ny * r->pitch))) return rc;
      CK(cudaStreamSynchronize(r->stream));
    }
  }
  // FP32 copies of the constants of the compensated kernels (one rounding
  // of the same double expressions the FP64 kernels use)
  std::memset(a.fc, 0, sizeof(a.fc));
  a.fc[qgw::FC_D2] = (float)(r->Delta * r->Delta);
  a.fc[qgw::FC_CBC] = (float)a.cbc;
  a.fc[qgw::FC_MINV12] = (float)(-a.inv12d2);
  a.fc[qgw::FC_B2D] = (float)a.b2d;
  a.fc[qgw::FC_NUD2] = (float)a.nu_d2;
  a.fc[qgw::FC_NUH] = (float)a.nuh_scaled;
  a.fc[qgw::FC_DRAG] = (float)a.drag_d2;
  a.fc[qgw::FC_TOPOC] = (float)(-(a.inv12d2 * a.topo_fac));
  for (int g = 1; g <= 4; ++g) {
    a.fc[qgw::FC_GH1 + g - 1] = (float)a.gh[g];
    a.fc[qgw::FC_GHD1 + g - 1] = (float)(a.gh[g] / (r->Delta * r->Delta));
  }
  a.fc[qgw::FC_NORM] = (float)r->norm;
  a.fc[qgw::FC_NUHS] = (float)nuh;
  a.fc[qgw::FC_NUHD2] = (float)(a.nuh_scaled * r->Delta * r->Delta);
  a.fc[qgw::FC_LX2] = (float)a.lx2;
  a.fc[qgw::FC_LY2] = (float)a.ly2;
  float* fi;
  if ((rc = upload<float>(r, &fi, r->iRd2))) return rc;
  a.iRd2f = fi;
  // column tiles of 32-byte rows, or 16-byte rows where the former's
  // buffers would pass 200 KiB of shared memory (long columns with the
  // second spectral field: FP32 NY = 2048 in zeta mode) and for the chirp-z
  // form's columns (its kernels are built for 16-byte tiles and for one
  // column per tile), whose long buffers (two per column) take one column per
  // tile where 16-byte rows would pass 200 KiB (chirp-z lengths above 512 in
  // FP32c, 1024 in FP64)
  {
    auto need = [&]() -> size_t {
      if constexpr (sizeof(T) == 8) return qgw::smem_bytes_cols_f64(a);
      else return qgw::smem_bytes_cols_f32c(a);
    };
    const size_t limit = (size_t)200 * 1024;
    if (a.gy.blue) a.CT = (32 / (int)sizeof(T)) / 2;
    if (need() > limit) a.CT = (32 / (int)sizeof(T)) / 2;
    if (a.gy.blue && need() > limit) a.CT = 1;
  }
  // TMA tensor maps of the RHS kernel's tiles (psi with halo R, q with halo
  // 1, in zeta mode 1 zeta over the first sweep's region; zeta mode 2 reads
  // its field point by point)
  a.rhs_grid = 0;
  // work-tile shape: RHS tiles of 16 rows (QGW_RHS_TILE_ROWS=32: 32 rows),
  // the default column-tile width (a.CT = 0); qgw_set_shape changes them
  a.rhs_ty = 16;
  if (const char* e = std::getenv("QGW_RHS_TILE_ROWS")) a.rhs_ty = std::atoi(e) == 32 ? 32 : 16;
  encode_rhs_maps<T>(r, a);
  // K3 over rows x layer groups in FP64 (measured at 1024^2 x 10: 0.575 ->
  // 0.552 ms); the FP32c kernel keeps one block per row (0.109 against 0.123
  // ms split).  QGW_INV_SPLIT=0/1 overrides.
  a.inv_split = sizeof(T) == 8;
  if (const char* e = std::getenv("QGW_INV_SPLIT")) a.inv_split = std::atoi(e) != 0;
  // QGW_TEST_FIRST_WAIT_ITERS (tests of the timeout path only) lowers the
  // limit of the first wait for a tile's TMA bytes, down to 0 polls; the
  // second wait keeps the full limit, so the bytes still land before the
  // block moves on
  a.wait_iters = qgw::kWaitIters;
  if (const char* w = std::getenv("QGW_TEST_FIRST_WAIT_ITERS")) {
    const long v = std::strtol(w, nullptr, 10);
    a.wait_iters = v < 0 ? 0 : v > qgw::kWaitIters ? qgw::kWaitIters : (int)v;
  }
  return QGW_OK;
}

// Work-tile shape of a run (qgw_set_shape): validated on a copy of the
// run's arguments, whose shared-memory needs must fit the device, then
// applied.  None of the choices changes any arithmetic.
template <typename T>
int set_shape(qgw_run* r, StepArgs<T>& a, const qgw_shape& sh) {
  StepArgs<T> b = a;
  if (sh.rhs_tile_rows) {
    if (sh.rhs_tile_rows != 16 && sh.rhs_tile_rows != 32) return QGW_ERR_PARAM;
    b.rhs_ty = sh.rhs_tile_rows;
  }
  const int ctd = 32 / (int)sizeof(T);
  if (sh.col_tile) {
    if (a.gy.blue) {
      // the chirp-z columns keep the width chosen at creation
      if (sh.col_tile != a.CT) return QGW_ERR_PARAM;
    } else {
      if (sh.col_tile != ctd && sh.col_tile != ctd / 2) return QGW_ERR_PARAM;
      b.CT = sh.col_tile == ctd ? 0 : sh.col_tile;
    }
  }
  const bool per = a.periodic != 0;
  const int bufs_x = (!per && !a.gx.blue && qgw::warp_dst_len(a.gx.H, (int)sizeof(T))) ? 1 : 2;
  const int Mx = a.gx.blue ? 2 * a.gx.H : per ? r->nx : r->nx + 1;  // reals per row buffer
  const size_t any = (size_t)1 << 30;  // the device's limit is checked below
  if (sh.row_group_fwd) {
    if (sh.row_group_fwd < 1 || sh.row_group_fwd > 16) return QGW_ERR_PARAM;
    b.G1 = mode_group(r->nl, Mx, sizeof(T), any, 1, 16, sh.row_group_fwd, bufs_x);
  }
  if (sh.row_group_inv) {
    if (sh.row_group_inv < 1 || sh.row_group_inv > 16) return QGW_ERR_PARAM;
    const bool zm = a.zeta_mode != 0;
    b.G3 = mode_group(r->nl, Mx, sizeof(T), any, zm ? 2 : 1, zm ? 8 : 16, sh.row_group_inv, bufs_x);
  }
  if (b.rhs_ty != a.rhs_ty) encode_rhs_maps<T>(r, b);
  cudaError_t e;
  if constexpr (sizeof(T) == 8) e = qgw::prepare_f64(b);
  else e = qgw::prepare_f32c(b);
  if (e == cudaErrorInvalidValue) return QGW_ERR_PARAM;  // beyond the device's shared memory
  if (e != cudaSuccess) return QGW_ERR_CUDA;
  if constexpr (sizeof(T) == 8) b.rhs_grid = qgw::rhs_grid_f64(b);
  else b.rhs_grid = qgw::rhs_grid_f32c(b);
  a = b;
  return QGW_OK;
}

template <typename T>
void get_shape(const StepArgs<T>& a, qgw_shape* sh) {
  sh->rhs_tile_rows = a.rhs_ty == 32 ? 32 : 16;
  sh->col_tile = a.CT ? a.CT : 32 / (int)sizeof(T);
  sh->row_group_fwd = a.G1;
  sh->row_group_inv = a.G3;
}

}  // namespace

extern "C" {

int qgw_abi_version(void) { return QGW_ABI_VERSION; }

int qgw_set_shape(qgw_run* r, const qgw_shape* sh) {
  if (!r || !sh) return QGW_ERR_PARAM;
  if (cudaStreamSynchronize(r->stream) != cudaSuccess) return QGW_ERR_CUDA;
  return r->precision == QGW_FP64 ? set_shape<double>(r, r->a64, *sh) : set_shape<float>(r, r->a32, *sh);
}

int qgw_get_shape(qgw_run* r, qgw_shape* sh) {
  if (!r || !sh) return QGW_ERR_PARAM;
  if (r->precision == QGW_FP64) get_shape<double>(r->a64, sh);
  else get_shape<float>(r->a32, sh);
  return QGW_OK;
}

const char* qgw_strerror(int s) {
  switch (s) {
    case QGW_OK: return "ok";
    case QGW_ERR_PARAM: return "invalid parameter";
    case QGW_ERR_FILE: return "params file not found";
    case QGW_ERR_CUDA: return "CUDA runtime error";
    case QGW_ERR_NOMEM: return "out of memory";
    case QGW_ERR_NAN: return "non-finite value in the state";
    case QGW_ERR_UNSUPPORTED: return "configuration not supported by the GPU kernels";
    case QGW_ERR_EIGEN: return "stretching-matrix eigensolver failed";
    case QGW_ERR_STATE: return "call out of order";
    case QGW_ERR_ADMISSION: return "request exceeds the HBM budget";
    case QGW_ERR_TIMEOUT: return "device wait timed out";
    case QGW_ERR_NOT_READY: return "result not ready";
    default: return "unknown status";
  }
}

int qgw_footprint(const qgw_params* p, int precision, size_t* bytes) {
  if (!p || !bytes) return QGW_ERR_PARAM;
  const bool per = p->bc_fac == -1;
  const size_t nx = p->NX - (per ? 0 : 1), ny = p->NY - (per ? 0 : 1);
  const size_t field = (size_t)p->nl * ny * (per ? (size_t)periodic_pitch(p->NX) : nx + 1);
  size_t b;
  if (precision == QGW_FP64) b = field * 8 * 7;  // q psi spec f0 f1 f2 hinv
  else b = field * 4 * 9;                        // q_hi q_lo psi spec spec2 zeta f0 f1 f2
  b += (size_t)p->nl * (ny + 2) * (nx + 2) * 8;  // reference-layout staging for host copies
  if (p->k_f != 0) b += (size_t)3 * p->NX * periodic_pitch(p->NX) * (precision == QGW_FP64 ? 8 : 4);  // forcing
  *bytes = b + (size_t)(nx + ny) * 64 + (1 << 20);
  return QGW_OK;
}

int qgw_create(const qgw_params* pin, const double* cl2m, const double* cm2l, const double* iRd2,
               const double* topo, int precision, qgw_run** out) {
  if (!pin || !out) return QGW_ERR_PARAM;
  *out = nullptr;
  if (precision != QGW_FP64 && precision != QGW_FP32C) return QGW_ERR_PARAM;
  const qgw_params& p = *pin;
  const bool per = p.bc_fac == -1;
  // negative bc_fac other than the periodic flag has no meaning in the reference
  if (p.bc_fac < 0 && !per) return QGW_ERR_UNSUPPORTED;
  // periodic: the reference's r2c layout (src/elliptic.h:26,45) is only
  // consistent for a square grid; the real FFT needs NX >= 8
  if (per && (p.NX != p.NY || p.NX < 8)) return QGW_ERR_UNSUPPORTED;
  if (p.dt_forc_period != 0) {
    // init_4d_forcing's checks (src/forcing.h:236-250), as errors
    if (p.dt_forc == 0) return QGW_ERR_PARAM;
    const int n_rec = (int)std::floor(p.dt_forc_period / p.dt_forc);
    if (n_rec < 1 || n_rec * p.dt_forc != p.dt_forc_period) return QGW_ERR_PARAM;
  }
  // transform lengths: closed DST-I of M = NX, NY (any M >= 4: the
  // half-length FFT where M is even with M/2 a product of 2, 3, 5 and 7,
  // else the chirp-z form); periodic real FFT of NX and complex FFT of NY
  // (M = 2 NY), which take only the former
  if (p.NX > 8192 || p.NY > 8192) return QGW_ERR_UNSUPPORTED;
  if (p.NX < 4 || p.NY < 4) return QGW_ERR_UNSUPPORTED;
  if (per && (!qgw::transform_length_ok(p.NX) || !qgw::transform_length_ok(2 * p.NY))) return QGW_ERR_UNSUPPORTED;
  if (p.nl < 1 || p.nl > QGW_NL_GPU_MAX) return QGW_ERR_UNSUPPORTED;
  if (!(p.Lx > 0) || !(p.cfl > 0)) return QGW_ERR_PARAM;
  qgw_run* r = new qgw_run();
  r->precision = precision;
  r->p = p;
  r->nx = per ? p.NX : p.NX - 1;
  r->ny = per ? p.NY : p.NY - 1;
  r->nl = p.nl;
  // periodic rows also hold the NX/2 + 1 complex values of a spectral row
  r->pitch = per ? periodic_pitch(p.NX) : r->nx + 1;
  r->lstride = (size_t)r->ny * r->pitch;
  r->Delta = p.Lx / p.NX;
  r->Ly = p.NY * r->Delta;
  r->norm = per ? (double)p.NX * p.NY : 4.0 * (r->nx + 1) * (r->ny + 1);
  r->cl2m.resize((size_t)r->nl * r->nl);
  r->cm2l.resize((size_t)r->nl * r->nl);
  r->iRd2.resize(r->nl);
  int rc = QGW_OK;
  if (cl2m && cm2l && iRd2) {
    std::memcpy(r->cl2m.data(), cl2m, sizeof(double) * r->nl * r->nl);
    std::memcpy(r->cm2l.data(), cm2l, sizeof(double) * r->nl * r->nl);
    std::memcpy(r->iRd2.data(), iRd2, sizeof(double) * r->nl);
  } else if ((rc = qgw_eigmode(&p, r->cl2m.data(), r->cm2l.data(), r->iRd2.data()))) {
    delete r;
    return rc;
  }
  auto fail = [&](int code) {
    qgw_destroy(r);
    return code;
  };
  if (cudaGetDevice(&r->device) != cudaSuccess) return fail(QGW_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(QGW_ERR_CUDA);
  if (cudaMallocHost(&r->h_state, sizeof(DevState)) != cudaSuccess) return fail(QGW_ERR_NOMEM);
  if ((rc = dalloc(r, &r->d_state, 1))) return fail(rc);
  if (precision == QGW_FP64) {
    if ((rc = setup_args<double>(r, r->a64))) return fail(rc);
  } else {
    if ((rc = setup_args<float>(r, r->a32))) return fail(rc);
  }
  {
    const size_t nfull = (size_t)r->nl * (r->ny + 2) * (r->nx + 2);
    if ((rc = dalloc(r, &r->d_full, nfull))) return fail(rc);
  }
  // topography: explicit array, or the analytic shelf when h_topo != 0
  std::vector<double> th;
  const double* tsrc = topo;
  if (!tsrc && p.h_topo != 0) {
    th.resize((size_t)(r->nx + 2) * (r->ny + 2));
    qgw_topo(&p, th.data());
    tsrc = th.data();
  }
  if (tsrc) {
    bool nz = false;
    const size_t n2 = (size_t)(r->nx + 2) * (r->ny + 2);
    for (size_t s = 0; s < n2 && !nz; ++s) nz = tsrc[s] != 0;
    if (nz) {
      std::vector<double> tv(tsrc, tsrc + n2);
      double* dt;
      if ((rc = upload<double>(r, &dt, tv))) return fail(rc);
      r->a64.topo = dt;
      r->a64.has_topo = 1;
      r->a32.topo = dt;
      r->a32.has_topo = 1;
    }
  }
  // FP64 diagnostics buffers
  std::vector<double> w(r->nl);
  double H = 0;
  for (int k = 0; k < r->nl; ++k) H += p.dh[k];
  for (int k = 0; k < r->nl; ++k) w[k] = p.dh[k] / H;
  if ((rc = upload<double>(r, &r->d_wts, w))) return fail(rc);
  r->budget_blocks = 304;
  if ((rc = dalloc(r, &r->d_part, (size_t)4 * r->budget_blocks))) return fail(rc);
  if ((rc = dalloc(r, &r->d_bout, 4))) return fail(rc);
  // initial time scalars: init_timestep (src/timestep.h:56-67), or the
  // fixed dt of the optional `dt` key
  DevState s{};
  double DT, dt0;
  if ((rc = qgw_check_timestep(&p, &DT, &dt0))) return fail(rc);
  if (p.dt > 0) { DT = p.dt; dt0 = p.dt; }
  s.t = 0; s.dt = dt0; s.dt0 = dt0; s.dt1 = dt0; s.DT_max = DT;
  if (cudaMemcpyAsync(r->d_state, &s, sizeof(s), cudaMemcpyHostToDevice, r->stream) != cudaSuccess)
    return fail(QGW_ERR_CUDA);
  cudaError_t e = precision == QGW_FP64 ? qgw::prepare_f64(r->a64) : qgw::prepare_f32c(r->a32);
  // a configuration whose work buffers pass the device's shared memory (the
  // chirp-z form's rows of long, odd or prime-sized grids) is refused
  if (e == cudaErrorInvalidValue) return fail(QGW_ERR_UNSUPPORTED);
  if (e != cudaSuccess) return fail(cuda_fail(e));
  // persistent grid of the RHS kernel (after the shared-memory limits are set)
  if (precision == QGW_FP64) r->a64.rhs_grid = qgw::rhs_grid_f64(r->a64);
  else r->a32.rhs_grid = qgw::rhs_grid_f32c(r->a32);
  if (cudaStreamSynchronize(r->stream) != cudaSuccess) return fail(QGW_ERR_CUDA);
  *out = r;
  return QGW_OK;
}

void qgw_destroy(qgw_run* r) {
  if (!r) return;
  if (r->stream) cudaStreamSynchronize(r->stream);
  for (void* ptr : r->allocs) cudaFree(ptr);
  if (r->h_state) cudaFreeHost(r->h_state);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
}

void* qgw_stream(qgw_run* r) { return r ? (void*)r->stream : nullptr; }
int qgw_kernels_per_step(qgw_run* r) { return r ? 4 : 0; }

static int reset_history(qgw_run* r) {
  const size_t field = (size_t)r->nl * r->lstride;
  void* fab = r->precision == QGW_FP64 ? (void*)r->a64.fab : (void*)r->a32.fab;
  const size_t esz = r->precision == QGW_FP64 ? 8 : 4;
  CK(cudaMemsetAsync(fab, 0, 3 * field * esz, r->stream));
  // pending = 0, step_index = 0, maxbits = 0, done_blocks = 0
  DevState* d = r->d_state;
  CK(cudaMemsetAsync(&d->maxbits, 0, sizeof(unsigned long long), r->stream));
  CK(cudaMemsetAsync(&d->done_blocks, 0, sizeof(unsigned int), r->stream));
  CK(cudaMemsetAsync(&d->pending, 0, sizeof(int), r->stream));
  CK(cudaMemsetAsync(&d->step_index, 0, sizeof(int), r->stream));
  CK(cudaMemsetAsync(&d->forc_step, 0, sizeof(int), r->stream));
  CK(cudaMemsetAsync(&d->nonfinite, 0, sizeof(int), r->stream));
  CK(cudaMemsetAsync(&d->dev_error, 0, sizeof(int), r->stream));
  return QGW_OK;
}

// A device-usable address of a host array, or null: pinned (registered)
// memory through its mapped address; pageable memory itself where the GPU
// reads host page tables (the Grace C2C link's address translation).
// QGW_HOST_ACCESS=copy turns this off (every host array then crosses the
// link as one copy-engine transfer through the staging buffer).
static const void* device_view(const qgw_run* r, const void* host) {
  static const int mode = [] {
    const char* e = std::getenv("QGW_HOST_ACCESS");
    return (e && !std::strcmp(e, "copy")) ? 0 : 1;
  }();
  if (!mode || !host) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeHost) return at.devicePointer;
  if (at.type == cudaMemoryTypeUnregistered) {
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, r->device) ==
            cudaSuccess &&
        pageable)
      return host;
  }
  return nullptr;
}

// q in the reference layout -> the run layout: the unpack kernel reads the
// caller's array where the device can address it (host arrays over the
// C2C link), else one contiguous copy into the staging buffer first
static int load_q(qgw_run* r, const double* q, bool device_src) {
  const double* full = q;
  const double* view = device_src ? nullptr : (const double*)device_view(r, q);
  if (view) {
    full = view;
  } else if (!device_src) {
    const size_t nfull = (size_t)r->nl * (r->ny + 2) * (r->nx + 2);
    CK(cudaMemcpyAsync(r->d_full, q, sizeof(double) * nfull, cudaMemcpyHostToDevice, r->stream));
    full = r->d_full;
  }
  if (r->precision == QGW_FP64)
    qgw::enqueue_unpack_f64(full, r->a64.q, r->nx, r->ny, r->nl, r->pitch, r->stream);
  else
    qgw::enqueue_unpack_split(full, r->a32.q, r->a32.qlo, r->nx, r->ny, r->nl, r->pitch, r->stream);
  return QGW_OK;
}

static int set_q_impl(qgw_run* r, const double* q, bool device_src) {
  if (!r || !q) return QGW_ERR_PARAM;
  int rc = load_q(r, q, device_src);
  if (rc) return rc;
  if ((rc = reset_history(r))) return rc;
  CK(cudaStreamSynchronize(r->stream));
  CK(cudaGetLastError());
  r->has_q = true;
  return QGW_OK;
}

int qgw_set_q(qgw_run* r, const double* q) { return set_q_impl(r, q, false); }
int qgw_set_q_device(qgw_run* r, const double* q) { return set_q_impl(r, q, true); }

int qgw_put_q(qgw_run* r, const double* q) {
  if (!r || !q) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  int rc = load_q(r, q, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(r->stream));
  CK(cudaGetLastError());
  return QGW_OK;
}

int qgw_get_time(qgw_run* r, qgw_time* out) {
  if (!r || !out) return QGW_ERR_PARAM;
  CK(cudaMemcpyAsync(r->h_state, r->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  out->t = r->h_state->t;
  out->dt = r->h_state->dt;
  out->dt0 = r->h_state->dt0;
  out->dt1 = r->h_state->dt1;
  out->DT_max = r->h_state->DT_max;
  return QGW_OK;
}

}  // extern "C"

template <typename T>
static int set_records(qgw_run* r, StepArgs<T>& a, const double* rec, int n_rec) {
  const size_t rs = (size_t)r->nl * r->lstride;
  const int nxp2 = r->nx + 2, nyp2 = r->ny + 2;
  std::vector<T> h(rs * n_rec, T(0));
  for (int n = 0; n < n_rec; ++n)
    for (int l = 0; l < r->nl; ++l)
      for (int j = 0; j < r->ny; ++j)
        for (int i = 0; i < r->nx; ++i)
          h[n * rs + (size_t)l * r->lstride + (size_t)j * r->pitch + i] =
              (T)rec[(((size_t)n * r->nl + l) * nyp2 + (j + 1)) * nxp2 + (i + 1)];
  if (!a.frec) {
    T* d;
    int rc = dalloc(r, &d, h.size());
    if (rc) return rc;
    a.frec = d;
  }
  CK(cudaMemcpyAsync((void*)a.frec, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  a.nrec = n_rec;
  a.dt_forc = r->p.dt_forc;
  return QGW_OK;
}

extern "C" {

int qgw_set_forcing_records(qgw_run* r, const double* rec, int nrec) {
  if (!r || !rec) return QGW_ERR_PARAM;
  if (r->p.dt_forc_period == 0) return QGW_ERR_STATE;
  const int n_rec = (int)std::floor(r->p.dt_forc_period / r->p.dt_forc);
  if (nrec < n_rec) return QGW_ERR_PARAM;
  return r->precision == QGW_FP64 ? set_records<double>(r, r->a64, rec, n_rec)
                                  : set_records<float>(r, r->a32, rec, n_rec);
}

int qgw_set_forcing_seed(qgw_run* r, unsigned int seed) {
  if (!r) return QGW_ERR_PARAM;
  qgw::GlibcRand* rng = r->precision == QGW_FP64 ? r->a64.fr.rng : r->a32.fr.rng;
  if (!rng) return QGW_ERR_STATE;
  qgw::GlibcRand g;
  qgw::glibc_rand_seed(&g, seed);
  CK(cudaMemcpyAsync(rng, &g, sizeof(g), cudaMemcpyHostToDevice, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  return QGW_OK;
}

int qgw_set_time(qgw_run* r, const qgw_time* in) {
  if (!r || !in) return QGW_ERR_PARAM;
  double v[5] = {in->t, in->dt, in->dt0, in->dt1, in->DT_max};
  CK(cudaMemcpyAsync(r->d_state, v, sizeof(v), cudaMemcpyHostToDevice, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  return QGW_OK;
}

static void enqueue_invert(qgw_run* r) {
  if (r->precision == QGW_FP64) qgw::enqueue_invert_f64(r->a64, r->stream);
  else qgw::enqueue_invert_f32c(r->a32, r->stream);
}

int qgw_step(qgw_run* r, int nsteps, double t_out, double tend, qgw_step_info* info) {
  if (!r) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  if (r->p.dt_forc_period != 0 && (r->precision == QGW_FP64 ? r->a64.nrec : r->a32.nrec) == 0)
    return QGW_ERR_STATE;  // 4-D forcing records not set
  if (nsteps < 0) return QGW_ERR_PARAM;
  qgw::enqueue_begin(r->d_state, t_out, tend, r->stream);
  const int chunk = 256;
  int launched = 0;
  while (launched < nsteps) {
    const int n = (nsteps - launched) < chunk ? (nsteps - launched) : chunk;
    for (int s = 0; s < n; ++s) {
      if (r->precision == QGW_FP64) qgw::enqueue_step_f64(r->a64, r->stream);
      else qgw::enqueue_step_f32c(r->a32, r->stream);
      // a host q (qgw_step_host) is read by the first step only
      r->a64.qin = nullptr;
      r->a32.qin = nullptr;
    }
    launched += n;
    if (launched < nsteps) {
      // stop launching once the device loop has ended
      CK(cudaMemcpyAsync(r->h_state, r->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, r->stream));
      CK(cudaStreamSynchronize(r->stream));
      if (!r->h_state->active) break;
    }
  }
  if (r->precision == QGW_FP64) qgw::enqueue_flush_f64(r->a64, r->stream);
  else qgw::enqueue_flush_f32c(r->a32, r->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(r->h_state, r->d_state, sizeof(DevState), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  const DevState& s = *r->h_state;
  if (info) {
    info->time.t = s.t;
    info->time.dt = s.dt;
    info->time.dt0 = s.dt0;
    info->time.dt1 = s.dt1;
    info->time.DT_max = s.DT_max;
    info->steps_taken = s.steps_taken;
    info->stop_reason = s.stop_reason;
    info->nonfinite = s.nonfinite;
  }
  if (s.dev_error) return QGW_ERR_TIMEOUT;  // a bounded device wait ran out
  return s.nonfinite ? QGW_ERR_NAN : QGW_OK;
}

static void fill_ghosts(const qgw_run* r, double* psi, double* q, const double* ps);

// qgw_step with the caller's q going in and out (the reference's
// timestep(q) on a host array, n times): q_in replaces q keeping the AB3
// history (as qgw_put_q), read by the first kernel of the call straight from
// the host array where the device can address it; q_out receives q after
// the steps (as qgw_get).  q_in and q_out may be the same array.
int qgw_step_host(qgw_run* r, int nsteps, double t_out, double tend, const double* q_in, double* q_out,
                  qgw_step_info* info) {
  if (!r) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  int rc;
  // the direct read needs the first step to run: no t_out / tend stop
  const bool direct = q_in && nsteps > 0 && t_out == 0 && tend == 0;
  const double* view = direct ? (const double*)device_view(r, q_in) : nullptr;
  if (q_in && !view && (rc = load_q(r, q_in, false))) return rc;
  // q out: the end-of-call flush writes the interior into the caller's array
  // where the device can address it and the ghost ring needs no psi
  // (free-slip or periodic); otherwise as qgw_get
  double* oview = q_out && (r->p.bc_fac == 0 || r->p.bc_fac == -1) ? (double*)device_view(r, q_out) : nullptr;
  if (r->precision == QGW_FP64) {
    r->a64.qin = view;
    r->a64.qout = oview;
  } else {
    r->a32.qin = view;
    r->a32.qout = oview;
  }
  rc = qgw_step(r, nsteps, t_out, tend, info);
  r->a64.qin = r->a32.qin = nullptr;
  r->a64.qout = r->a32.qout = nullptr;
  if (rc != QGW_OK && rc != QGW_ERR_NAN) return rc;
  int rc2 = QGW_OK;
  if (oview) fill_ghosts(r, nullptr, q_out, nullptr);
  else if (q_out) rc2 = qgw_get(r, nullptr, q_out);
  return rc2 != QGW_OK ? rc2 : rc;
}

int qgw_invert(qgw_run* r) {
  if (!r) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  enqueue_invert(r);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(r->stream));
  return QGW_OK;
}

// Ghost rings as adjust_bc leaves them after invert_pv (src/elliptic.h:152-153,
// src/domain.h:308-348): periodic copies; at walls psi = 0 and
// q = 2 bc_fac / Delta^2 * psi_adjacent (ps: psi, needed when bc_fac != 0).
static void fill_ghosts(const qgw_run* r, double* psi, double* q, const double* ps) {
  const int nxp2 = r->nx + 2, nyp2 = r->ny + 2;
  const size_t L = (size_t)nxp2 * nyp2;
  if (r->p.bc_fac == -1) {
    // periodic copies, South, North, West, East in turn (src/domain.h:225-256)
    for (double* F : {psi, q}) {
      if (!F) continue;
      for (int k = 0; k < r->nl; ++k) {
        double* f = F + k * L;
        for (int i = 0; i < nxp2; ++i) f[i] = f[(size_t)r->ny * nxp2 + i];
        for (int i = 0; i < nxp2; ++i) f[(size_t)(nyp2 - 1) * nxp2 + i] = f[(size_t)nxp2 + i];
        for (int j = 0; j < nyp2; ++j) f[(size_t)j * nxp2] = f[(size_t)j * nxp2 + r->nx];
        for (int j = 0; j < nyp2; ++j) f[(size_t)j * nxp2 + nxp2 - 1] = f[(size_t)j * nxp2 + 1];
      }
    }
    return;
  }
  const double c = 2 * r->p.bc_fac / (r->Delta * r->Delta);
  for (int k = 0; k < r->nl; ++k) {
    double* P = psi ? psi + k * L : nullptr;
    double* Q = q ? q + k * L : nullptr;
    const double* PS = ps ? ps + k * L : nullptr;
    for (int i = 0; i < nxp2; ++i) {
      for (int jj : {0, nyp2 - 1}) {
        if (P) P[(size_t)jj * nxp2 + i] = 0.0;
        if (Q) {
          const int ja = jj == 0 ? 1 : nyp2 - 2;
          const bool corner = (i == 0 || i == nxp2 - 1);
          Q[(size_t)jj * nxp2 + i] = (corner || c == 0) ? 0.0 : c * PS[(size_t)ja * nxp2 + i];
        }
      }
    }
    for (int j = 0; j < nyp2; ++j) {
      for (int ii : {0, nxp2 - 1}) {
        if (P) P[(size_t)j * nxp2 + ii] = 0.0;
        if (Q) {
          const int ia = ii == 0 ? 1 : nxp2 - 2;
          const bool corner = (j == 0 || j == nyp2 - 1);
          Q[(size_t)j * nxp2 + ii] = (corner || c == 0) ? 0.0 : c * PS[(size_t)j * nxp2 + ia];
        }
      }
    }
  }
}

int qgw_get(qgw_run* r, double* psi, double* q) {
  if (!r) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  // psi is the inversion of the current q; q alone needs it only for the
  // ghost values of a no-slip or partial-slip wall
  if (psi || (r->p.bc_fac != 0 && r->p.bc_fac != -1)) enqueue_invert(r);
  const size_t nfull = (size_t)r->nl * (r->ny + 2) * (r->nx + 2);
  // one field out through the staging buffer: pack (interior), contiguous copy
  // (the pack kernel writes the caller's array directly where the device
  // can address it)
  auto fetch = [&](bool want_psi, double* host) -> int {
    double* view = (double*)device_view(r, host);
    double* dst = view ? view : r->d_full;
    if (r->precision == QGW_FP64)
      qgw::enqueue_pack_f64(want_psi ? r->a64.psi : r->a64.q, dst, r->nx, r->ny, r->nl, r->pitch, r->stream);
    else
      qgw::enqueue_pack_join(want_psi ? r->a32.psi : r->a32.q, want_psi ? nullptr : r->a32.qlo, dst, r->nx, r->ny,
                             r->nl, r->pitch, r->stream);
    if (!view) CK(cudaMemcpyAsync(host, r->d_full, sizeof(double) * nfull, cudaMemcpyDeviceToHost, r->stream));
    CK(cudaStreamSynchronize(r->stream));
    return QGW_OK;
  };
  int rc;
  if (psi && (rc = fetch(true, psi))) return rc;
  if (q && (rc = fetch(false, q))) return rc;
  CK(cudaGetLastError());
  const double c = 2 * r->p.bc_fac / (r->Delta * r->Delta);
  std::vector<double> psi_tmp;
  const double* ps = psi;
  if (r->p.bc_fac != -1 && q && !psi && c != 0) {
    psi_tmp.resize((size_t)(r->nx + 2) * (r->ny + 2) * r->nl);
    if ((rc = fetch(true, psi_tmp.data()))) return rc;
    ps = psi_tmp.data();
  }
  fill_ghosts(r, psi, q, ps);
  return QGW_OK;
}

int qgw_budget(qgw_run* r, qgw_budget_out* out) {
  if (!r || !out) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  enqueue_invert(r);
  const double scale = r->Delta * r->Delta / (r->p.Lx * r->Ly);
  if (r->precision == QGW_FP64)
    qgw::enqueue_budget_f64(r->a64, r->d_wts, r->d_part, r->budget_blocks, scale, r->d_bout, r->stream);
  else
    qgw::enqueue_budget_f32c(r->a32, r->d_wts, r->d_part, r->budget_blocks, scale, r->d_bout, r->stream);
  double v[4];
  CK(cudaMemcpyAsync(v, r->d_bout, sizeof(v), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  CK(cudaGetLastError());
  out->ke = v[0];
  out->energy = v[1];
  out->enstrophy = v[2];
  out->wind_work = v[3];
  return QGW_OK;
}

// Measurement helper: runs nsteps steps with CUDA events between the four
// kernels of each step on the run's stream and returns the mean duration of
// each kernel in ms (ms4[0..3]: rows forward, columns, rows inverse, RHS).
int qgw_profile_kernels(qgw_run* r, int nsteps, float* ms4) {
  if (!r || !ms4 || nsteps < 1) return QGW_ERR_PARAM;
  if (!r->has_q) return QGW_ERR_STATE;
  std::vector<cudaEvent_t> ev(5 * (size_t)nsteps);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  qgw::enqueue_begin(r->d_state, 0.0, 0.0, r->stream);
  for (int s = 0; s < nsteps; ++s) {
    CK(cudaEventRecord(ev[5 * s], r->stream));
    for (int k = 0; k < 4; ++k) {
      if (r->precision == QGW_FP64) qgw::enqueue_step_kernel_f64(r->a64, k, r->stream);
      else qgw::enqueue_step_kernel_f32c(r->a32, k, r->stream);
      CK(cudaEventRecord(ev[5 * s + k + 1], r->stream));
    }
  }
  if (r->precision == QGW_FP64) qgw::enqueue_flush_f64(r->a64, r->stream);
  else qgw::enqueue_flush_f32c(r->a32, r->stream);
  CK(cudaStreamSynchronize(r->stream));
  for (int k = 0; k < 4; ++k) ms4[k] = 0;
  for (int s = 0; s < nsteps; ++s)
    for (int k = 0; k < 4; ++k) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, ev[5 * s + k], ev[5 * s + k + 1]));
      ms4[k] += ms / nsteps;
    }
  for (auto& e : ev) cudaEventDestroy(e);
  return QGW_OK;
}

}  // extern "C"
