// noalloc.cu -- qgw_invert_pv_noalloc: the PV inversion (psi from q, the
// reference's invert_pv) for callers that cannot allocate device memory.
//
// Who cannot allocate: a host model that owns every device buffer through
// its own memory manager (a coupled ocean/climate driver, an OpenACC or
// Fortran code whose arrays already live on the GPU), or a time-critical
// loop that is not allowed to call cudaMalloc/cudaFree because those calls
// synchronise the device and may fail under memory pressure.  Such a caller
// hands in its own device arrays for q and psi and wants nothing else
// allocated on its behalf.
//
// The inversion needs scratch memory beyond q and psi: the per-mode
// spectral field, the Helmholtz divisors, the DST tables and the mode
// matrices.  Here they live in one file-scope __device__ array
// (g_noalloc_scratch, 32 MiB + 0.1 MiB) that every GPU which loads the
// library holds until the process exits.  No call here allocates device or
// host memory: tables are built in file-scope host arrays and copied in
// with cudaMemcpyAsync; the Helmholtz divisors are computed on the device.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/qgw_gpu.h"
#include "dst_core.h"
#include "host.h"
#include "kernels.h"
#include "qgw_device.cuh"

namespace {

constexpr size_t kFieldMax = (size_t)1 << 21;  // doubles: nl*(NX+1)*(NY+1) limit
constexpr int kMMax = 1024;                     // NX, NY limit (DST length + 1)
constexpr int kNlMax = 32;  // layers the shared scratch array holds
constexpr int kDevMax = 16;
// DST tables of one dimension: tw (H), pre (H+1), spl (H/2+1), twp (< H)
// complex values
constexpr size_t kTab = 2 * (2 * ((size_t)kMMax / 2) + ((size_t)kMMax / 2 + 1) + ((size_t)kMMax / 4 + 1));
constexpr size_t kStateD = (sizeof(qgw::DevState) + 7) / 8;

// offsets (in doubles) inside the scratch array
constexpr size_t oSpec = 0;
constexpr size_t oHinv = oSpec + kFieldMax;
constexpr size_t oTx = oHinv + kFieldMax;
constexpr size_t oTy = oTx + kTab;
constexpr size_t oCl = oTy + kTab;
constexpr size_t oCm = oCl + (size_t)kNlMax * kNlMax;
constexpr size_t oIrd = oCm + (size_t)kNlMax * kNlMax;
constexpr size_t oLsq = oIrd + kNlMax;
constexpr size_t oKsq = oLsq + kMMax;
constexpr size_t oState = oKsq + kMMax;
constexpr size_t kTotal = oState + kStateD;

// host staging of the small tables (file scope: no heap use per call)
double h_tab[oState - oTx];
double h_key[kDevMax][3 * kNlMax * kNlMax + 16];  // set-up held by each device
bool h_key_valid[kDevMax];
double* d_base[kDevMax];

}  // namespace

// The scratch array.  Host code must not use this symbol as an address: its
// device address is obtained per device with cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_scratch[kTotal];

namespace {

// 1 / (fact * norm) with fact = -(sq(L[i]) + sq(K[j]) + iRd2[m])
// (src/elliptic.h:122-127, normalisation :134-138), on the caller's pitched layout
__global__ void k_noalloc_hinv(double* hinv, const double* Lsq, const double* Ksq, const double* ird, int nx,
                               int ny, int nl, int pitch, long long lstride, double norm) {
  const size_t n = (size_t)nl * ny * nx;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(w % nx);
    const size_t row = w / nx;
    const int j = (int)(row % ny);
    const int m = (int)(row / ny);
    const double fact = -(Lsq[k] + Ksq[j] + ird[m]);
    hinv[(size_t)m * lstride + (size_t)j * pitch + k] = 1.0 / (fact * norm);
  }
}

// Ghost rings as adjust_bc leaves them at the end of invert_pv
// (src/elliptic.h:152-153, src/domain.h:308-348): psi = 0 on the ring,
// q = 2 bc_fac / Delta^2 * psi at the adjacent interior point, corners 0.
__global__ void k_noalloc_ghosts(double* q, double* psi, int nx, int ny, int nl, double c) {
  const int nxp2 = nx + 2, nyp2 = ny + 2;
  const int per = 2 * nxp2 + 2 * ny;
  const size_t n = (size_t)nl * per;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(w / per);
    int e = (int)(w % per);
    int i, j, ia, ja;
    if (e < nxp2) { i = e; j = 0; ia = i; ja = 1; }
    else if ((e -= nxp2) < nxp2) { i = e; j = nyp2 - 1; ia = i; ja = nyp2 - 2; }
    else if ((e -= nxp2) < ny) { i = 0; j = e + 1; ia = 1; ja = j; }
    else { e -= ny; i = nxp2 - 1; j = e + 1; ia = nxp2 - 2; ja = j; }
    const size_t base = (size_t)k * nxp2 * nyp2;
    psi[base + (size_t)j * nxp2 + i] = 0.0;
    const bool corner = (i == 0 || i == nxp2 - 1) && (j == 0 || j == nyp2 - 1);
    q[base + (size_t)j * nxp2 + i] = corner ? 0.0 : c * psi[base + (size_t)ja * nxp2 + ia];
  }
}

double sinpi_r(long m, long N) {
  long r = m % (2 * N);
  if (r < 0) r += 2 * N;
  double sg = 1.0;
  if (r >= N) { r -= N; sg = -1.0; }
  if (2 * r > N) r = N - r;
  return sg * std::sin(M_PI * (double)r / (double)N);
}

// the DST tables of dst_core.h for length M into dst (tw | pre | spl)
void fill_tables(int M, double* dst) {
  const int H = M / 2;
  double* tw = dst;
  double* pre = tw + 2 * H;
  double* spl = pre + 2 * (H + 1);
  for (int m = 0; m < H; ++m) {
    tw[2 * m] = sinpi_r(4L * m + H, 2L * H);
    tw[2 * m + 1] = -sinpi_r(2L * m, H);
  }
  for (int j = 0; j <= H; ++j) {
    const double s = sinpi_r(j, M);
    pre[2 * j] = s + 0.5;
    pre[2 * j + 1] = s - 0.5;
  }
  for (int k = 0; k <= H / 2; ++k) {
    spl[2 * k] = sinpi_r(4L * k + M, 2L * M);
    spl[2 * k + 1] = sinpi_r(2L * k, M);
  }
  qgw::fill_pass_twiddles(qgw::make_geom(M), tw, spl + 2 * (H / 2 + 1));
}

// a grid size of a closed basin the transforms take (the run path's rule:
// NX even, NX/2 a product of 2, 3, 5 and 7), up to the scratch tables' limit
bool length_ok(int v) { return v >= 4 && v <= kMMax && qgw::transform_length_ok(v); }

}  // namespace

extern "C" int qgw_invert_pv_noalloc(const qgw_params* p, const double* cl2m, const double* cm2l,
                                     const double* iRd2, double* q_dev, double* psi_dev, void* stream) {
  if (!p || !cl2m || !cm2l || !iRd2 || !q_dev || !psi_dev) return QGW_ERR_PARAM;
  if (p->bc_fac < 0) return QGW_ERR_UNSUPPORTED;  // closed basins only
  if (!length_ok(p->NX) || !length_ok(p->NY)) return QGW_ERR_UNSUPPORTED;
  if (p->nl < 1 || p->nl > kNlMax) return QGW_ERR_UNSUPPORTED;
  const int nx = p->NX - 1, ny = p->NY - 1, nl = p->nl;
  const int pitch = nx + 2;
  const long long lstride = (long long)(ny + 2) * (nx + 2);
  if ((size_t)nl * (size_t)lstride > kFieldMax) return QGW_ERR_UNSUPPORTED;
  // A launch error the caller left pending could not be told apart from one
  // of the launches below: refuse, and leave it for the caller to read.
  if (cudaPeekAtLastError() != cudaSuccess) return QGW_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevMax) return QGW_ERR_CUDA;
  // once per device, with that device current: the device address of the
  // scratch array and the kernels' shared-memory limit
  if (!d_base[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return QGW_ERR_CUDA;
    qgw::StepArgs<double> probe{};
    probe.nl = 1;
    probe.G1 = 1;
    probe.G3 = 1;
    probe.CT = 1;
    probe.gx.M = probe.gy.M = 4;
    if (qgw::prepare_f64(probe) != cudaSuccess) return QGW_ERR_CUDA;
    d_base[dev] = (double*)ptr;
  }
  double* base = d_base[dev];
  // the caller's modes and sizes identify the set-up held by the scratch
  double key[3 * kNlMax * kNlMax + 16];
  double* kcl = key;
  double* kcm = kcl + nl * nl;
  double* kir = kcm + nl * nl;
  std::memcpy(kcl, cl2m, sizeof(double) * nl * nl);
  std::memcpy(kcm, cm2l, sizeof(double) * nl * nl);
  std::memcpy(kir, iRd2, sizeof(double) * nl);
  double* kp = kir + nl;
  kp[0] = p->NX; kp[1] = p->NY; kp[2] = nl; kp[3] = p->Lx;
  const size_t klen = (size_t)(kp + 4 - key);
  const bool same = h_key_valid[dev] && std::memcmp(h_key[dev], key, sizeof(double) * klen) == 0;
  const double norm = 4.0 * (nx + 1) * (ny + 1);
  if (!same) {
    // the scratch no longer holds a complete set-up until this one is in
    h_key_valid[dev] = false;
    // small tables: DST (x, y), modes, wavenumbers
    std::memset(h_tab, 0, sizeof(h_tab));
    fill_tables(nx + 1, h_tab + (oTx - oTx));
    fill_tables(ny + 1, h_tab + (oTy - oTx));
    std::memcpy(h_tab + (oCl - oTx), kcl, sizeof(double) * nl * nl);
    std::memcpy(h_tab + (oCm - oTx), kcm, sizeof(double) * nl * nl);
    std::memcpy(h_tab + (oIrd - oTx), kir, sizeof(double) * nl);
    for (int k = 0; k < nx; ++k) { const double L = M_PI * (k + 1) / p->Lx; h_tab[oLsq - oTx + k] = L * L; }
    for (int j = 0; j < ny; ++j) { const double K = M_PI * (j + 1) / p->Lx; h_tab[oKsq - oTx + j] = K * K; }
    if (cudaMemcpyAsync(base + oTx, h_tab, sizeof(double) * (oState - oTx), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return QGW_ERR_CUDA;
    k_noalloc_hinv<<<304, 256, 0, s>>>(base + oHinv + pitch + 1, base + oLsq, base + oKsq, base + oIrd, nx, ny, nl,
                                       pitch, lstride, norm);
    // the set-up is marked held only once its divisor launch was accepted
    if (cudaGetLastError() != cudaSuccess) return QGW_ERR_CUDA;
    std::memcpy(h_key[dev], key, sizeof(double) * klen);
    h_key_valid[dev] = true;
  }
  // device scalars start at zero for every call (nothing pending)
  if (cudaMemsetAsync(base + oState, 0, sizeof(qgw::DevState), s) != cudaSuccess) return QGW_ERR_CUDA;
  qgw::StepArgs<double> a{};
  a.nx = nx;
  a.ny = ny;
  a.nl = nl;
  a.pitch = pitch;
  a.lstride = lstride;
  a.gx = qgw::make_geom(nx + 1);
  a.gy = qgw::make_geom(ny + 1);
  const int Hx = (nx + 1) / 2, Hy = (ny + 1) / 2;
  a.tx.tw = (const qgw::C2<double>*)(base + oTx);
  a.tx.pre = (const qgw::C2<double>*)(base + oTx + 2 * Hx);
  a.tx.spl = (const qgw::C2<double>*)(base + oTx + 2 * Hx + 2 * (Hx + 1));
  a.tx.twp = (const qgw::C2<double>*)(base + oTx + 2 * Hx + 2 * (Hx + 1) + 2 * (Hx / 2 + 1));
  a.ty.tw = (const qgw::C2<double>*)(base + oTy);
  a.ty.pre = (const qgw::C2<double>*)(base + oTy + 2 * Hy);
  a.ty.spl = (const qgw::C2<double>*)(base + oTy + 2 * Hy + 2 * (Hy + 1));
  a.ty.twp = (const qgw::C2<double>*)(base + oTy + 2 * Hy + 2 * (Hy + 1) + 2 * (Hy / 2 + 1));
  a.cl2m = base + oCl;
  a.cm2l = base + oCm;
  a.iRd2 = base + oIrd;
  a.q = q_dev + pitch + 1;
  a.psi = psi_dev + pitch + 1;
  a.spec = base + oSpec + pitch + 1;
  a.fab = a.spec;
  a.hinv = base + oHinv + pitch + 1;
  a.Lsq = base + oLsq;
  a.Ksq = base + oKsq;
  a.state = (qgw::DevState*)(base + oState);
  a.Delta = p->Lx / p->NX;
  a.norm = norm;
  // same grouping rule as the library's runs (96 KiB of work buffers)
  const size_t budget = 96 * 1024;
  int g = (int)(budget / (2 * (size_t)qgw::padded_len<double>(nx + 1) * sizeof(double)));
  g = g < 1 ? 1 : (g > 16 ? 16 : g);
  const int ngroups = (nl + g - 1) / g;
  a.G1 = (nl + ngroups - 1) / ngroups;
  a.G3 = a.G1;
  int ct = (int)(budget / (2 * (size_t)(ny + 1) * sizeof(double)));
  a.CT = ct < 1 ? 1 : (ct > 16 ? 16 : ct);
  qgw::enqueue_invert_f64(a, s);
  const double c = 2 * p->bc_fac / (a.Delta * a.Delta);
  k_noalloc_ghosts<<<64, 256, 0, s>>>(q_dev, psi_dev, nx, ny, nl, c);
  return cudaGetLastError() == cudaSuccess ? QGW_OK : QGW_ERR_CUDA;
}
