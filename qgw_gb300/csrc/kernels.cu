// kernels.cu -- the single-run step kernels, the small kernels (begin,
// flush, forcing, boundary copies, budget) and their launchers; the device
// side they share with the ensemble kernels is step_device.cuh.
#include "step_device.cuh"

// The FP64 and the FP32c instantiations compile as two translation units
// (in parallel): this file compiled directly is part 1 (the FP64 kernels and
// the precision-free helpers), kernels_f32c.cu includes it as part 2 (the
// FP32c kernels).  The few non-template kernels are static to each unit.
#ifndef QGW_KERNELS_PART
#define QGW_KERNELS_PART 1
#endif

namespace qgw {

// ------------------------------------------------- single-run wrappers
// HL: 0, or the half-length whose transform alone the kernel holds (512:
// the 1024-point rows and columns of the common grid)
template <typename T, bool COMP, bool PER, int HL>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 4 : 3) k_rows_fwd(StepArgs<T> a, int step_mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tot[GMAX * 32];
  body_rows_fwd<T, COMP, PER, HL>(a, step_mode, blockIdx.x, smem_raw + cst_bytes<T>(a.nl), tot, (T*)smem_raw);
}
// CT: columns per tile (closed basin; the periodic kernel takes two complex
// columns whatever CT)
template <typename T, bool COMP, bool PER, int CT, int HL>
__global__ void __launch_bounds__(NT, 3) k_cols(StepArgs<T> a, int step_mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tot[GMAX * 32];
  if (PER) body_cols_per<T, COMP>(a, step_mode, blockIdx.x, blockIdx.y, smem_raw);
  else body_cols<T, COMP, CT, HL>(a, step_mode, blockIdx.x, blockIdx.y, smem_raw, tot);
}
template <typename T> constexpr int CTD = ColsPer<T>::value;
// FP32: four blocks per SM (64 registers; at 1024^2 x 10 the kernel drops
// from 0.109 to 0.101 ms); FP64 keeps three (64 registers spill there)
template <typename T, bool COMP, bool PER, int HL>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 4 : 3) k_rows_inv(StepArgs<T> a, int step_mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tot[GMAX * 32];
  body_rows_inv<T, COMP, PER, HL>(a, step_mode, blockIdx.x, smem_raw + cst_bytes<T>(a.nl), tot, (T*)smem_raw,
                                  gridDim.y > 1 ? (int)blockIdx.y : -1);
}
// The RHS of a step: a persistent grid (a.rhs_grid blocks) over the
// ntx x nty x nl tiles (body_rhs_tiles); the FP64 path launches one block
// per tile (its tiles keep the FP64 pipe busy, and blocks that each load
// one tile overlap one another's loads without a second buffer).
template <typename T, bool COMP, int R, int TY>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 5 : 4) k_rhs(const __grid_constant__ StepArgs<T> a, int ntx,
                                                                    int nty) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long bar[4];
  // TMA destinations are 128-byte aligned (the launch adds 128 bytes)
  unsigned char* base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  if (threadIdx.x == 0 && threadIdx.y == 0)
    for (int b = 0; b < 4; ++b) mbar_init(&bar[b]);
  __syncthreads();
  body_rhs_tiles<T, COMP, R, TY, rhs_nbuf<T>()>(a, ntx, nty, base, a.use_tma ? &a.tm[0] : nullptr, bar);
}

// ------------------------------------------------------- small kernels
static __global__ void k_begin(DevState* st, double t_out, double tend) { begin_state(st, t_out, tend, 0); }

template <typename T, bool COMP>
// (a.qout: also writes the final q, joined to FP64, into the caller's array
// in the reference layout -- the interior; the host fills the ghost ring)
__global__ void __launch_bounds__(NT) k_flush(StepArgs<T> a) {
  DevState* st = a.state;
  const bool pend = st->pending != 0;
  if (!pend && !a.qout) return;
  int s0, s1, s2;
  slabs(st->step_index, s0, s1, s2);
  const double c0 = st->c0, c1 = st->c1, c2 = st->c2;
  const double sqdt = sqrt(st->dt);
  const size_t fs = (size_t)a.nl * a.lstride;
  const T* f0 = a.fab + s0 * fs;
  const T* f1 = a.fab + s1 * fs;
  const T* f2 = a.fab + s2 * fs;
  const size_t n = (size_t)a.nl * a.ny * a.nx;
  const T* r1 = nullptr;
  const T* r2 = nullptr;
  T w1 = T(0), w2 = T(0);
  if (a.nrec > 0) {
    const Forc4D fw = forc4d_at(st->t_prev, a.dt_forc, a.nrec);
    r1 = a.frec + fw.i1 * fs;
    r2 = a.frec + fw.i2 * fs;
    w1 = (T)fw.w1;
    w2 = (T)fw.w2;
  }
  for (size_t w = blockIdx.x * (size_t)NT + threadIdx.x; w < n; w += (size_t)gridDim.x * NT) {
    const size_t row = w / a.nx;
    const int i = (int)(w - row * a.nx);
    const size_t o = row * a.pitch + i;
    // layer 0 also takes the stochastic forcing (src/timestep.h:143-150)
    const T* fo = (a.fr.on && row < (size_t)a.ny) ? a.fr.field + o : nullptr;
    double out;
    if (COMP) {
      float hi = (float)a.q[o], lo = (float)a.qlo[o];
      if (pend) {
        const float d = ab3_increment((float)c0, (float)c1, (float)c2, (float)f0[o], (float)f1[o], (float)f2[o]);
        comp_add(hi, lo, d);
        if (fo) comp_add(hi, lo, (float)*fo * (float)sqdt);
        if (r1) comp_add(hi, lo, (float)forc4d_term<T>(r1, r2, o, w1, w2, (T)st->dt));
        a.q[o] = (T)hi;
        a.qlo[o] = (T)lo;
      }
      out = (double)hi + (double)lo;
    } else {
      T v = a.q[o];
      if (pend) {
        v = ab3_plain<T>(v, (T)c0, (T)c1, (T)c2, f0[o], f1[o], f2[o]);
        if (fo) v = v + *fo * (T)sqdt;
        if (r1) v = v + forc4d_term<T>(r1, r2, o, w1, w2, (T)st->dt);
        a.q[o] = v;
      }
      out = (double)v;
    }
    if (a.qout) {
      const size_t l = row / a.ny, jj = row - l * a.ny;
      a.qout[(l * (a.ny + 2) + jj + 1) * (a.nx + 2) + i + 1] = out;
    }
  }
}

static __global__ void k_end(DevState* st) { st->pending = 0; }

// --------------------------------------------------- stochastic forcing
// F1: new ring amplitudes after each completed step (calc_forc,
// src/forcing.h:170-190): three draws per ring point from the C-library
// sequence in the order the reference consumes them (the logarithm's,
// the cosine's, the phase's), made by one thread chunk by chunk; the
// transcendental functions run on all threads.
constexpr double QGW_PI = 3.14159265358979323846;
constexpr int FORC_CHUNK = 1024;

template <typename T>
__global__ void __launch_bounds__(NT) k_forc_modes(StepArgs<T> a) {
  DevState* st = a.state;
  const ForcArgs<T>& f = a.fr;
  __shared__ uint32_t rv[3 * FORC_CHUNK];
  __shared__ GlibcRand g;
  __shared__ int go;
  const int tid = threadIdx.x;
  if (tid == 0) {
    go = st->forc_step != st->step_index;  // one field per completed step
    if (go) g = *f.rng;
  }
  __syncthreads();
  if (!go) return;
  for (int c0 = 0; c0 < f.nring; c0 += FORC_CHUNK) {
    const int nc = min(FORC_CHUNK, f.nring - c0);
    if (tid == 0)
      for (int k = 0; k < 3 * nc; ++k) rv[k] = glibc_rand_next(&g);
    __syncthreads();
    for (int k = tid; k < nc; k += NT) {
      const int ii = c0 + k;
      const int i = f.ring[2 * ii], j = f.ring[2 * ii + 1];
      const double rl = (double)rv[3 * k], rc = (double)rv[3 * k + 1], rp = (double)rv[3 * k + 2];
      const double nn = sqrt(-2. * log((rl + 1.) / (GLIBC_RAND_MAX + 2.))) * cos(2 * QGW_PI * rc / GLIBC_RAND_MAX);
      const double em = f.env * (f.sigma * nn);
      const double ph = rp / GLIBC_RAND_MAX * 2 * QGW_PI;
      T* d = f.spec + (size_t)j * f.fpitch + 2 * i;
      d[0] = (T)(em * cos(ph));
      d[1] = (T)(em * sin(ph));
    }
    __syncthreads();
  }
  if (tid == 0) {
    *f.rng = g;
    st->forc_step = st->step_index;
  }
}

// F2: backward complex FFT along j of two complex columns i per block
// (the first dimension of the NF x NF c2r, unnormalised); only the columns
// up to the ring's largest i: the others stay zero in both buffers.
template <typename T>
__global__ void __launch_bounds__(NT) k_forc_cols(StepArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const ForcArgs<T>& f = a.fr;
  const int ld = padded_len<T>(f.gy.M);
  T* A = (T*)smem_raw;
  T* B = A + 2 * ld;
  const int c4 = 4 * blockIdx.x;
  for (int j = threadIdx.x; j < f.NF; j += NT) {
    T v[4];
    load_cols<T, 4>(f.spec + (size_t)j * f.fpitch + c4, v);
    C2<T> z0, z1;
    z0.x = v[0]; z0.y = -v[1]; z1.x = v[2]; z1.y = -v[3];
    ((C2<T>*)A)[pc<T>(j)] = z0;
    ((C2<T>*)(A + ld))[pc<T>(j)] = z1;
  }
  __syncthreads();
  T* O = cfft_block<T>(A, B, 2, ld, f.gy, f.ty.tw);
  for (int j = threadIdx.x; j < f.NF; j += NT) {
    const C2<T> z0 = ((const C2<T>*)O)[pc<T>(j)];
    const C2<T> z1 = ((const C2<T>*)(O + ld))[pc<T>(j)];
    T v[4] = {z0.x, -z0.y, z1.x, -z1.y};
    store_cols<T, 4>(f.spec2 + (size_t)j * f.fpitch + c4, v);
  }
}

// F3: c2r along i of row j, written as the forcing of the run's interior
// row j (forc[i+1][j+1] = forc_p[j][i], src/forcing.h:196-200).
template <typename T>
__global__ void __launch_bounds__(NT) k_forc_rows(StepArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const ForcArgs<T>& f = a.fr;
  const int j = blockIdx.x;
  const int ld = padded_len<T>(f.gx.M);
  T* A = (T*)smem_raw;
  T* B = A + ld;
  const T* src = f.spec2 + (size_t)j * f.fpitch;
  for (int i = threadIdx.x; i < f.NF + 2; i += NT) A[pr<T>(i)] = src[i];
  __syncthreads();
  T* O = irfft_block<T>(A, B, 1, ld, f.gx, f.tx);
  T* dst = f.field + (size_t)j * a.pitch;
  for (int i = threadIdx.x; i < a.nx; i += NT) dst[i] = (i & 1) ? -O[pr<T>(i)] : O[pr<T>(i)];
}

template <typename T>
static void launch_forcing(const StepArgs<T>& a, cudaStream_t s) {
  const ForcArgs<T>& f = a.fr;
  if (!f.on) return;
  k_forc_modes<T><<<1, NT, 0, s>>>(a);
  k_forc_cols<T><<<f.col_blocks, NT, (size_t)4 * padded_len<T>(f.gy.M) * sizeof(T), s>>>(a);
  k_forc_rows<T><<<a.ny, NT, (size_t)2 * padded_len<T>(f.gx.M) * sizeof(T), s>>>(a);
}

// Boundary copies: the reference layout (nl, ny+2, nx+2) in one contiguous
// device buffer <-> the interior-only run layout; a host array then crosses
// the link in one contiguous copy instead of one row per DMA segment.
template <typename T, bool SPLIT>
__global__ void __launch_bounds__(256) k_unpack(const double* __restrict__ full, T* __restrict__ dst,
                                                T* __restrict__ lo, int nx, int ny, int nl, int pitch) {
  const size_t n = (size_t)nl * ny * nx;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x) {
    const size_t row = w / nx;
    const int i = (int)(w - row * nx);
    const int l = (int)(row / ny), j = (int)(row - (size_t)l * ny);
    const double v = full[((size_t)l * (ny + 2) + (j + 1)) * (nx + 2) + (i + 1)];
    const size_t o = row * pitch + i;
    if (SPLIT) {
      const float h = (float)v;
      dst[o] = (T)h;
      lo[o] = (T)(float)(v - (double)h);
    } else {
      dst[o] = (T)v;
    }
  }
}
template <typename T>
__global__ void __launch_bounds__(256) k_pack(const T* __restrict__ src, const T* __restrict__ lo,
                                              double* __restrict__ full, int nx, int ny, int nl, int pitch) {
  const size_t n = (size_t)nl * ny * nx;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x) {
    const size_t row = w / nx;
    const int i = (int)(w - row * nx);
    const int l = (int)(row / ny), j = (int)(row - (size_t)l * ny);
    const size_t o = row * pitch + i;
    full[((size_t)l * (ny + 2) + (j + 1)) * (nx + 2) + (i + 1)] = (double)src[o] + (lo ? (double)lo[o] : 0.0);
  }
}

// FP32c <-> FP64 conversions for the boundary copies
static __global__ void k_split_f64(const double* src, float* hi, float* lo, size_t n) {
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x) {
    const double x = src[w];
    const float h = (float)x;
    hi[w] = h;
    lo[w] = (float)(x - (double)h);
  }
}
static __global__ void k_join_f64(const float* hi, const float* lo, double* dst, size_t n) {
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < n; w += (size_t)gridDim.x * blockDim.x)
    dst[w] = (double)hi[w] + (lo ? (double)lo[w] : 0.0);
}

// FP64 diagnostics: per-block partial sums, then one block adds them up in a
// fixed order (bit-reproducible).
template <typename T>
__global__ void __launch_bounds__(NT) k_budget_partial(StepArgs<T> a, const double* wts, double* part) {
  __shared__ double red[4][NT];
  double ke = 0, en = 0, ens = 0, ww = 0;
  const size_t n = (size_t)a.nl * a.ny * a.nx;
  for (size_t w = blockIdx.x * (size_t)NT + threadIdx.x; w < n; w += (size_t)gridDim.x * NT) {
    const size_t row = w / a.nx;
    const int i = (int)(w - row * a.nx);
    const int l = (int)(row / a.ny);
    const int j = (int)(row - (size_t)l * a.ny);
    const size_t o = row * a.pitch + i;
    const double p = (double)a.psi[o];
    const double qv = (double)a.q[o] + (a.qlo ? (double)a.qlo[o] : 0.0);
    // closed basin: psi = 0 on the walls; periodic: the opposite side
    const double pe = (i + 1 < a.nx) ? (double)a.psi[o + 1] : (a.periodic ? (double)a.psi[o + 1 - a.nx] : 0.0);
    const double pn = (j + 1 < a.ny) ? (double)a.psi[o + a.pitch]
                                     : (a.periodic ? (double)a.psi[o - (size_t)(a.ny - 1) * a.pitch] : 0.0);
    const double u = (pe - p) / a.Delta, v = (pn - p) / a.Delta;
    const double wl = wts[l];
    ke += wl * 0.5 * (u * u + v * v);
    en -= wl * p * qv;
    ens += wl * qv * qv;
    if (l == 0 && a.wind) ww -= wl * p * (double)a.wind[j];
  }
  red[0][threadIdx.x] = ke; red[1][threadIdx.x] = en; red[2][threadIdx.x] = ens; red[3][threadIdx.x] = ww;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 4) part[blockIdx.x * 4 + threadIdx.x] = red[threadIdx.x][0];
}

static __global__ void k_budget_final(const double* part, int nblk, double scale, double* out) {
  if (threadIdx.x < 4) {
    double s = 0;
    for (int b = 0; b < nblk; ++b) s += part[b * 4 + threadIdx.x];
    out[threadIdx.x] = s * scale;
  }
}

// ------------------------------------------------------------- launchers
// The dynamic shared-memory limit is a process-wide attribute of each kernel,
// shared by every run in the process; it is set to the device's opt-in
// maximum (never lowered) so that runs of different sizes can coexist.
template <typename T, bool COMP>
static cudaError_t set_attrs(const StepArgs<T>& a) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const size_t static_tot = sizeof(T) * GMAX * 32 + 64;
  if (smem_rows<T, COMP>(a) + static_tot > (size_t)optin || smem_cols<T, COMP>(a) + static_tot > (size_t)optin ||
      smem_rows_inv<T, COMP>(a) + static_tot > (size_t)optin || rhs_halo(a) > RHS_RMAX ||
      smem_rhs<T>(a) + 1024 > (size_t)optin || smem_rhs_tiles<T>(a) + 1024 > (size_t)optin)
    return cudaErrorInvalidValue;
  const int lim = optin - (int)static_tot;
  const void* transforms[] = {
      (const void*)k_rows_fwd<T, COMP, false, 0>,         (const void*)k_rows_fwd<T, COMP, false, 512>,
      (const void*)k_rows_inv<T, COMP, false, 0>,         (const void*)k_rows_inv<T, COMP, false, 512>,
      (const void*)k_cols<T, COMP, false, CTD<T>, 0>,     (const void*)k_cols<T, COMP, false, CTD<T>, 512>,
      (const void*)k_cols<T, COMP, false, CTD<T> / 2, 0>, (const void*)k_cols<T, COMP, false, CTD<T> / 2, 512>,
      (const void*)k_rows_fwd<T, COMP, false, -1>,        (const void*)k_rows_inv<T, COMP, false, -1>,
      (const void*)k_cols<T, COMP, false, CTD<T> / 2, -1>, (const void*)k_cols<T, COMP, false, 1, -1>,
      (const void*)k_rows_fwd<T, COMP, true, 0>,          (const void*)k_rows_inv<T, COMP, true, 0>,
      (const void*)k_cols<T, COMP, true, CTD<T>, 0>};
  for (const void* f : transforms)
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
  if ((e = cudaFuncSetAttribute(k_forc_cols<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
  if ((e = cudaFuncSetAttribute(k_forc_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim))) return e;
  const int rl = optin - 1024;
  const void* rhs_kernels[] = {(const void*)k_rhs<T, COMP, 1, 16>, (const void*)k_rhs<T, COMP, 2, 16>,
                               (const void*)k_rhs<T, COMP, 3, 16>, (const void*)k_rhs<T, COMP, 4, 16>,
                               (const void*)k_rhs<T, COMP, 1, 32>, (const void*)k_rhs<T, COMP, 2, 32>,
                               (const void*)k_rhs<T, COMP, 3, 32>, (const void*)k_rhs<T, COMP, 4, 32>};
  for (const void* f : rhs_kernels)
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, rl)) != cudaSuccess) return e;
  return cudaSuccess;
}

template <typename T, bool COMP>
static void launch_k1(const StepArgs<T>& a, int step_mode, cudaStream_t s) {
  const size_t sm = smem_rows<T, COMP>(a);
  if (a.periodic) k_rows_fwd<T, COMP, true, 0><<<dim3(a.ny), NT, sm, s>>>(a, step_mode);
  else if (a.gx.blue) k_rows_fwd<T, COMP, false, -1><<<dim3(a.ny), NT, sm, s>>>(a, step_mode);
  else if (a.gx.H == 512) k_rows_fwd<T, COMP, false, 512><<<dim3(a.ny), NT, sm, s>>>(a, step_mode);
  else k_rows_fwd<T, COMP, false, 0><<<dim3(a.ny), NT, sm, s>>>(a, step_mode);
}
template <typename T, bool COMP>
static void launch_k2(const StepArgs<T>& a, int step_mode, cudaStream_t s) {
  const dim3 grid(col_tiles(a), a.nl);
  const size_t sm = smem_cols<T, COMP>(a);
  const bool wide = col_width(a) == CTD<T>, h512 = a.gy.H == 512 && !a.gy.blue;
  if (a.periodic) k_cols<T, COMP, true, CTD<T>, 0><<<grid, NT, sm, s>>>(a, step_mode);
  else if (a.gy.blue && col_width(a) == 1) k_cols<T, COMP, false, 1, -1><<<grid, NT, sm, s>>>(a, step_mode);
  else if (a.gy.blue) k_cols<T, COMP, false, CTD<T> / 2, -1><<<grid, NT, sm, s>>>(a, step_mode);
  else if (wide && h512) k_cols<T, COMP, false, CTD<T>, 512><<<grid, NT, sm, s>>>(a, step_mode);
  else if (wide) k_cols<T, COMP, false, CTD<T>, 0><<<grid, NT, sm, s>>>(a, step_mode);
  else if (h512) k_cols<T, COMP, false, CTD<T> / 2, 512><<<grid, NT, sm, s>>>(a, step_mode);
  else k_cols<T, COMP, false, CTD<T> / 2, 0><<<grid, NT, sm, s>>>(a, step_mode);
}
template <typename T, bool COMP>
static void launch_k3(const StepArgs<T>& a, int step_mode, cudaStream_t s) {
  const size_t sm = smem_rows_inv<T, COMP>(a);
  // rows x layer groups: a row's groups read the same spectral rows, so
  // splitting them over blocks adds no traffic and evens out the SMs' loads
  const dim3 grid(a.ny, a.inv_split ? (a.nl + a.G3 - 1) / a.G3 : 1);
  if (a.periodic) k_rows_inv<T, COMP, true, 0><<<grid, NT, sm, s>>>(a, step_mode);
  else if (a.gx.blue) k_rows_inv<T, COMP, false, -1><<<grid, NT, sm, s>>>(a, step_mode);
  else if (a.gx.H == 512) k_rows_inv<T, COMP, false, 512><<<grid, NT, sm, s>>>(a, step_mode);
  else k_rows_inv<T, COMP, false, 0><<<grid, NT, sm, s>>>(a, step_mode);
}
// tiles of the RHS kernel along x and y
template <typename T> static int rhs_ntx(const StepArgs<T>& a) { return (a.nx + TX - 1) / TX; }
template <typename T> static int rhs_nty(const StepArgs<T>& a) { return (a.ny + rhs_ty(a) - 1) / rhs_ty(a); }

template <typename T, bool COMP>
static void launch_rhs(const StepArgs<T>& a, cudaStream_t s) {
  const int ntx = rhs_ntx(a), nty = rhs_nty(a), ntiles = ntx * nty * a.nl;
  const int grid = (a.rhs_grid > 0 && a.rhs_grid < ntiles) ? a.rhs_grid : ntiles;
  const dim3 blk(32, 8);
  const size_t sm = smem_rhs_tiles(a);
  const bool t32 = rhs_ty(a) == 32;
  switch (rhs_halo(a)) {
    case 1:
      if (t32) k_rhs<T, COMP, 1, 32><<<grid, blk, sm, s>>>(a, ntx, nty);
      else k_rhs<T, COMP, 1, 16><<<grid, blk, sm, s>>>(a, ntx, nty);
      break;
    case 2:
      if (t32) k_rhs<T, COMP, 2, 32><<<grid, blk, sm, s>>>(a, ntx, nty);
      else k_rhs<T, COMP, 2, 16><<<grid, blk, sm, s>>>(a, ntx, nty);
      break;
    case 3:
      if (t32) k_rhs<T, COMP, 3, 32><<<grid, blk, sm, s>>>(a, ntx, nty);
      else k_rhs<T, COMP, 3, 16><<<grid, blk, sm, s>>>(a, ntx, nty);
      break;
    default:
      if (t32) k_rhs<T, COMP, 4, 32><<<grid, blk, sm, s>>>(a, ntx, nty);
      else k_rhs<T, COMP, 4, 16><<<grid, blk, sm, s>>>(a, ntx, nty);
      break;
  }
}

// Persistent grid of the RHS kernel: as many blocks as stay resident on the
// device at once (the occupancy of the run's halo and shared memory).
template <typename T, bool COMP>
static int rhs_grid(const StepArgs<T>& a) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const size_t sm = smem_rhs_tiles(a);
  const int h = rhs_halo(a);
  const void* f = rhs_ty(a) == 32 ? (h == 1 ? (const void*)k_rhs<T, COMP, 1, 32> : h == 2 ? (const void*)k_rhs<T, COMP, 2, 32>
                                     : h == 3 ? (const void*)k_rhs<T, COMP, 3, 32> : (const void*)k_rhs<T, COMP, 4, 32>)
                                  : (h == 1 ? (const void*)k_rhs<T, COMP, 1, 16> : h == 2 ? (const void*)k_rhs<T, COMP, 2, 16>
                                     : h == 3 ? (const void*)k_rhs<T, COMP, 3, 16> : (const void*)k_rhs<T, COMP, 4, 16>);
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, NT, sm);
  return (e == cudaSuccess && per > 0) ? per * sms : 0;
}

template <typename T, bool COMP>
static void launch_invert(const StepArgs<T>& a, int step_mode, cudaStream_t s) {
  launch_k1<T, COMP>(a, step_mode, s);
  launch_k2<T, COMP>(a, step_mode, s);
  launch_k3<T, COMP>(a, step_mode, s);
}

template <typename T, bool COMP>
static void launch_flush(const StepArgs<T>& a, cudaStream_t s) {
  const size_t n = (size_t)a.nl * a.ny * a.nx;
  int blocks = (int)((n + NT - 1) / NT);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_flush<T, COMP><<<blocks, NT, 0, s>>>(a);
  k_end<<<1, 1, 0, s>>>(a.state);
}

template <typename T, bool COMP>
static void launch_one(const StepArgs<T>& a, int which, cudaStream_t s) {
  if (which == 0) launch_k1<T, COMP>(a, 1, s);
  if (which == 1) launch_k2<T, COMP>(a, 1, s);
  if (which == 2) launch_k3<T, COMP>(a, 1, s);
  if (which == 3) launch_rhs<T, COMP>(a, s);
}

// ---- entry points used by api.cu (see kernels.h)
template <typename T>
static void budget_impl(const StepArgs<T>& a, const double* wts, double* part, int nblk, double scale, double* out,
                        cudaStream_t s) {
  k_budget_partial<T><<<nblk, NT, 0, s>>>(a, wts, part);
  k_budget_final<<<1, 32, 0, s>>>(part, nblk, scale, out);
}

#if QGW_KERNELS_PART == 1
void enqueue_begin(DevState* st, double t_out, double tend, cudaStream_t s) { k_begin<<<1, 1, 0, s>>>(st, t_out, tend); }

void enqueue_unpack_split(const double* full, float* hi, float* lo, int nx, int ny, int nl, int pitch,
                          cudaStream_t s) {
  k_unpack<float, true><<<152 * 8, 256, 0, s>>>(full, hi, lo, nx, ny, nl, pitch);
}

void enqueue_pack_join(const float* hi, const float* lo, double* full, int nx, int ny, int nl, int pitch,
                       cudaStream_t s) {
  k_pack<float><<<152 * 8, 256, 0, s>>>(hi, lo, full, nx, ny, nl, pitch);
}

int rhs_tile_x() { return TX; }

int rhs_box_width() { return TW; }

cudaError_t prepare_f64(const StepArgs<double>& a) { return set_attrs<double, false>(a); }

int rhs_grid_f64(const StepArgs<double>&) { return 0; }  // one block per tile

void enqueue_step_f64(const StepArgs<double>& a, cudaStream_t s) {
  launch_invert<double, false>(a, 1, s);
  launch_rhs<double, false>(a, s);
  launch_forcing<double>(a, s);
}

void enqueue_forcing_f64(const StepArgs<double>& a, cudaStream_t s) { launch_forcing<double>(a, s); }

void enqueue_invert_f64(const StepArgs<double>& a, cudaStream_t s) { launch_invert<double, false>(a, 0, s); }

void enqueue_flush_f64(const StepArgs<double>& a, cudaStream_t s) { launch_flush<double, false>(a, s); }

void enqueue_step_kernel_f64(const StepArgs<double>& a, int which, cudaStream_t s) { launch_one<double, false>(a, which, s); }

void enqueue_unpack_f64(const double* full, double* q, int nx, int ny, int nl, int pitch, cudaStream_t s) {
  k_unpack<double, false><<<152 * 8, 256, 0, s>>>(full, q, nullptr, nx, ny, nl, pitch);
}

void enqueue_pack_f64(const double* src, double* full, int nx, int ny, int nl, int pitch, cudaStream_t s) {
  k_pack<double><<<152 * 8, 256, 0, s>>>(src, nullptr, full, nx, ny, nl, pitch);
}

void enqueue_split_f64(const double* src, float* hi, float* lo, size_t n, cudaStream_t s) {
  k_split_f64<<<1024, 256, 0, s>>>(src, hi, lo, n);
}

void enqueue_join_f64(const float* hi, const float* lo, double* dst, size_t n, cudaStream_t s) {
  k_join_f64<<<1024, 256, 0, s>>>(hi, lo, dst, n);
}

void enqueue_budget_f64(const StepArgs<double>& a, const double* w, double* part, int nblk, double scale, double* out,
                        cudaStream_t s) { budget_impl<double>(a, w, part, nblk, scale, out, s); }

int cols_per_tile_f64() { return ColsPer<double>::value; }

int rhs_tile_y_f64(const StepArgs<double>& a) { return rhs_ty(a); }

size_t smem_bytes_rows_f64(const StepArgs<double>& a) { return smem_rows<double, false>(a); }

size_t smem_bytes_cols_f64(const StepArgs<double>& a) { return smem_cols<double, false>(a); }

size_t smem_bytes_rhs_f64(const StepArgs<double>& a) { return smem_rhs_tiles<double>(a); }
#else
cudaError_t prepare_f32c(const StepArgs<float>& a) { return set_attrs<float, true>(a); }

int rhs_grid_f32c(const StepArgs<float>& a) { return rhs_grid<float, true>(a); }

void enqueue_step_f32c(const StepArgs<float>& a, cudaStream_t s) {
  launch_invert<float, true>(a, 1, s);
  launch_rhs<float, true>(a, s);
  launch_forcing<float>(a, s);
}

void enqueue_forcing_f32c(const StepArgs<float>& a, cudaStream_t s) { launch_forcing<float>(a, s); }

void enqueue_invert_f32c(const StepArgs<float>& a, cudaStream_t s) { launch_invert<float, true>(a, 0, s); }

void enqueue_flush_f32c(const StepArgs<float>& a, cudaStream_t s) { launch_flush<float, true>(a, s); }

void enqueue_step_kernel_f32c(const StepArgs<float>& a, int which, cudaStream_t s) { launch_one<float, true>(a, which, s); }

void enqueue_budget_f32c(const StepArgs<float>& a, const double* w, double* part, int nblk, double scale, double* out,
                         cudaStream_t s) { budget_impl<float>(a, w, part, nblk, scale, out, s); }

int cols_per_tile_f32c() { return ColsPer<float>::value; }

int rhs_tile_y_f32c(const StepArgs<float>& a) { return rhs_ty(a); }

size_t smem_bytes_rows_f32c(const StepArgs<float>& a) { return smem_rows<float, true>(a); }

size_t smem_bytes_cols_f32c(const StepArgs<float>& a) { return smem_cols<float, true>(a); }

size_t smem_bytes_rhs_f32c(const StepArgs<float>& a) { return smem_rhs_tiles<float>(a); }
#endif  // QGW_KERNELS_PART

}  // namespace qgw
