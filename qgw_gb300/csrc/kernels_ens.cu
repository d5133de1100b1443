// kernels_ens.cu -- the ensemble step kernels: one persistent launch per
// stage over all members of a batch, and their launchers; the device side
// they share with the single-run kernels is step_device.cuh.
#include "step_device.cuh"

// The FP64 and the FP32c instantiations compile as two translation units:
// this file compiled directly is part 1 (FP64 and the precision-free
// helpers), kernels_ens_f32c.cu includes it as part 2 (FP32c).
#ifndef QGW_ENS_PART
#define QGW_ENS_PART 1
#endif

namespace qgw {

// default columns per K2 tile (the alternative is half as many)
template <typename T> constexpr int CTE = ColsPer<T>::value;

// --------------------------------------------------- ensemble wrappers
// Persistent launches over all members of an ensemble: work item w of a
// stage belongs to member mi with start[mi] <= w < start[mi+1]; each block
// copies that member's arguments into shared memory and runs the same body
// as a single run would.  Members are independent (own fields, own device
// scalars, own CFL counter), so a member's result does not depend on which
// other members share the launch.
template <typename T>
__device__ __forceinline__ int ens_item(const EnsArgs<T>& e, const int* start, int item, StepArgs<T>* sa,
                                        int* cur) {
  __shared__ int s_mi, s_start;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  if (tid == 0) {
    // a block's items increase, so its member index never decreases: scan
    // forward from the member it holds (binary search for the first item)
    int lo;
    if (*cur >= 0) {
      lo = *cur;
      while (lo + 1 < e.n && start[lo + 1] <= item) ++lo;
    } else {
      lo = 0;
      int hi = e.n - 1;
      while (lo < hi) {  // last member whose start <= item
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= item) lo = mid;
        else hi = mid - 1;
      }
    }
    s_mi = lo;
    s_start = start[lo];
  }
  __syncthreads();
  const int mi = s_mi;
  if (mi != *cur) {
    // the block moves to another member: copy its arguments (block-uniform)
    const int* srcw = reinterpret_cast<const int*>(e.members + mi);
    int* dstw = reinterpret_cast<int*>(sa);
    for (int w = tid; w < (int)(sizeof(StepArgs<T>) / 4); w += blockDim.x * blockDim.y) dstw[w] = srcw[w];
    __syncthreads();
    if (tid == 0) *cur = mi;
  }
  return item - s_start;
}

// the member whose arguments a block holds: none yet
__device__ __forceinline__ void ens_init_cur(int* cur) {
  if (threadIdx.x == 0 && threadIdx.y == 0) *cur = -1;
  __syncthreads();
}

template <typename T, bool COMP, bool PER>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 3 : 2) k_rows_fwd_ens(EnsArgs<T> e, int step_mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tot[GMAX * 32];
  __shared__ StepArgs<T> sa;
  __shared__ int cur;
  ens_init_cur(&cur);
  for (int item = blockIdx.x; item < e.total[0]; item += gridDim.x) {
    const int local = ens_item(e, e.start_rows, item, &sa, &cur);
    body_rows_fwd<T, COMP, PER>(sa, step_mode, local, smem_raw + cst_bytes<T>(sa.nl), tot, (T*)smem_raw);
    __syncthreads();
  }
}
template <typename T, bool COMP, bool PER, int CT>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 3 : 2) k_cols_ens(EnsArgs<T> e, int step_mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tot[GMAX * 32];
  __shared__ StepArgs<T> sa;
  __shared__ int cur;
  ens_init_cur(&cur);
  for (int item = blockIdx.x; item < e.total[1]; item += gridDim.x) {
    const int local = ens_item(e, e.start_cols, item, &sa, &cur);
    const int ntx = PER ? (sa.gx.H + 2) / 2 : (sa.nx + CT - 1) / CT;
    if (PER) body_cols_per<T, COMP>(sa, step_mode, local % ntx, local / ntx, smem_raw);
    else body_cols<T, COMP, CT>(sa, step_mode, local % ntx, local / ntx, smem_raw, tot);
    __syncthreads();
  }
}
template <typename T, bool COMP, bool PER>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 3 : 2) k_rows_inv_ens(EnsArgs<T> e, int step_mode) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T tot[GMAX * 32];
  __shared__ StepArgs<T> sa;
  __shared__ int cur;
  ens_init_cur(&cur);
  for (int item = blockIdx.x; item < e.total[2]; item += gridDim.x) {
    const int local = ens_item(e, e.start_rows, item, &sa, &cur);
    body_rows_inv<T, COMP, PER>(sa, step_mode, local, smem_raw + cst_bytes<T>(sa.nl), tot, (T*)smem_raw);
    __syncthreads();
  }
}
// RHS stage of an ensemble: one launch per halo radius R over the members
// with that radius (the work list of the launch gives the others no items),
// so each launch runs the same specialised body as a single run.
template <typename T, bool COMP, int R, int TY>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 5 : 3) k_rhs_ens(EnsArgs<T> e) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StepArgs<T> sa;
  __shared__ int cur;
  __shared__ unsigned long long bar;
  unsigned char* base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  if (threadIdx.x == 0 && threadIdx.y == 0) mbar_init(&bar);
  unsigned int phase = 0;
  ens_init_cur(&cur);
  for (int item = blockIdx.x; item < e.total[3]; item += gridDim.x) {
    const int local = ens_item(e, e.start_rhs, item, &sa, &cur);
    const int ntx = (sa.nx + TX - 1) / TX, nty = (sa.ny + TY - 1) / TY;
    const int bx = local % ntx, rest = local / ntx, by = rest % nty, bz = rest / nty;
    const unsigned int total = (unsigned int)(ntx * nty * sa.nl);
    // the tensor maps are read from the member table in global memory (TMA
    // takes them from the parameter, constant or global space, not shared);
    // only thread 0, which wrote cur, issues the copies
    body_rhs<T, COMP, R, TY>(sa, bx, by, bz, total, base, sa.use_tma ? &e.members[cur].tm[0] : nullptr, &bar, &phase);
    __syncthreads();
  }
}


// the RHS ensemble kernel of halo radius r and tile height ty
template <typename T, bool COMP>
static const void* rhs_ens_kernel(int r, int ty) {
  if (ty == 32)
    return r == 1 ? (const void*)k_rhs_ens<T, COMP, 1, 32> : r == 2 ? (const void*)k_rhs_ens<T, COMP, 2, 32>
         : r == 3 ? (const void*)k_rhs_ens<T, COMP, 3, 32> : (const void*)k_rhs_ens<T, COMP, 4, 32>;
  return r == 1 ? (const void*)k_rhs_ens<T, COMP, 1, 16> : r == 2 ? (const void*)k_rhs_ens<T, COMP, 2, 16>
       : r == 3 ? (const void*)k_rhs_ens<T, COMP, 3, 16> : (const void*)k_rhs_ens<T, COMP, 4, 16>;
}

template <typename T>
__global__ void k_begin_ens(EnsArgs<T> e, double t_out, double tend, const int* max_steps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < e.n) begin_state(e.members[i].state, t_out, tend, max_steps ? max_steps[i] : 0);
}
template <typename T>
__global__ void k_end_ens(EnsArgs<T> e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < e.n) e.members[i].state->pending = 0;
}


// flush of the pending AB3 update for every member, one row per work item
template <typename T, bool COMP>
__global__ void __launch_bounds__(NT) k_flush_ens(EnsArgs<T> e) {
  __shared__ StepArgs<T> sa;
  __shared__ int cur;
  ens_init_cur(&cur);
  for (int item = blockIdx.x; item < e.total[0]; item += gridDim.x) {
    const int j = ens_item(e, e.start_rows, item, &sa, &cur);
    const DevState* st = sa.state;
    if (st->pending) {
      int s0, s1, s2;
      slabs(st->step_index, s0, s1, s2);
      const double c0 = st->c0, c1 = st->c1, c2 = st->c2;
      const double sqdt = sqrt(st->dt);
      const size_t fs = (size_t)sa.nl * sa.lstride;
      const T* r1 = nullptr;
      const T* r2 = nullptr;
      T w1 = T(0), w2 = T(0);
      if (sa.nrec > 0) {
        const Forc4D fw = forc4d_at(st->t_prev, sa.dt_forc, sa.nrec);
        r1 = sa.frec + fw.i1 * fs;
        r2 = sa.frec + fw.i2 * fs;
        w1 = (T)fw.w1;
        w2 = (T)fw.w2;
      }
      for (int l = 0; l < sa.nl; ++l)
        for (int i = threadIdx.x; i < sa.nx; i += NT) {
          const size_t o = (size_t)l * sa.lstride + (size_t)j * sa.pitch + i;
          const T* fo = (sa.fr.on && l == 0) ? sa.fr.field + o : nullptr;
          if (COMP) {
            float hi = (float)sa.q[o], lo = (float)sa.qlo[o];
            const float d = ab3_increment((float)c0, (float)c1, (float)c2, (float)sa.fab[s0 * fs + o],
                                          (float)sa.fab[s1 * fs + o], (float)sa.fab[s2 * fs + o]);
            comp_add(hi, lo, d);
            if (fo) comp_add(hi, lo, (float)*fo * (float)sqdt);
            if (r1) comp_add(hi, lo, (float)forc4d_term<T>(r1, r2, o, w1, w2, (T)st->dt));
            sa.q[o] = (T)hi;
            sa.qlo[o] = (T)lo;
          } else {
            T v = ab3_plain<T>(sa.q[o], (T)c0, (T)c1, (T)c2, sa.fab[s0 * fs + o], sa.fab[s1 * fs + o],
                               sa.fab[s2 * fs + o]);
            if (fo) v = v + *fo * (T)sqdt;
            if (r1) v = v + forc4d_term<T>(r1, r2, o, w1, w2, (T)st->dt);
            sa.q[o] = v;
          }
        }
    }
    __syncthreads();
  }
}

// ---- ensembles: one persistent launch per stage over all members
template <typename T, bool COMP>
static cudaError_t set_attrs_ens() {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const int lim = optin - (int)(sizeof(T) * GMAX * 32 + sizeof(StepArgs<T>) + 128);
  if ((e = cudaFuncSetAttribute(k_rows_fwd_ens<T, COMP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)))
    return e;
  if ((e = cudaFuncSetAttribute(k_rows_inv_ens<T, COMP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)))
    return e;
  if ((e = cudaFuncSetAttribute(k_cols_ens<T, COMP, false, CTE<T>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)))
    return e;
  if ((e = cudaFuncSetAttribute(k_cols_ens<T, COMP, false, CTE<T> / 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                lim)))
    return e;
  if ((e = cudaFuncSetAttribute(k_rows_fwd_ens<T, COMP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)))
    return e;
  if ((e = cudaFuncSetAttribute(k_rows_inv_ens<T, COMP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)))
    return e;
  if ((e = cudaFuncSetAttribute(k_cols_ens<T, COMP, true, CTE<T>>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)))
    return e;
  const int rl = optin - (int)(sizeof(StepArgs<T>) + 1024);
  for (int t = 0; t < 2; ++t)
    for (int r = 1; r <= 4; ++r)
      if ((e = cudaFuncSetAttribute(rhs_ens_kernel<T, COMP>(r, t ? 32 : 16), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    rl)))
        return e;
  return cudaSuccess;
}

template <typename T, bool COMP>
static EnsSmem ens_smem(const StepArgs<T>* host_members, int n) {
  EnsSmem s{};
  for (int i = 0; i < n; ++i) {
    const StepArgs<T>& a = host_members[i];
    s.bytes[0] = std::max(s.bytes[0], smem_rows<T, COMP>(a));
    s.bytes[1] = std::max(s.bytes[1], smem_cols<T, COMP>(a));
    s.bytes[2] = std::max(s.bytes[2], smem_rows_inv<T, COMP>(a));
    s.bytes[3] = std::max(s.bytes[3], smem_rhs<T>(a));
    s.rhs_bytes[rhs_halo(a)] = smem_rhs<T>(a);
    s.rhs_ty = rhs_ty(a);  // the same for every member of an ensemble
    s.ct = col_width(a);
  }
  return s;
}

// the closed-basin column stage at the ensemble's column-tile width
template <typename T, bool COMP>
static void launch_cols_ens(const EnsArgs<T>& e, const EnsSmem& sm, int grid, int step_mode, cudaStream_t s) {
  if (sm.ct == CTE<T> / 2) k_cols_ens<T, COMP, false, CTE<T> / 2><<<grid, NT, sm.bytes[1], s>>>(e, step_mode);
  else k_cols_ens<T, COMP, false, CTE<T>><<<grid, NT, sm.bytes[1], s>>>(e, step_mode);
}

template <typename T, bool COMP>
static void ens_step(const EnsArgs<T>& e, const EnsArgs<T>* er, const EnsSmem& sm, const int* grid, const int* rgrid,
                     int which_mask, int periodic, cudaStream_t s) {
  if (periodic) {
    if (which_mask & 1) k_rows_fwd_ens<T, COMP, true><<<grid[0], NT, sm.bytes[0], s>>>(e, 1);
    if (which_mask & 2) k_cols_ens<T, COMP, true, CTE<T>><<<grid[1], NT, sm.bytes[1], s>>>(e, 1);
    if (which_mask & 4) k_rows_inv_ens<T, COMP, true><<<grid[2], NT, sm.bytes[2], s>>>(e, 1);
  } else {
    if (which_mask & 1) k_rows_fwd_ens<T, COMP, false><<<grid[0], NT, sm.bytes[0], s>>>(e, 1);
    if (which_mask & 2) launch_cols_ens<T, COMP>(e, sm, grid[1], 1, s);
    if (which_mask & 4) k_rows_inv_ens<T, COMP, false><<<grid[2], NT, sm.bytes[2], s>>>(e, 1);
  }
  if (which_mask & 8) {
    const dim3 blk(32, 8);
    for (int r = 1; r <= 4; ++r)
      if (rgrid[r] > 0) {
        void* args[] = {(void*)&er[r]};
        cudaLaunchKernel(rhs_ens_kernel<T, COMP>(r, sm.rhs_ty), dim3(rgrid[r]), blk, args, sm.rhs_bytes[r], s);
      }
  }
}
template <typename T, bool COMP>
static void ens_invert(const EnsArgs<T>& e, const EnsSmem& sm, const int* grid, int periodic, cudaStream_t s) {
  if (periodic) {
    k_rows_fwd_ens<T, COMP, true><<<grid[0], NT, sm.bytes[0], s>>>(e, 0);
    k_cols_ens<T, COMP, true, CTE<T>><<<grid[1], NT, sm.bytes[1], s>>>(e, 0);
    k_rows_inv_ens<T, COMP, true><<<grid[2], NT, sm.bytes[2], s>>>(e, 0);
    return;
  }
  k_rows_fwd_ens<T, COMP, false><<<grid[0], NT, sm.bytes[0], s>>>(e, 0);
  launch_cols_ens<T, COMP>(e, sm, grid[1], 0, s);
  k_rows_inv_ens<T, COMP, false><<<grid[2], NT, sm.bytes[2], s>>>(e, 0);
}

template <typename T, bool COMP>
static int ens_occupancy(int stage, size_t smem) {
  int b = 0;
  cudaError_t e = cudaSuccess;
  // the periodic variants have the same register and shared-memory needs
  if (stage == 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_rows_fwd_ens<T, COMP, false>, NT, smem);
  if (stage == 1) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_cols_ens<T, COMP, false, CTE<T>>, NT, smem);
  if (stage == 2) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_rows_inv_ens<T, COMP, false>, NT, smem);
  // stage 3 + R: the RHS kernel of halo radius R (both tile heights have the
  // same register needs; smem gives the difference)
  if (stage >= 4 && stage <= 7)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, rhs_ens_kernel<T, COMP>(stage - 3, 16), NT, smem);
  if (stage >= 8 && stage <= 11)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, rhs_ens_kernel<T, COMP>(stage - 7, 32), NT, smem);
  return e == cudaSuccess && b > 0 ? b : 1;
}
#if QGW_ENS_PART == 1
int ens_blocks_per_sm_f64(int stage, size_t smem) { return ens_occupancy<double, false>(stage, smem); }
int rhs_halo_of_f64(const StepArgs<double>& a) { return rhs_halo(a); }
int col_tiles_f64(const StepArgs<double>& a) { return col_tiles(a); }
cudaError_t ens_prepare_f64() { return set_attrs_ens<double, false>(); }
EnsSmem ens_smem_f64(const StepArgs<double>* m, int n) { return ens_smem<double, false>(m, n); }
void ens_begin_f64(const EnsArgs<double>& e, const int* max_steps, cudaStream_t s) {
  k_begin_ens<double><<<(e.n + 63) / 64, 64, 0, s>>>(e, 0.0, 0.0, max_steps);
}
void ens_step_f64(const EnsArgs<double>& e, const EnsArgs<double>* er, const EnsSmem& sm, const int* grid,
                  const int* rgrid, int mask, int periodic, cudaStream_t s) {
  ens_step<double, false>(e, er, sm, grid, rgrid, mask, periodic, s);
}
void ens_invert_f64(const EnsArgs<double>& e, const EnsSmem& sm, const int* grid, int periodic, cudaStream_t s) {
  ens_invert<double, false>(e, sm, grid, periodic, s);
}
void ens_flush_f64(const EnsArgs<double>& e, int grid, cudaStream_t s) {
  k_flush_ens<double, false><<<grid, NT, 0, s>>>(e);
  k_end_ens<double><<<(e.n + 63) / 64, 64, 0, s>>>(e);
}
#else
int ens_blocks_per_sm_f32c(int stage, size_t smem) { return ens_occupancy<float, true>(stage, smem); }
int col_tiles_f32c(const StepArgs<float>& a) { return col_tiles(a); }
int rhs_halo_of_f32c(const StepArgs<float>& a) { return rhs_halo(a); }
cudaError_t ens_prepare_f32c() { return set_attrs_ens<float, true>(); }
EnsSmem ens_smem_f32c(const StepArgs<float>* m, int n) { return ens_smem<float, true>(m, n); }
void ens_begin_f32c(const EnsArgs<float>& e, const int* max_steps, cudaStream_t s) {
  k_begin_ens<float><<<(e.n + 63) / 64, 64, 0, s>>>(e, 0.0, 0.0, max_steps);
}
void ens_step_f32c(const EnsArgs<float>& e, const EnsArgs<float>* er, const EnsSmem& sm, const int* grid,
                   const int* rgrid, int mask, int periodic, cudaStream_t s) {
  ens_step<float, true>(e, er, sm, grid, rgrid, mask, periodic, s);
}
void ens_invert_f32c(const EnsArgs<float>& e, const EnsSmem& sm, const int* grid, int periodic, cudaStream_t s) {
  ens_invert<float, true>(e, sm, grid, periodic, s);
}
void ens_flush_f32c(const EnsArgs<float>& e, int grid, cudaStream_t s) {
  k_flush_ens<float, true><<<grid, NT, 0, s>>>(e);
  k_end_ens<float><<<(e.n + 63) / 64, 64, 0, s>>>(e);
}
#endif  // QGW_ENS_PART

}  // namespace qgw
