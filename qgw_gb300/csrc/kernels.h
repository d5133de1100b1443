// kernels.h -- host-side launchers of the step kernels (kernels.cu, kernels_ens.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "qgw_device.cuh"

namespace qgw {

cudaError_t prepare_f64(const StepArgs<double>& a);
cudaError_t prepare_f32c(const StepArgs<float>& a);
// blocks of the persistent RHS kernel (resident blocks per SM x SMs; 0:
// one block per tile, as the FP64 path runs); after prepare_*
int rhs_grid_f64(const StepArgs<double>& a);
int rhs_grid_f32c(const StepArgs<float>& a);

void enqueue_begin(DevState* st, double t_out, double tend, cudaStream_t s);
void enqueue_step_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_step_f32c(const StepArgs<float>& a, cudaStream_t s);
void enqueue_invert_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_invert_f32c(const StepArgs<float>& a, cudaStream_t s);
// the stochastic forcing kernels of one step (ensembles launch them per member)
void enqueue_forcing_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_forcing_f32c(const StepArgs<float>& a, cudaStream_t s);
void enqueue_flush_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_flush_f32c(const StepArgs<float>& a, cudaStream_t s);
// which: 0 rows forward, 1 columns, 2 rows inverse, 3 RHS (step mode)
void enqueue_step_kernel_f64(const StepArgs<double>& a, int which, cudaStream_t s);
void enqueue_step_kernel_f32c(const StepArgs<float>& a, int which, cudaStream_t s);

// reference layout (nl, ny+2, nx+2), contiguous on the device <-> run layout
void enqueue_unpack_f64(const double* full, double* q, int nx, int ny, int nl, int pitch, cudaStream_t s);
void enqueue_unpack_split(const double* full, float* hi, float* lo, int nx, int ny, int nl, int pitch,
                          cudaStream_t s);
void enqueue_pack_f64(const double* src, double* full, int nx, int ny, int nl, int pitch, cudaStream_t s);
void enqueue_pack_join(const float* hi, const float* lo, double* full, int nx, int ny, int nl, int pitch,
                       cudaStream_t s);
void enqueue_split_f64(const double* src, float* hi, float* lo, size_t n, cudaStream_t s);
void enqueue_join_f64(const float* hi, const float* lo, double* dst, size_t n, cudaStream_t s);

void enqueue_budget_f64(const StepArgs<double>& a, const double* wts, double* part, int nblk, double scale,
                        double* out, cudaStream_t s);
void enqueue_budget_f32c(const StepArgs<float>& a, const double* wts, double* part, int nblk, double scale,
                         double* out, cudaStream_t s);

// ensembles (one persistent launch per stage over all members)
// dynamic shared memory per stage; the RHS stage per halo radius R (rhs_bytes[R], 0: no member)
// and the (ensemble-wide) RHS tile height and column-tile width
struct EnsSmem { size_t bytes[4]; size_t rhs_bytes[5]; int rhs_ty; int ct; };
cudaError_t ens_prepare_f64();
cudaError_t ens_prepare_f32c();
EnsSmem ens_smem_f64(const StepArgs<double>* host_members, int n);
EnsSmem ens_smem_f32c(const StepArgs<float>* host_members, int n);
void ens_begin_f64(const EnsArgs<double>& e, const int* max_steps, cudaStream_t s);
void ens_begin_f32c(const EnsArgs<float>& e, const int* max_steps, cudaStream_t s);
// mask: bit k launches kernel k (0 rows forward, 1 columns, 2 rows inverse,
// 3 RHS); the RHS stage is one launch per halo radius R with er[R] (whose
// work list holds only the members of that radius) and grid rgrid[R] (0: none)
// periodic != 0: every member is a doubly periodic basin (the row and column
// kernels use the real / complex FFT instead of the DST-I)
void ens_step_f64(const EnsArgs<double>& e, const EnsArgs<double>* er, const EnsSmem& sm, const int* grid,
                  const int* rgrid, int mask, int periodic, cudaStream_t s);
void ens_step_f32c(const EnsArgs<float>& e, const EnsArgs<float>* er, const EnsSmem& sm, const int* grid,
                   const int* rgrid, int mask, int periodic, cudaStream_t s);
void ens_invert_f64(const EnsArgs<double>& e, const EnsSmem& sm, const int* grid, int periodic, cudaStream_t s);
void ens_invert_f32c(const EnsArgs<float>& e, const EnsSmem& sm, const int* grid, int periodic, cudaStream_t s);
void ens_flush_f64(const EnsArgs<double>& e, int grid, cudaStream_t s);
void ens_flush_f32c(const EnsArgs<float>& e, int grid, cudaStream_t s);
// resident blocks per SM of an ensemble stage kernel with `smem` bytes of
// dynamic shared memory (stage 0 rows forward, 1 columns, 2 rows inverse,
// 3 + R the RHS kernel of halo radius R = 1..4)
int ens_blocks_per_sm_f64(int stage, size_t smem);
int ens_blocks_per_sm_f32c(int stage, size_t smem);
// halo radius R of a run's RHS kernel (the number of hyperviscosity sweeps, at least 1)
int rhs_halo_of_f64(const StepArgs<double>& a);
// column-kernel work items (tiles) per mode of a run
int col_tiles_f64(const StepArgs<double>& a);
int col_tiles_f32c(const StepArgs<float>& a);
int rhs_halo_of_f32c(const StepArgs<float>& a);
int cols_per_tile_f64();
int cols_per_tile_f32c();
int rhs_tile_x();
// TMA box width (columns) of the RHS kernel's interior tiles
int rhs_box_width();
// RHS tile height of a run (16 or 32 rows)
int rhs_tile_y_f64(const StepArgs<double>& a);
int rhs_tile_y_f32c(const StepArgs<float>& a);

size_t smem_bytes_rows_f64(const StepArgs<double>& a);
size_t smem_bytes_cols_f64(const StepArgs<double>& a);
size_t smem_bytes_rhs_f64(const StepArgs<double>& a);
size_t smem_bytes_rows_f32c(const StepArgs<float>& a);
size_t smem_bytes_cols_f32c(const StepArgs<float>& a);
size_t smem_bytes_rhs_f32c(const StepArgs<float>& a);

}  // namespace qgw
