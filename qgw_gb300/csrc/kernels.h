// kernels.h -- host-side launchers of the step kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "qgw_device.cuh"

namespace qgw {

cudaError_t prepare_f64(const StepArgs<double>& a);
cudaError_t prepare_f32c(const StepArgs<float>& a);

void enqueue_begin(DevState* st, double t_out, double tend, cudaStream_t s);
void enqueue_step_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_step_f32c(const StepArgs<float>& a, cudaStream_t s);
void enqueue_invert_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_invert_f32c(const StepArgs<float>& a, cudaStream_t s);
void enqueue_flush_f64(const StepArgs<double>& a, cudaStream_t s);
void enqueue_flush_f32c(const StepArgs<float>& a, cudaStream_t s);
// which: 0 rows forward, 1 columns, 2 rows inverse, 3 RHS (step mode)
void enqueue_step_kernel_f64(const StepArgs<double>& a, int which, cudaStream_t s);
void enqueue_step_kernel_f32c(const StepArgs<float>& a, int which, cudaStream_t s);

void enqueue_split_f64(const double* src, float* hi, float* lo, size_t n, cudaStream_t s);
void enqueue_join_f64(const float* hi, const float* lo, double* dst, size_t n, cudaStream_t s);

void enqueue_budget_f64(const StepArgs<double>& a, const double* wts, double* part, int nblk, double scale,
                        double* out, cudaStream_t s);
void enqueue_budget_f32c(const StepArgs<float>& a, const double* wts, double* part, int nblk, double scale,
                         double* out, cudaStream_t s);

size_t smem_bytes_rows_f64(const StepArgs<double>& a);
size_t smem_bytes_cols_f64(const StepArgs<double>& a);
size_t smem_bytes_rhs_f64(const StepArgs<double>& a);
size_t smem_bytes_rows_f32c(const StepArgs<float>& a);
size_t smem_bytes_cols_f32c(const StepArgs<float>& a);
size_t smem_bytes_rhs_f32c(const StepArgs<float>& a);

}  // namespace qgw
