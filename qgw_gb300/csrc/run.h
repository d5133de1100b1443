// run.h -- the run handle shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/qgw_gpu.h"
#include "qgw_device.cuh"

struct qgw_run {
  int precision = 0;
  qgw_params p{};
  int nx = 0, ny = 0, nl = 0, pitch = 0;
  size_t lstride = 0;
  double Delta = 0, Ly = 0, norm = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  qgw::DevState* d_state = nullptr;
  qgw::DevState* h_state = nullptr;  // pinned
  double* d_full = nullptr;        // (nl, ny+2, nx+2) reference-layout staging for host copies
  double* d_wts = nullptr;
  double* d_part = nullptr;
  double* d_bout = nullptr;
  int budget_blocks = 0;
  qgw::StepArgs<double> a64{};
  qgw::StepArgs<float> a32{};
  std::vector<double> cl2m, cm2l, iRd2;
  bool has_q = false;
};
