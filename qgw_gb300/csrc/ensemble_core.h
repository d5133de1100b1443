// ensemble_core.h -- a batch of runs advanced by one launch per step stage;
// shared by the ensemble and pool (serving) entry points.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "kernels.h"
#include "qgw_device.cuh"
#include "run.h"

namespace qgw {

struct EnsembleCore {
  int precision = 0;
  int periodic = 0;               // all members doubly periodic (else all bounded)
  int nsm = 0;
  cudaStream_t stream = nullptr;
  std::vector<qgw_run*> members;  // not owned by the core
  void* d_members = nullptr;      // device member table
  // start_rows | start_cols | start_rhs | total[4], then per halo radius
  // R = 1..4: start_rhs of the members with radius R | total[4]
  int* d_lists = nullptr;
  int* d_maxsteps = nullptr;
  EnsArgs<double> e64{};
  EnsArgs<float> e32{};
  EnsArgs<double> r64[5]{};       // RHS stage per halo radius R (index 1..4)
  EnsArgs<float> r32[5]{};
  EnsSmem sm{};
  int total[4] = {0, 0, 0, 0};
  int rhs_total[5] = {0, 0, 0, 0, 0};
  // persistent blocks per SM, per stage (tuned; capped by residency);
  // 0: one block per work item
  int bps[4] = {8, 8, 8, 8};
  int grid[4] = {0, 0, 0, 0};
  int rhs_grid[5] = {0, 0, 0, 0, 0};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<DevState> h_states;
};

// (re)build the device member table and work lists from e->members
int ens_core_build(EnsembleCore* e);
void ens_core_free_tables(EnsembleCore* e);
// enqueue up to nsteps steps for every member (max_steps[i] > 0 caps member
// i) and the final flush on e->stream; returns without waiting
int ens_core_step(EnsembleCore* e, int nsteps, const int* max_steps, bool use_graph);
// wait for the stream and read every member's device scalars into h_states
int ens_core_finish(EnsembleCore* e);

}  // namespace qgw
