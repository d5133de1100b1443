// qgw_device.cuh -- device-side state and kernel argument types of the
// GB300 time step.
//
// Data layout in HBM (one run):
//   interior-only fields, [nl][ny][pitch] with pitch = nx+1 (the DST length
//   plus one padding column); reference point (i, j, k) with 1 <= i <= nx,
//   1 <= j <= ny lives at k*ny*pitch + (j-1)*pitch + (i-1).  Ghost/wall
//   values are never stored: kernels derive them from the boundary rule of
//   adjust_bc (src/domain.h:308-348).
//   q      FP64 (plain) or FP32 hi + FP32 lo (compensated)
//   psi    streamfunction, same precision as the arithmetic
//   spec   spectral work field between the row and column passes
//   fab    3 slabs of the AB3 history (f0/f1/f2 rotate by step index)
//   hinv   FP64 path only: 1 / (-(L^2 + K^2 + iRd2_m) * norm) per (m, j, k)
//   topo   (ny+2) x (nx+2) reference layout (only when non-zero)
// The doubly periodic basin keeps the same layout with nx = NX, ny = NY and
// pitch = NX + 2 rounded up to a multiple of 4 (room for the NX/2 + 1
// complex values of a spectral row, 16-byte aligned rows).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "dst_core.h"
#include "glibc_rand.h"

namespace qgw {

// try_wait polls of a bounded mbarrier wait (each poll may itself suspend the
// thread for a hardware-defined interval): far longer than any tile load
// takes, short enough that a lost copy ends the kernel with an error status
constexpr int kWaitIters = 1 << 22;

// Scalars that evolve on the device (the reference globals t, dt, dt0,
// dt1 of src/qg.c:63-64 and src/timestep.h:14, plus the control flags of
// the device-side driver loop).
struct DevState {
  double t, dt, dt0, dt1, DT_max;
  double t_out, tend;
  double c0, c1, c2;               // AB3 coefficients of the pending update
  unsigned long long maxbits;      // CFL: max |dpsi| over the step, as bits
  unsigned int done_blocks;        // last-block detection in the RHS kernel
  int pending;                     // AB3 update computed but not yet applied
  int active;                      // steps continue while 1
  int first;                       // first step of the current call
  int steps_taken;
  int stop_reason;                 // 0 nsteps, 1 t_out, 2 tend, 3 non-finite
  int nonfinite;
  int step_index;                  // RHS evaluations so far (slab rotation)
  int max_steps;                   // > 0: stop after this many steps in the call
  int forc_step;                   // step_index of the current stochastic forcing field
  double t_prev;                   // t before the last step's increment (4-D forcing time)
  int dev_error;                   // 1: a bounded device wait ran out (tile skipped)
};

// Stochastic thin-ring forcing (src/forcing.h:67-201): each step a new
// field of random complex amplitudes on the ring of the NF x (NF/2+1) half
// spectrum, transformed by a 2-D c2r of size NF x NF (NF = NX), added to
// layer 0 as forc * sqrt(dt) after the AB3 update (src/timestep.h:143-150).
template <typename T> struct ForcArgs {
  int on;                          // k_f != 0 and more than one ring point
  int nring;                       // ring points (i, j)
  int NF;                          // transform size
  int fpitch;                      // row pitch (reals) of the spectral buffers
  int col_blocks;                  // column pairs holding ring points: the
                                   // transform along j skips the zero columns
  DstGeom gx, gy;                  // real FFT of NF along i; complex FFT of NF along j
  DstTables<T> tx, ty;
  const int* ring;                 // 2 * nring: i, j
  double env;                      // sqrt(8 / ((N_P - 1) 2)) pi k_f / (2 pi)
  double sigma;                    // sigma_f
  GlibcRand* rng;                  // the C-library generator's state
  T* spec;                         // NF x fpitch: ring amplitudes (zero elsewhere)
  T* spec2;                        // NF x fpitch: after the transform along j
  T* field;                        // [ny][pitch] of the run: the forcing of layer 0
};

// Everything a step kernel needs, passed by value.
template <typename T> struct StepArgs {
  // sizes
  int nx, ny, nl, pitch;
  long long lstride;               // ny * pitch
  DstGeom gx, gy;
  DstTables<T> tx, ty;
  // vertical modes (FP64 master copies and T copies)
  const T* cl2m;                   // nl*nl row-major, mode m row: cl2m[m*nl+l]
  const T* cm2l;                   // cm2l[l*nl+m]
  const double* iRd2;
  // fields
  T* q;                            // plain: q; compensated: q_hi
  T* qlo;                          // compensated only
  T* psi;
  T* spec;
  T* spec2;                        // compensated: spectral zeta between K2 and K3
  T* zeta;                         // compensated: discrete Laplacian of psi
  T* fab;                          // 3 slabs of nl*lstride
  const double* hinv;              // FP64 path
  const double* Lsq;               // L_{k+1}^2, k < nx
  const double* Ksq;               // K_{j+1}^2, j < ny
  const T* wind;                   // per interior row j: forcing_q (layer 0)
  const double* topo;              // (ny+2)*(nx+2) or null
  DevState* state;
  // physics
  double Delta, norm, cfl;
  double inv12d2;                  // 1 / (12 Delta^2)
  double b2d;                      // beta / (2 Delta)
  double nu_d2;                    // nu / Delta^2
  double nuh_scaled;               // nu_hyper / Delta^(2S)  (unscaled chain)
  double drag_d2;                  // -hEkb f0 / (2 dh_{nl-1}) / Delta^2
  double topo_fac;                 // f0 / dh_{nl-1}
  double cbc;                      // 2 bc_fac / Delta^2 (ghost rule)
  double gh[8];                    // ghost factor of chain sweep s: 2 bc Delta^(2s-2)
  int nsweep;                      // hyperviscosity Laplacian sweeps (0: off)
  int has_nu, has_topo, has_wind, has_drag;
  // grouping
  int G1;                          // modes per block in the row passes
  int G3;                          // modes per block in K3 (zeta doubles the rows)
  // compensated path: a second spectral field formed in K2, transformed by
  // K3 into `zeta`, read by K4.  0: none.  1: zeta = L psi (the 5-point
  // Laplacian), which K4 continues into the hyperviscosity chain and uses
  // for the bottom drag.  2: zeta = L^nsweep psi, the whole hyperviscosity
  // chain, which is diagonal in the transform basis when every sweep sees
  // zero ghosts (free-slip walls) or wrapped ones (periodic): K4 runs no
  // sweeps and needs a halo of 1 (runs without bottom drag).
  int zeta_mode;
  double lx2, ly2;                 // -4/Delta^2 factors of the discrete symbol
  const double* sx2;               // sin^2(pi k / (2 Mx)), k = 1..nx
  const double* sy2;               // sin^2(pi j / (2 My)), j = 1..ny
  // FP32 copies of the per-wavenumber tables (compensated path)
  const float* Lsqf;
  const float* Ksqf;
  const float* sx2f;
  const float* sy2f;
  // FP32 copies of the RHS and Helmholtz constants (compensated path), made
  // on the host: a double -> float conversion runs on the FP64 pipe
  float fc[24];
  const float* iRd2f;
  int CT;                          // (unused by the kernels; kept for layout)
  int vec_cols;                    // rows are 16-byte aligned: 16-byte column loads
  int low_k64;                     // compensated: FP64 divide for mode 0, j,k < low_k64
  ForcArgs<T> fr;                  // stochastic forcing (fr.on = 0: none)
  // 4-D forcing (src/forcing.h:226-288): nrec records [nrec][nl][ny][pitch],
  // interpolated linearly in time with period nrec * dt_forc, added to every
  // layer as q_forc * dt after the AB3 update (src/timestep.h:152-163)
  const T* frec;
  int nrec;                        // 0: no 4-D forcing
  double dt_forc;
  // TMA tensor maps of the RHS kernel's interior tiles (psi, q, zeta), boxes
  // of 40 columns starting at x = i0 - 4 (16-byte aligned); use_tma = 0:
  // the element-wise asynchronous copies instead
  CUtensorMap tm[3];
  int use_tma;
  int rhs_grid;  // blocks of the persistent RHS kernel (0: one per tile)
  int rhs_ty;    // RHS tile height: 16 (default) or 32 rows
  // K3 grid: 1 = one block per (row, layer group), 0 = one block per row
  // that runs the row's layer groups in turn (same arithmetic per layer)
  int inv_split;
  // iterations of the first bounded wait for a tile's TMA bytes (normally
  // kWaitIters; lowered only by tests, to make that wait run out -- the
  // second wait, which lets the bytes land before the block moves on, always
  // keeps kWaitIters)
  int wait_iters;
  // doubly periodic basin (bc_fac = -1): nx = NX, ny = NY interior points,
  // pitch = NX + 2 rounded up to 4; gx has M = NX (real FFT of length NX as a complex FFT
  // of NX/2), gy has M = 2 NY (complex FFT of length NY); spectral rows hold
  // X_0..X_{NX/2} as (re, im) pairs; ghost values wrap around
  int periodic;
  // the first forward-rows pass of a call may read q straight from the
  // caller's host array (reference layout, an address the device can use;
  // null: q is already in the run's field)
  const double* qin;
  // the flush of a call may also write q to the caller's host array
  // (reference layout interior; null: none)
  double* qout;
};

// indices into StepArgs::fc
enum FcIndex {
  FC_D2 = 0,      // Delta^2
  FC_CBC,         // cbc
  FC_MINV12,      // -inv12d2
  FC_B2D,         // b2d
  FC_NUD2,        // nu_d2
  FC_NUH,         // nuh_scaled
  FC_DRAG,        // drag_d2
  FC_TOPOC,       // -(inv12d2 * topo_fac)
  FC_GH1,         // gh[1..4]
  FC_NORM = FC_GH1 + 4,
  FC_LX2,
  FC_LY2,
  FC_NUHS,        // nu_hyper itself (zeta_mode 2: the field is scaled)
  FC_NUHD2,       // nuh_scaled * Delta^2 (zeta_mode 1: the chain runs on L psi / Delta^2)
  FC_GHD1,        // gh[1..4] / Delta^2 (its ghost factors)
  FC_COUNT = FC_GHD1 + 4
};
static_assert(FC_COUNT <= (int)(sizeof(StepArgs<float>::fc) / sizeof(float)), "fc holds every constant");

// A batch of runs advanced by one launch per stage (see kernels_ens.cu).
template <typename T> struct EnsArgs {
  const StepArgs<T>* members;  // device array, n entries
  const int* start_rows;       // n+1 prefix sums of per-member work items (rows, ny)
  const int* start_cols;       // column tiles x modes
  const int* start_rhs;        // RHS tiles x layers
  const int* total;            // [4]: items of K1, K2, K3, K4
  int n;
};

}  // namespace qgw
