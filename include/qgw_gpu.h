/*
 * qgw_gpu.h -- C ABI of libqgw_gpu.so, the GB300 (sm_103a) time-stepping
 * engine of the multi-layer quasi-geostrophic model qgw.
 *
 * The reference program keeps its whole state in globals and advances it
 * with four C functions that the driver calls directly:
 *
 *   invert_pv(q, psi)        src/elliptic.h:76    (called at src/qg.c:167,188)
 *   timestep(q)              src/timestep.h:114   (called at src/qg.c:197)
 *   rhs(q, f)                src/dynamics.h:47    (inside timestep)
 *   adjust_timestep(psi)     src/timestep.h:69    (inside timestep)
 *
 * plus the host-side set-up read_params (src/extra.h:118),
 * compute_eigmode (src/eigmode.h:87) and check_timestep (src/timestep.h:18).
 * This header replaces that global-state interface with an opaque run handle.
 * A host driver that used to call the functions above calls the entry points
 * below instead; fields cross the boundary in the reference's own array
 * layout, so output code written against the reference stays unchanged.
 *
 * Array layout at the boundary ("reference layout"): a 3-D field is
 * (nl, ny+2, nx+2) row-major doubles with a one-point ghost/wall ring,
 * element (i, j, k) at k*(ny+2)*(nx+2) + j*(nx+2) + i, exactly the idx()
 * macro of src/domain.h:62.  For a closed basin (bc_fac >= 0) the interior
 * sizes are nx = NX-1, ny = NY-1 (src/domain.h:71-74).
 *
 * Conventions: every entry point returns 0 on success or a negative
 * qgw_status; nothing in the library calls exit().  All device memory is
 * owned by the library; host arrays are owned by the caller and are only
 * read/written during the call that receives them.  One run handle may be
 * used from one host thread at a time.
 */
#ifndef QGW_GPU_H
#define QGW_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QGW_ABI_VERSION 2

/* Largest number of layers a params struct can describe: the reference's
 * nl_max (src/qg.c:45), which sizes its dh/N2 arrays.  The GPU kernels
 * accept nl <= QGW_NL_GPU_MAX (their per-block projection coefficients,
 * nl x 16 values, sit in shared memory); the allocation-free inversion
 * keeps nl <= 32. */
#define QGW_NL_MAX 1000
#define QGW_NL_GPU_MAX 256

typedef enum qgw_status {
  QGW_OK = 0,
  QGW_ERR_PARAM = -1,       /* invalid or unsupported parameter            */
  QGW_ERR_FILE = -2,        /* params file missing (reference: exit(0))    */
  QGW_ERR_CUDA = -3,        /* a CUDA runtime call failed                  */
  QGW_ERR_NOMEM = -4,       /* device or host allocation failed            */
  QGW_ERR_NAN = -5,         /* NaN/Inf detected in the state               */
  QGW_ERR_UNSUPPORTED = -6, /* configuration outside what the kernels do   */
  QGW_ERR_EIGEN = -7,       /* stretching-matrix eigensolver failed        */
  QGW_ERR_STATE = -8,       /* call out of order (e.g. step before set_q)  */
  QGW_ERR_ADMISSION = -9,   /* pool: request does not fit the HBM budget   */
  QGW_ERR_TIMEOUT = -10,    /* a bounded device wait gave up               */
  QGW_ERR_NOT_READY = -11   /* pool: result not available yet              */
} qgw_status;

typedef enum qgw_precision {
  QGW_FP64 = 0,  /* plain FP64: the drop-in step                           */
  QGW_FP32C = 1  /* FP32 arithmetic, q kept as an FP32 hi+lo pair           */
} qgw_precision;

/* Every key the reference registers from params.in (src/qg.c:113-137),
 * with the reference's defaults (src/qg.c:57-83, src/forcing.h:13-14,38-39),
 * plus one optional extra key `dt` (fixed time step; 0 = adaptive, the
 * reference behaviour).  The reference parser ignores unknown keys, so a
 * params.in carrying `dt` still drives the reference unchanged. */
typedef struct qgw_params {
  int NX, NY, nl, n_hyper;
  double Lx;
  double dh[QGW_NL_MAX];
  double N2[QGW_NL_MAX];
  double tau0, forc_mode, f0, beta, nu, nu_hyper, hEkb, Ld;
  double h_topo, w_topo, bc_fac, tend, dt_out;
  double dt_forc, dt_forc_period, sigma_f, k_f, cfl;
  double dt;  /* extra key: fixed dt when > 0 */
} qgw_params;

/* Time-stepping scalars of a run (the reference globals t, dt, dt0, dt1,
 * DT_max, src/qg.c:63-69 and src/timestep.h:14). */
typedef struct qgw_time {
  double t, dt, dt0, dt1, DT_max;
} qgw_time;

typedef struct qgw_step_info {
  qgw_time time;   /* after the last step taken                        */
  int steps_taken; /* <= nsteps; fewer when a stop condition was hit    */
  int stop_reason; /* 0 = nsteps done, 1 = reached t_out, 2 = reached tend */
  int nonfinite;   /* 1 if a NaN/Inf was seen in the CFL reduction       */
} qgw_step_info;

/* FP64 domain diagnostics (no reference counterpart in C; the energy and
 * enstrophy formulas follow test/test_energy_injection.py:24-25).  All sums
 * are over interior points and weighted by Delta^2/(Lx*Ly). */
typedef struct qgw_budget_out {
  double ke;          /* sum_k dh_k/H * 1/2 |grad psi_k|^2 (one-sided, as CFL) */
  double energy;      /* -sum_k dh_k/H * psi_k q_k  (test_energy_injection.py) */
  double enstrophy;   /* sum_k dh_k/H * q_k^2                                  */
  double wind_work;   /* -dh_0/H * psi_0 * forcing_q  (rate of energy input)   */
} qgw_budget_out;

typedef struct qgw_run qgw_run;

/* ---- host-side set-up (no GPU needed) ---------------------------------- */

/* Fill p with the reference defaults (src/qg.c:57-83). */
void qgw_params_default(qgw_params* p);

/* Parse a params.in file into p (which should hold defaults first).
 * Same grammar as read_params, src/extra.h:118-153: lines `key = value` or
 * `key = [a, b, ...]`, spaces ignored, unknown keys and comments ignored.
 * Returns QGW_ERR_FILE where the reference calls exit(0). */
int qgw_params_read(qgw_params* p, const char* path);

/* Vertical modes of the stretching matrix: replaces compute_eigmode,
 * src/eigmode.h:87-271 (LAPACKE_dgeev there, the implicit-QL
 * symmetric-tridiagonal solver here; the Flierl normalisation makes both
 * give the same result, up to the sign of a mode trapped at depth, whose
 * surface value -- the sign rule -- is at round-off level; such a flip of a
 * mode's cm2l column and cl2m row together changes no result).  cl2m, cm2l
 * are nl*nl row-major, iRd2 has nl entries. */
int qgw_eigmode(const qgw_params* p, double* cl2m, double* cm2l, double* iRd2);

/* Maximum and initial time step: replaces check_timestep,
 * src/timestep.h:18-54, including its operator-precedence quirks. */
int qgw_check_timestep(const qgw_params* p, double* DT_max, double* dt);

/* Topography on the reference layout (ny+2, nx+2): init_vars,
 * src/domain.h:200-207. */
int qgw_topo(const qgw_params* p, double* topo);

/* ---- one run on one GPU ------------------------------------------------ */

/* Create a run on the current CUDA device.  cl2m/cm2l/iRd2 may be NULL, in
 * which case qgw_eigmode() is used.  topo may be NULL (flat bottom, or the
 * analytic shelf of qgw_topo() when h_topo != 0); otherwise it is a
 * (ny+2, nx+2) reference-layout array.  The time scalars start as the
 * reference's init_timestep leaves them (src/timestep.h:56-67), or at the
 * fixed dt when p->dt > 0.  q starts at zero.  Grids: 4 <= NX, NY <= 8192.
 * Closed basins take any size: where NX or NY is even with NX/2 (NY/2) a
 * product of 2, 3, 5 and 7 the transform is a half-length FFT, otherwise a
 * chirp-z transform of power-of-two length (slower; up to 2048 points;
 * such runs are refused by ensembles and the serving pool).  Periodic grids
 * square, NX even with NX/2 a product of 2, 3, 5 and 7.  1..QGW_NL_GPU_MAX
 * layers.  The column kernel holds whole columns in shared memory, which
 * bounds NY: closed basins NY <= 6300 (FP32C with hyperviscosity or bottom
 * drag, whose second spectral field doubles the buffers: NY <= 3150);
 * periodic NX = NY <= 3150 (FP64), 4200 (FP32C with that field) or 6300.
 * Anything else returns QGW_ERR_UNSUPPORTED. */
int qgw_create(const qgw_params* p, const double* cl2m, const double* cm2l,
               const double* iRd2, const double* topo, int precision,
               qgw_run** out);

/* Release the run and its device memory. */
void qgw_destroy(qgw_run* run);

/* Copy q in (reference layout; ghost values are ignored).  Replaces the
 * restart read of q, src/qg.c:160-164.  Clears the AB3 history. */
int qgw_set_q(qgw_run* run, const double* q);

/* Same, from a device pointer holding the reference layout. */
int qgw_set_q_device(qgw_run* run, const double* q_dev);

/* Replace q but keep the AB3 history: the reference's timestep(q)
 * (src/timestep.h:114-167) works on the caller's q array while f0/f1/f2 stay in
 * globals, so a driver that owns q on the host calls qgw_put_q, qgw_step(1),
 * qgw_get(NULL, q) per step.  Requires a prior qgw_set_q. */
int qgw_put_q(qgw_run* run, const double* q);

/* Read and overwrite the time scalars (t, dt, dt0, dt1, DT_max). */
int qgw_get_time(qgw_run* run, qgw_time* out);
int qgw_set_time(qgw_run* run, const qgw_time* in);

/* Stochastic ring forcing (k_f != 0, src/forcing.h:67-201): the noise is
 * the C library's rand() sequence, which the reference draws unseeded, so a
 * run starts from seed 1 like a fresh reference process and continues it
 * across qgw_step calls.  qgw_set_forcing_seed restarts the sequence as
 * srand(seed) would (independent realisations for ensembles).  No reference
 * counterpart (the reference never seeds).  QGW_ERR_STATE when the run has
 * no forcing. */
int qgw_set_forcing_seed(qgw_run* run, unsigned int seed);

/* 4-D forcing (dt_forc_period != 0, src/forcing.h:226-288): the
 * n_rec = dt_forc_period / dt_forc records of q_forcing_3d that the
 * reference reads from input_vars.nc (read_nc, src/netcdf_io.h:286-382),
 * given here in the reference layout (n_rec, nl, ny+2, nx+2) as read_nc
 * fills them; they stay resident on the device.  Each step adds
 * (w1 rec[i1] + w2 rec[i2]) * dt to every layer, the weights linear in the
 * time before the step (calc_4d_forcing).  nrec must be at least n_rec
 * (the first n_rec are used).  A run configured with 4-D forcing refuses
 * to step (QGW_ERR_STATE) until its records are set. */
int qgw_set_forcing_records(qgw_run* run, const double* records, int nrec);

/* Advance up to nsteps reference time steps (timestep(), src/timestep.h:114-167).
 * t_out is the next output time used by the dt snapping of
 * adjust_timestep (src/timestep.h:97-109); pass 0 for none.  Mirrors the
 * driver loop src/qg.c:181-199: before each step, stop if t >= tend
 * (tend <= 0: no limit) or |t - t_out| < 1e-9*dt.  Work stays on the device
 * between steps; the call returns after the last step has finished. */
int qgw_step(qgw_run* run, int nsteps, double t_out, double tend,
             qgw_step_info* info);

/* The reference's timestep(q) on the caller's host array, nsteps times:
 * q_in (reference layout, or NULL) replaces q keeping the AB3 history, as
 * qgw_put_q; q_out (or NULL) receives q after the steps, as qgw_get.  The
 * two may be the same array.  Where the device can address q_in (pinned
 * memory, or any host memory on a Grace host), the first kernel of the call
 * reads it across the C2C link itself, so the transfer overlaps that
 * kernel's arithmetic instead of preceding it. */
int qgw_step_host(qgw_run* run, int nsteps, double t_out, double tend,
                  const double* q_in, double* q_out, qgw_step_info* info);

/* Recompute psi from the current q (invert_pv, src/elliptic.h:76-155). */
int qgw_invert(qgw_run* run);

/* Copy psi and/or q out in the reference layout (either may be NULL).  The
 * ghost ring is what the reference holds after invert_pv:
 * psi = 0, q = 2*bc_fac/Delta^2 * psi_adjacent (src/domain.h:308-348).
 * psi is the inversion of the current q (qgw_invert is implied when psi is
 * requested, or for q when bc_fac != 0). */
int qgw_get(qgw_run* run, double* psi, double* q);

/* FP64 diagnostics of the current state (implies qgw_invert). */
int qgw_budget(qgw_run* run, qgw_budget_out* out);

/* Device bytes held by a run of these parameters (admission control). */
int qgw_footprint(const qgw_params* p, int precision, size_t* bytes);

/* Launch sequencing for measurement: the CUDA stream the run uses
 * (cudaStream_t as void*) and the number of kernels one step launches. */
void* qgw_stream(qgw_run* run);
int qgw_kernels_per_step(qgw_run* run);

/* Run nsteps steps with CUDA events between the four kernels of each step
 * and return each kernel's mean duration in ms: ms4[0] rows forward
 * (AB3 + projection + x-DST), ms4[1] columns (y-DST, Helmholtz divide,
 * inverse y-DST), ms4[2] rows inverse (x-DST + back-projection), ms4[3] RHS. */
int qgw_profile_kernels(qgw_run* run, int nsteps, float* ms4);

/* Work-tile shape of a run's step kernels (no counterpart in the
 * reference, which has no tiles): rhs_tile_rows, the RHS tile height (16 or
 * 32 rows); col_tile, columns per tile of the column transform (FP32: 8 or
 * 4, FP64: 4 or 2; a chirp-z NY keeps the width chosen at creation, 4 or 1
 * in FP32 and 2 or 1 in FP64); row_group_fwd and row_group_inv, modes (layers) per
 * block of the forward and inverse row kernels (1..16, balanced over the
 * run's layers; the inverse kernel takes at most 8 when it also transforms
 * zeta).  0 keeps a value.  No choice changes the arithmetic: a run's
 * results are bitwise the same for every shape.  QGW_ERR_PARAM when a value
 * is not one of these or the shape needs more shared memory than the
 * device has (the run keeps its shape). */
typedef struct {
  int rhs_tile_rows;
  int col_tile;
  int row_group_fwd;
  int row_group_inv;
} qgw_shape;
int qgw_set_shape(qgw_run* run, const qgw_shape* shape);
int qgw_get_shape(qgw_run* run, qgw_shape* shape);

/* PV inversion without any allocation (no counterpart in the reference,
 * whose invert_pv, src/elliptic.h:76-155, allocates nothing only because its
 * work array is a global made at start-up).  For callers that cannot
 * allocate device memory -- a host model whose memory manager owns every
 * device buffer, or a loop that must not call cudaMalloc/cudaFree, which
 * synchronise the device and can fail under memory pressure.  q_dev and
 * psi_dev are the caller's device arrays in the reference layout
 * (nl, NY+1, NX+1); on return (asynchronously, on `stream`) psi_dev holds
 * psi with a zero ghost ring and q_dev's ghost ring is set as invert_pv sets
 * it.  cl2m, cm2l, iRd2 are host arrays (e.g. from qgw_eigmode).  Scratch
 * is one file-scope device array of 32 MiB held by every GPU that loads the
 * library.  Accepted: closed basins (bc_fac >= 0; the periodic basin is
 * QGW_ERR_UNSUPPORTED here) on the half-length grids of the run path (NX,
 * NY even, NX/2 and NY/2 products of 2, 3, 5 and 7) with 4 <= NX, NY <= 1024, 1 <= nl <= 32
 * and nl*(NX+1)*(NY+1) <= 2097152; anything else returns
 * QGW_ERR_UNSUPPORTED.  A launch error already pending in the calling thread
 * makes the call return QGW_ERR_CUDA without clearing it.  The first call on
 * a device looks up the array's device address (with that device current)
 * and should come before any stream capture.  Calls share the array: calls
 * that overlap on the GPU, or come from several host threads at once, race. */
int qgw_invert_pv_noalloc(const qgw_params* p, const double* cl2m, const double* cm2l,
                          const double* iRd2, double* q_dev, double* psi_dev, void* stream);

/* Measured FMA throughput of the current device in TFLOP/s (FP64 and FP32,
 * independent FMA chains): the arithmetic roofs of the FP64 kernels. */
int qgw_probe_fp_rates(double* fp64_tflops, double* fp32_tflops);

/* ---- ensembles: many runs, one launch per step stage --------------------
 * Members may differ in grid size and layer count (one precision per
 * ensemble).  qgw_ensemble_step advances every member by up to nsteps steps
 * (max_steps[i] > 0 caps member i), each stage as one persistent launch
 * over all members' work items, the four launches of a step captured once
 * as a CUDA graph (use_graph != 0) and replayed.  A member's result is
 * bitwise the same alone and in any ensemble.  qgw_ensemble_tune chooses
 * the members' work-tile shape (RHS tile height, column-tile width, modes
 * per row-kernel block; qgw_set_shape) and then each stage's persistent
 * grid size, one choice at a time, timing whole steps for every candidate;
 * the trial steps advance the state, so set q afterwards.  No reference
 * counterpart: the reference runs one configuration per process. */
typedef struct qgw_ensemble qgw_ensemble;
int qgw_ensemble_create(int nmembers, const qgw_params* params, int precision, qgw_ensemble** out);
void qgw_ensemble_destroy(qgw_ensemble* ens);
int qgw_ensemble_size(qgw_ensemble* ens);
qgw_run* qgw_ensemble_member(qgw_ensemble* ens, int i);
int qgw_ensemble_set_q(qgw_ensemble* ens, int i, const double* q);
int qgw_ensemble_set_time(qgw_ensemble* ens, int i, const qgw_time* tm);
int qgw_ensemble_get(qgw_ensemble* ens, int i, double* psi, double* q);
int qgw_ensemble_step(qgw_ensemble* ens, int nsteps, const int* max_steps, int use_graph,
                      qgw_step_info* infos);
int qgw_ensemble_tune(qgw_ensemble* ens, int trial_steps, float* best_ms);
int qgw_ensemble_grids(qgw_ensemble* ens, int* blocks_per_sm);
/* qgw_set_shape for every member (one shape for the whole ensemble; the
 * member table is rebuilt), and member i's shape (the tuner's choice). */
int qgw_ensemble_set_shape(qgw_ensemble* ens, const qgw_shape* shape);
int qgw_ensemble_shape(qgw_ensemble* ens, int i, qgw_shape* shape);
/* qgw_set_forcing_records for member i (the member table is rebuilt). */
int qgw_ensemble_set_forcing_records(qgw_ensemble* ens, int i, const double* records, int nrec);

/* ---- serving: continuous batching on one GPU -----------------------------
 * Any thread submits requests (params, initial q in the reference layout,
 * precision, step count); a worker thread admits them in arrival order
 * while their device footprint fits the HBM budget (0: 80% of free memory),
 * keeps admitted runs resident, advances all resident runs by up to
 * steps_per_tick steps per tick (FP64 and FP32c batches on two streams), and
 * retires finished runs, freeing their memory for the next admission.  A
 * request whose footprint exceeds the budget finishes with
 * QGW_ERR_ADMISSION.  Results are bitwise those of the same run alone.
 * No reference counterpart: the reference runs one configuration per
 * process. */
typedef struct qgw_pool qgw_pool;
int qgw_pool_create(size_t hbm_budget_bytes, int steps_per_tick, qgw_pool** out);
int qgw_pool_submit(qgw_pool* pool, const qgw_params* p, const double* q0, int precision, int nsteps,
                    long long* id);
/* QGW_OK when request id has finished (its own status in *status), else
 * QGW_ERR_NOT_READY; blocks up to wait_ms. */
int qgw_pool_poll(qgw_pool* pool, long long id, int wait_ms, int* status);
/* Copy out and forget a finished request; latency[3] = seconds queued,
 * seconds resident, seconds from submit to result. */
int qgw_pool_fetch(qgw_pool* pool, long long id, double* psi, double* q, qgw_time* tm, double* latency);
/* stats[6]: completed, admitted, ticks, max resident, lgp-steps, bytes in use */
int qgw_pool_stats(qgw_pool* pool, double* stats);
void qgw_pool_destroy(qgw_pool* pool);

/* ---- netCDF-3 output and restart (host code, no netCDF library) --------
 * vars.nc as create_nc/write_nc write it (src/netcdf_io.h:38-277): dims
 * t (unlimited), level, y, x; float variables t, y, x, level, psi, q, the
 * fields including the wall ring.  qgw_nc_read replaces read_nc
 * (src/netcdf_io.h:286-382): record `rec` of a variable with `count` values
 * per record, e.g. "q" (nl*(NY+1)*(NX+1)) or "topo" ((NY+1)*(NX+1)); it
 * returns the number of values read or a negative status. */
typedef struct qgw_nc qgw_nc;
qgw_nc* qgw_nc_create(const char* path, int nl, int ny_out, int nx_out, double Delta);
int qgw_nc_write(qgw_nc* nc, double t, const double* psi, const double* q);
void qgw_nc_close(qgw_nc* nc);
long qgw_nc_read(const char* path, const char* name, int rec, double* out, long count);

const char* qgw_strerror(int status);
int qgw_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* QGW_GPU_H */
