/*
 * qgw_port.h -- CPU restatement of the reference's time step (ORACLE: test
 * infrastructure only; used by tests/, the smoke check and bench.py's CPU
 * baseline, never by the product library).
 *
 * State is held in a struct instead of globals; arrays use the reference
 * layout (nl, ny+2, nx+2) with the ghost ring, idx() of src/domain.h:62.
 */
#ifndef QGW_PORT_H
#define QGW_PORT_H

#include "../include/qgw_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct port_run port_run;

void port_params_default(qgw_params* p);
int port_params_read(qgw_params* p, const char* path);

/* fast_dst: 1 = O(n log n) DST (n+1 a power of two), 0 = direct sums. */
port_run* port_create(const qgw_params* p, int fast_dst);
void port_destroy(port_run* r);

void port_sizes(const port_run* r, int* nx, int* ny, int* nl);
void port_set_q(port_run* r, const double* q);
/* the 4-D forcing's records: nrec fields in the reference layout */
void port_set_forcing_records(port_run* r, const double* rec, int nrec);
void port_set_topo(port_run* r, const double* topo);
void port_get(const port_run* r, double* psi, double* q);
void port_get_modes(const port_run* r, double* cl2m, double* cm2l, double* iRd2);
void port_get_time(const port_run* r, qgw_time* tm, double* t_out);
void port_set_time(port_run* r, const qgw_time* tm, double t_out);

void port_invert(port_run* r);                     /* invert_pv(q, psi)   */
void port_timestep(port_run* r);                   /* timestep(q)         */
/* Driver loop of src/qg.c:181-199 without file output: before each step,
 * stop if t >= tend (tend > 0) and advance t_out by dt_out when t hits it.
 * snap = 0 skips the t_out bookkeeping (fixed-dt harness mode).  Returns
 * the number of steps taken. */
int port_run_steps(port_run* r, int nsteps, int snap);

/* DST-I of howmany contiguous rows of length n (pin test entry point). */
void port_dst1(int n, int howmany, double* data, int fast);

#ifdef __cplusplus
}
#endif
#endif
