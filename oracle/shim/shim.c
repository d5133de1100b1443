/*
 * shim.c -- project implementations of the FFTW / LAPACKE / netCDF calls the
 * reference makes, so that the reference's own src/qg.c can be compiled and
 * run in place as the oracle (test infrastructure only).
 *
 * FFTW: the closed-basin 2-D RODFT00 plan (src/elliptic.h:136-139), the
 * periodic in-place r2c/c2r plans (src/elliptic.h:32-47) and the
 * out-of-place c2r of the stochastic forcing (src/forcing.h:124).
 * The DST uses direct sums with an exactly reduced sine table unless
 * QGW_SHIM_DST=fast, which selects the O(n log n) path of oracle_math.c.
 */
#include "fftw3.h"
#include "lapacke.h"
#include "netcdf.h"
#include "../oracle_math.h"

#include <stdlib.h>
#include <string.h>

struct shim_fftw_plan_s {
  int n0, n1;
  int kind;  /* 0 RODFT00 2-D, 1 r2c 2-D in place, 2 c2r 2-D in place, 3 c2r 2-D out of place */
  double *in, *out;
};

static int shim_fast(void) {
  const char* e = getenv("QGW_SHIM_DST");
  return e && !strcmp(e, "fast");
}

fftw_plan fftw_plan_r2r_2d(int n0, int n1, double* in, double* out,
                           fftw_r2r_kind kind0, fftw_r2r_kind kind1, unsigned flags) {
  (void)flags;
  if (kind0 != FFTW_RODFT00 || kind1 != FFTW_RODFT00) return NULL;
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  p->n0 = n0; p->n1 = n1; p->in = in; p->out = out;
  return p;
}

/* in-place plans only, as the reference makes them */
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags) {
  (void)flags;
  if ((void*)in != (void*)out) return NULL;
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  p->n0 = n0; p->n1 = n1; p->kind = 1; p->in = in; p->out = in;
  return p;
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  p->n0 = n0; p->n1 = n1; p->in = (double*)in; p->out = out;
  p->kind = ((void*)in == (void*)out) ? 2 : 3;
  return p;
}

void fftw_execute(const fftw_plan p) {
  if (!p) return;
  if (p->kind == 1) { om_dft_r2c_2d_any(p->n0, p->n1, p->out, shim_fast()); return; }
  if (p->kind == 2) { om_dft_c2r_2d_any(p->n0, p->n1, p->out, shim_fast()); return; }
  if (p->kind == 3) {
    /* input n0 x (n1/2+1) complex, output n0 x n1 reals: run in place on a
     * copy with the padded row layout, then pack the rows */
    const size_t ld = 2 * (size_t)(p->n1 / 2 + 1);
    double* t = (double*)malloc(sizeof(double) * ld * (size_t)p->n0);
    memcpy(t, p->in, sizeof(double) * ld * (size_t)p->n0);
    om_dft_c2r_2d_any(p->n0, p->n1, t, shim_fast());
    for (int r = 0; r < p->n0; ++r) memcpy(p->out + (size_t)r * p->n1, t + (size_t)r * ld, sizeof(double) * (size_t)p->n1);
    free(t);
    return;
  }
  if (p->in != p->out) memcpy(p->out, p->in, sizeof(double) * (size_t)p->n0 * p->n1);
  om_dst2(p->n0, p->n1, p->out, shim_fast());
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
void fftw_cleanup(void) {}
double* fftw_alloc_real(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }
fftw_complex* fftw_alloc_complex(size_t n) { return (fftw_complex*)calloc(n ? n : 1, sizeof(fftw_complex)); }
void fftw_free(void* p) { free(p); }

lapack_int LAPACKE_dgeev(int matrix_layout, char jobvl, char jobvr, lapack_int n,
                         double* a, lapack_int lda, double* wr, double* wi,
                         double* vl, lapack_int ldvl, double* vr, lapack_int ldvr) {
  (void)jobvl; (void)jobvr;
  if (matrix_layout != LAPACK_ROW_MAJOR || n < 1) return -1;
  double* ac = (double*)malloc(sizeof(double) * (size_t)n * n);
  double* l = (double*)malloc(sizeof(double) * (size_t)n * n);
  double* r = (double*)malloc(sizeof(double) * (size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) ac[i * n + j] = a[(size_t)i * lda + j];
  int rc = om_tridiag_eig(n, ac, wr, l, r);
  if (rc == 0) {
    for (int i = 0; i < n; ++i) {
      wi[i] = 0.0;
      for (int j = 0; j < n; ++j) {
        vl[(size_t)i * ldvl + j] = l[i * n + j];
        vr[(size_t)i * ldvr + j] = r[i * n + j];
      }
    }
  }
  free(ac); free(l); free(r);
  return rc == 0 ? 0 : -1;
}

#define SHIM_NC_ERR (-1)
int nc_create(const char* path, int cmode, int* ncidp) { (void)path; (void)cmode; (void)ncidp; return SHIM_NC_ERR; }
int nc_open(const char* path, int mode, int* ncidp) { (void)path; (void)mode; (void)ncidp; return SHIM_NC_ERR; }
int nc_def_dim(int ncid, const char* name, size_t len, int* idp) { (void)ncid; (void)name; (void)len; (void)idp; return SHIM_NC_ERR; }
int nc_def_var(int ncid, const char* name, nc_type xtype, int ndims, const int* dimidsp, int* varidp) {
  (void)ncid; (void)name; (void)xtype; (void)ndims; (void)dimidsp; (void)varidp; return SHIM_NC_ERR;
}
int nc_enddef(int ncid) { (void)ncid; return SHIM_NC_ERR; }
int nc_close(int ncid) { (void)ncid; return SHIM_NC_ERR; }
int nc_put_var_float(int ncid, int varid, const float* op) { (void)ncid; (void)varid; (void)op; return SHIM_NC_ERR; }
int nc_put_vara_float(int ncid, int varid, const size_t* s, const size_t* c, const float* op) {
  (void)ncid; (void)varid; (void)s; (void)c; (void)op; return SHIM_NC_ERR;
}
int nc_get_vara_float(int ncid, int varid, const size_t* s, const size_t* c, float* ip) {
  (void)ncid; (void)varid; (void)s; (void)c; (void)ip; return SHIM_NC_ERR;
}
int nc_inq(int ncid, int* a, int* b, int* c, int* d) { (void)ncid; (void)a; (void)b; (void)c; (void)d; return SHIM_NC_ERR; }
int nc_inq_var(int ncid, int varid, char* name, nc_type* t, int* nd, int* di, int* na) {
  (void)ncid; (void)varid; (void)name; (void)t; (void)nd; (void)di; (void)na; return SHIM_NC_ERR;
}
const char* nc_strerror(int ncerr) { (void)ncerr; return "netCDF is not available in the oracle build"; }
