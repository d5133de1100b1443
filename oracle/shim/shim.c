/*
 * shim.c -- project implementations of the FFTW / LAPACKE / netCDF calls the
 * reference makes, so that the reference's own src/qg.c can be compiled and
 * run in place as the oracle (test infrastructure only).
 *
 * FFTW: the closed-basin 2-D RODFT00 plans (src/elliptic.h:63-66), the
 * periodic in-place r2c/c2r plans (src/elliptic.h:32-47) and the
 * out-of-place c2r of the stochastic forcing (src/forcing.h:124).
 * The DST uses direct sums with an exactly reduced sine table unless
 * QGW_SHIM_DST=fast, which selects the O(n log n) path of oracle_math.c.
 */
#include "fftw3.h"
#include "lapacke.h"
#include "netcdf.h"
#include "../oracle_math.h"

#include <stdint.h>
#include <stdio.h>
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
/* netCDF: the writers return an error (the reference's output code prints
 * it and returns, src/netcdf_io.h:16); a reader of the classic format
 * (CDF-1 and CDF-2: the published file format) serves read_nc
 * (src/netcdf_io.h:286-382), i.e. the 4-D forcing's input_vars.nc and the
 * restart file.  Float and double variables; record variables along the
 * unlimited dimension. */
int nc_create(const char* path, int cmode, int* ncidp) { (void)path; (void)cmode; (void)ncidp; return SHIM_NC_ERR; }
int nc_def_dim(int ncid, const char* name, size_t len, int* idp) { (void)ncid; (void)name; (void)len; (void)idp; return SHIM_NC_ERR; }
int nc_def_var(int ncid, const char* name, nc_type xtype, int ndims, const int* dimidsp, int* varidp) {
  (void)ncid; (void)name; (void)xtype; (void)ndims; (void)dimidsp; (void)varidp; return SHIM_NC_ERR;
}
int nc_enddef(int ncid) { (void)ncid; return SHIM_NC_ERR; }
int nc_put_var_float(int ncid, int varid, const float* op) { (void)ncid; (void)varid; (void)op; return SHIM_NC_ERR; }
int nc_put_vara_float(int ncid, int varid, const size_t* s, const size_t* c, const float* op) {
  (void)ncid; (void)varid; (void)s; (void)c; (void)op; return SHIM_NC_ERR;
}

#define SHIM_NC_MAXF 4
#define SHIM_NC_MAXD 16
#define SHIM_NC_MAXV 32
typedef struct {
  char name[NC_MAX_NAME + 1];
  int ndims, dimids[SHIM_NC_MAXD], type;
  long long vsize, begin;
} shim_ncvar;
typedef struct {
  FILE* f;
  int ndims, nvars, unlim;
  long long dimlen[SHIM_NC_MAXD], recsize, numrecs;
  shim_ncvar var[SHIM_NC_MAXV];
} shim_ncfile;
static shim_ncfile shim_nc[SHIM_NC_MAXF];

static int nc_rd32(FILE* f, long long* v) {
  unsigned char b[4];
  if (fread(b, 1, 4, f) != 4) return -1;
  *v = (long long)(((unsigned)b[0] << 24) | ((unsigned)b[1] << 16) | ((unsigned)b[2] << 8) | b[3]);
  return 0;
}
static int nc_rd64(FILE* f, long long* v) {
  long long hi, lo;
  if (nc_rd32(f, &hi) || nc_rd32(f, &lo)) return -1;
  *v = (hi << 32) | lo;
  return 0;
}
static int nc_rdname(FILE* f, char* out) {
  long long n;
  if (nc_rd32(f, &n) || n < 0 || n > NC_MAX_NAME) return -1;
  char buf[NC_MAX_NAME + 4];
  const long long padded = (n + 3) / 4 * 4;
  if (fread(buf, 1, (size_t)padded, f) != (size_t)padded) return -1;
  memcpy(out, buf, (size_t)n);
  out[n] = 0;
  return 0;
}
static int nc_tsize(int t) { return t == 1 || t == 2 ? 1 : t == 3 ? 2 : t == 6 ? 8 : 4; }
static int nc_skip_atts(FILE* f) {
  long long tag, n;
  if (nc_rd32(f, &tag) || nc_rd32(f, &n)) return -1;
  for (long long a = 0; a < n; ++a) {
    char name[NC_MAX_NAME + 1];
    long long t, m;
    if (nc_rdname(f, name) || nc_rd32(f, &t) || nc_rd32(f, &m)) return -1;
    if (fseek(f, (long)((m * nc_tsize((int)t) + 3) / 4 * 4), SEEK_CUR)) return -1;
  }
  return 0;
}

int nc_open(const char* path, int mode, int* ncidp) {
  (void)mode;
  int id = -1;
  for (int i = 0; i < SHIM_NC_MAXF; ++i) if (!shim_nc[i].f) { id = i; break; }
  if (id < 0) return SHIM_NC_ERR;
  shim_ncfile* nf = &shim_nc[id];
  memset(nf, 0, sizeof(*nf));
  nf->unlim = -1;
  FILE* f = fopen(path, "rb");
  if (!f) return SHIM_NC_ERR;
  unsigned char magic[4];
  long long tag, n;
  if (fread(magic, 1, 4, f) != 4 || memcmp(magic, "CDF", 3) || (magic[3] != 1 && magic[3] != 2)) goto fail;
  const int v2 = magic[3] == 2;
  if (nc_rd32(f, &nf->numrecs) || nc_rd32(f, &tag) || nc_rd32(f, &n) || n > SHIM_NC_MAXD) goto fail;
  nf->ndims = (int)n;
  for (int d = 0; d < nf->ndims; ++d) {
    char name[NC_MAX_NAME + 1];
    if (nc_rdname(f, name) || nc_rd32(f, &nf->dimlen[d])) goto fail;
    if (nf->dimlen[d] == 0) nf->unlim = d;
  }
  if (nc_skip_atts(f)) goto fail;
  if (nc_rd32(f, &tag) || nc_rd32(f, &n) || n > SHIM_NC_MAXV) goto fail;
  nf->nvars = (int)n;
  for (int v = 0; v < nf->nvars; ++v) {
    shim_ncvar* var = &nf->var[v];
    long long nd, t;
    if (nc_rdname(f, var->name) || nc_rd32(f, &nd) || nd > SHIM_NC_MAXD) goto fail;
    var->ndims = (int)nd;
    for (int d = 0; d < var->ndims; ++d) {
      long long di;
      if (nc_rd32(f, &di)) goto fail;
      var->dimids[d] = (int)di;
    }
    if (nc_skip_atts(f) || nc_rd32(f, &t) || nc_rd32(f, &var->vsize)) goto fail;
    var->type = (int)t;
    if (v2 ? nc_rd64(f, &var->begin) : nc_rd32(f, &var->begin)) goto fail;
    if (var->ndims > 0 && var->dimids[0] == nf->unlim) nf->recsize += var->vsize;
  }
  nf->f = f;
  *ncidp = id;
  return 0;
fail:
  fclose(f);
  return SHIM_NC_ERR;
}

int nc_close(int ncid) {
  if (ncid < 0 || ncid >= SHIM_NC_MAXF || !shim_nc[ncid].f) return SHIM_NC_ERR;
  fclose(shim_nc[ncid].f);
  shim_nc[ncid].f = NULL;
  return 0;
}

int nc_inq(int ncid, int* a, int* b, int* c, int* d) {
  if (ncid < 0 || ncid >= SHIM_NC_MAXF || !shim_nc[ncid].f) return SHIM_NC_ERR;
  if (a) *a = shim_nc[ncid].ndims;
  if (b) *b = shim_nc[ncid].nvars;
  if (c) *c = 0;
  if (d) *d = shim_nc[ncid].unlim;
  return 0;
}

int nc_inq_var(int ncid, int varid, char* name, nc_type* t, int* nd, int* di, int* na) {
  if (ncid < 0 || ncid >= SHIM_NC_MAXF || !shim_nc[ncid].f || varid < 0 || varid >= shim_nc[ncid].nvars)
    return SHIM_NC_ERR;
  const shim_ncvar* v = &shim_nc[ncid].var[varid];
  if (name) strcpy(name, v->name);
  if (t) *t = v->type;
  if (nd) *nd = v->ndims;
  if (di) for (int d = 0; d < v->ndims; ++d) di[d] = v->dimids[d];
  if (na) *na = 0;
  return 0;
}

/* big-endian float or double element at byte offset off, as float */
static int nc_rdval(FILE* f, long long off, int type, float* out) {
  unsigned char b[8];
  const int sz = nc_tsize(type);
  if (fseek(f, (long)off, SEEK_SET) || fread(b, 1, (size_t)sz, f) != (size_t)sz) return -1;
  if (type == NC_FLOAT) {
    uint32_t u = ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | b[3];
    memcpy(out, &u, 4);
  } else if (type == NC_DOUBLE) {
    uint64_t u = 0;
    for (int i = 0; i < 8; ++i) u = (u << 8) | b[i];
    double d;
    memcpy(&d, &u, 8);
    *out = (float)d;
  } else {
    return -1;
  }
  return 0;
}

int nc_get_vara_float(int ncid, int varid, const size_t* start, const size_t* count, float* ip) {
  if (ncid < 0 || ncid >= SHIM_NC_MAXF || !shim_nc[ncid].f || varid < 0 || varid >= shim_nc[ncid].nvars)
    return SHIM_NC_ERR;
  shim_ncfile* nf = &shim_nc[ncid];
  const shim_ncvar* v = &nf->var[varid];
  const int rec = v->ndims > 0 && v->dimids[0] == nf->unlim;
  long long len[SHIM_NC_MAXD], stride[SHIM_NC_MAXD];
  for (int d = 0; d < v->ndims; ++d) len[d] = nf->dimlen[v->dimids[d]];
  if (rec) len[0] = nf->numrecs;
  for (int d = 0; d < v->ndims; ++d)
    if ((long long)(start[d] + count[d]) > len[d]) return SHIM_NC_ERR;
  /* element strides (in elements) within one record / the whole variable */
  long long st = 1;
  for (int d = v->ndims - 1; d >= (rec ? 1 : 0); --d) { stride[d] = st; st *= len[d]; }
  long long total = 1;
  for (int d = 0; d < v->ndims; ++d) total *= (long long)count[d];
  long long idx[SHIM_NC_MAXD] = {0};
  const int esz = nc_tsize(v->type);
  for (long long e = 0; e < total; ++e) {
    long long off = v->begin;
    for (int d = 0; d < v->ndims; ++d) {
      const long long c = (long long)start[d] + idx[d];
      if (rec && d == 0) off += c * nf->recsize;
      else off += c * stride[d] * esz;
    }
    if (nc_rdval(nf->f, off, v->type, ip + e)) return SHIM_NC_ERR;
    for (int d = v->ndims - 1; d >= 0; --d) {
      if (++idx[d] < (long long)count[d]) break;
      idx[d] = 0;
    }
  }
  return 0;
}
const char* nc_strerror(int ncerr) { (void)ncerr; return "netCDF is not available in the oracle build"; }
