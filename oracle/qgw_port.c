/*
 * qgw_port.c -- CPU restatement of the reference's time step, FP64, single
 * thread (ORACLE: test infrastructure only; see qgw_port.h).
 *
 * Each function names the reference lines it restates.  Loop order and the
 * order of floating-point operations follow the reference, so that the port
 * agrees with the reference compiled in place to round-off; the only
 * difference is the DST, which the reference takes from FFTW (not available
 * here) and the port computes with oracle_math.c.
 */
#include "qgw_port.h"
#include "oracle_math.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const double PORT_PI = 3.141592653589793;  /* src/qg.c:44 */
static const double PORT_TEPS = 1e-9;            /* src/timestep.h:16 */
static const double PORT_HUGE = 1e30;            /* src/qg.c:43 */

struct port_run {
  qgw_params p;
  int nx, ny, nl, nxp2, nyp2;
  double Delta, Ly, norm, nu_hyper;
  double *q, *psi, *diff, *lapn, *topo, *fab[3];
  double *wrk, *cl2m, *cm2l, *iRd2, *K, *L, *X, *Y;
  double t, dt, dt0, dt1, DT_max, t_out;
  int fast;
  /* stochastic ring forcing (src/forcing.h:11-30,67-201) */
  double kf;               /* k_f / (2 pi) */
  int NF, NKf, NP, Np;     /* transform size, half size, ring points */
  int *ind_i, *ind_j;
  double *forc, *forc_f, *forc_p;
  /* 4-D forcing records (src/forcing.h:33-43,226-288): n_rec fields of the
   * reference layout, as read_nc loads them from input_vars.nc */
  int nrec;
  double* frec;
};

#define IDX(r, i, j, k) ((size_t)(k) * (r)->nxp2 * (r)->nyp2 + (size_t)(j) * (r)->nxp2 + (size_t)(i))
static double sq(double x) { return x * x; }
static void port_init_forcing(port_run* r);

/* ------------------------------------------------------------- params */

/* Defaults: src/qg.c:57-83, src/forcing.h:13-14,38-39. */
void port_params_default(qgw_params* p) {
  memset(p, 0, sizeof(*p));
  p->nl = 1;
  p->dh[0] = 1.0;
  p->N2[0] = 1.0;
  p->tend = 1.0;
  p->dt_out = 0.1;
  p->cfl = 0.2;
  p->forc_mode = 1.0;
  p->f0 = 1.e-5;
  p->w_topo = 1.0;
  p->sigma_f = 1.0;
}

/* read_params / str2array / trim_whitespace, src/extra.h:26-33,98-153. */
static void port_trim(char* s) {
  char* d = s;
  for (char* c = s; *c; ++c) if (*c != ' ') *d++ = *c;
  *d = 0;
}

static void port_str2array(char* v, double* a, int cap) {
  char* nl = strchr(v, '\n');
  if (nl) *nl = 0;
  int n = 0;
  char* tok = strtok(v, "[,]");
  while (tok) {
    if (n < cap) a[n] = atof(tok);
    ++n;
    tok = strtok(NULL, ",");
  }
}

int port_params_read(qgw_params* p, const char* path) {
  FILE* fp = fopen(path, "rt");
  if (!fp) return QGW_ERR_FILE;
  char line[300];
  while (fgets(line, sizeof line, fp)) {
    port_trim(line);
    char* key = strtok(line, "=");
    char* val = strtok(NULL, "=");
    if (!key) continue;
#define PINT(name) if (!strcmp(key, #name)) { p->name = atoi(val ? val : ""); continue; }
#define PDBL(name) if (!strcmp(key, #name)) { p->name = atof(val ? val : ""); continue; }
#define PARR(name) if (!strcmp(key, #name)) { if (val) port_str2array(val, p->name, QGW_NL_MAX); continue; }
    PINT(NX) PINT(NY) PINT(nl) PINT(n_hyper) PDBL(Lx) PARR(dh) PDBL(tau0)
    PDBL(forc_mode) PDBL(f0) PDBL(beta) PDBL(nu) PDBL(nu_hyper) PDBL(hEkb)
    PARR(N2) PDBL(Ld) PDBL(h_topo) PDBL(w_topo) PDBL(bc_fac) PDBL(tend)
    PDBL(dt_out) PDBL(dt_forc) PDBL(dt_forc_period) PDBL(sigma_f) PDBL(k_f)
    PDBL(cfl) PDBL(dt)
#undef PINT
#undef PDBL
#undef PARR
  }
  fclose(fp);
  return 0;
}

/* ------------------------------------------------------------ eigmode */

/* compute_eigmode, src/eigmode.h:87-271 (dgeev replaced by om_tridiag_eig). */
static int port_eigmode(port_run* r) {
  const int nl = r->nl;
  const qgw_params* p = &r->p;
  double dhc[QGW_NL_MAX];
  for (int l = 0; l < nl - 1; ++l) dhc[l] = 0.5 * (p->dh[l] + p->dh[l + 1]);
  double htotal = 0;
  for (int k = 0; k < nl; ++k) htotal += p->dh[k];
  double* G = (double*)calloc((size_t)nl * nl, sizeof(double));
  if (nl > 1) {
    int l = 0;
    G[nl * l + l + 1] = -sq(p->f0) / p->N2[l] / (dhc[l] * p->dh[l]);
    G[nl * l + l] = -G[nl * l + l + 1];
    for (l = 1; l < nl - 1; ++l) {
      G[nl * l + l - 1] = -sq(p->f0) / p->N2[l - 1] / (dhc[l - 1] * p->dh[l]);
      G[nl * l + l + 1] = -sq(p->f0) / p->N2[l] / (dhc[l] * p->dh[l]);
      G[nl * l + l] = -G[nl * l + l - 1] - G[nl * l + l + 1];
    }
    l = nl - 1;
    G[nl * l + l - 1] = -sq(p->f0) / p->N2[l - 1] / (dhc[l - 1] * p->dh[l]);
    G[nl * l + l] = -G[nl * l + l - 1];
  } else {
    G[0] = 1.0;
  }
  double *wr = malloc(sizeof(double) * nl), *vl = malloc(sizeof(double) * nl * nl),
         *vr = malloc(sizeof(double) * nl * nl), *tmp = malloc(sizeof(double) * nl * nl);
  int* order = malloc(sizeof(int) * nl);
  int rc = om_tridiag_eig(nl, G, wr, vl, vr);
  if (rc == 0) {
    /* ascending sort of eigenvalues carrying the vectors (stable insertion) */
    for (int m = 0; m < nl; ++m) order[m] = m;
    for (int a = 1; a < nl; ++a) {
      int v = order[a], b = a - 1;
      while (b >= 0 && wr[order[b]] > wr[v]) { order[b + 1] = order[b]; --b; }
      order[b + 1] = v;
    }
    double* ws = malloc(sizeof(double) * nl);
    for (int m = 0; m < nl; ++m) ws[m] = wr[order[m]];
    memcpy(tmp, vr, sizeof(double) * nl * nl);
    for (int m = 0; m < nl; ++m)
      for (int k = 0; k < nl; ++k) vr[k * nl + m] = tmp[k * nl + order[m]];
    memcpy(tmp, vl, sizeof(double) * nl * nl);
    for (int m = 0; m < nl; ++m)
      for (int k = 0; k < nl; ++k) vl[k * nl + m] = tmp[k * nl + order[m]];
    /* Flierl (1978) normalisation, surface-positive (src/eigmode.h:205-214) */
    for (int m = 0; m < nl; ++m) {
      double dotp = 0.0;
      for (int k = 0; k < nl; ++k) dotp += p->dh[k] * vr[k * nl + m] * vr[k * nl + m];
      double flfac = (vr[m] > 0 ? 1 : -1) * sqrt(htotal / dotp);
      for (int k = 0; k < nl; ++k) vr[k * nl + m] = flfac * vr[k * nl + m];
    }
    /* left vectors dual to the right ones (src/eigmode.h:215-223) */
    for (int m = 0; m < nl; ++m) {
      double dotp = 0.0;
      for (int k = 0; k < nl; ++k) dotp += vr[k * nl + m] * vl[k * nl + m];
      for (int k = 0; k < nl; ++k) vl[k * nl + m] = vl[k * nl + m] / dotp;
    }
    for (int m = 0; m < nl; ++m)
      for (int k = 0; k < nl; ++k) {
        r->cl2m[k * nl + m] = vl[m * nl + k];
        r->cm2l[k * nl + m] = vr[k * nl + m];
      }
    for (int k = 1; k < nl; ++k) r->iRd2[k] = ws[k];
    r->iRd2[0] = 0.0;
    if (nl == 1 && p->Ld != 0) r->iRd2[0] = 1 / sq(p->Ld);
    free(ws);
  }
  free(G); free(wr); free(vl); free(vr); free(tmp); free(order);
  return rc;
}

/* ------------------------------------------------------------- set-up */

/* check_timestep, src/timestep.h:18-54, with the unparenthesised min/max
 * macros of src/qg.c:40-41: max(max(a,b),c) is (a<b) ? b : (a<c ? c : a)
 * and 1e-3*min(A,B) is (1e-3*A > B) ? B : A. */
static void port_check_timestep(port_run* r) {
  const qgw_params* p = &r->p;
  double a = r->nu_hyper * 20. / pow(p->Lx / r->nx, p->n_hyper);
  double b = p->nu * 20. / pow(p->Lx / r->nx, 2);
  double c = 2. * p->beta * p->Lx;
  double mx = (a < b) ? b : ((a < c) ? c : a);
  r->DT_max = pow(mx, -1.);
  double dt = 0.0; /* the reference's global dt starts at 0 (src/qg.c:64) */
  if (p->tau0 != 0 && p->sigma_f != 0) {
    double A = sqrt(p->cfl * r->Delta / (p->tau0 / p->dh[0] * p->forc_mode * PORT_PI / r->Ly * r->Ly));
    double B = pow(sq(r->Delta * p->cfl) / p->sigma_f, 1. / 3.);
    dt = (1e-3 * A > B) ? B : A;
  } else if (p->tau0 != 0 && p->sigma_f == 0) {
    dt = 1e-3 * sqrt(p->cfl * r->Delta / (p->tau0 / p->dh[0] * p->forc_mode * PORT_PI / r->Ly * r->Ly));
  } else if (p->tau0 == 0 && p->sigma_f != 0) {
    dt = 1e-3 * pow(sq(r->Delta * p->cfl) / p->sigma_f, 1. / 3.);
  }
  if (r->DT_max != 0 && dt > r->DT_max) dt = r->DT_max;
  r->dt = dt;
}

port_run* port_create(const qgw_params* pin, int fast_dst) {
  port_run* r = (port_run*)calloc(1, sizeof(port_run));
  r->p = *pin;
  r->fast = fast_dst;
  const qgw_params* p = &r->p;
  /* init_domain, src/domain.h:64-176 (serial, bounded or periodic sizes) */
  r->Delta = p->Lx / p->NX;
  r->Ly = p->NY * r->Delta;
  r->nx = p->NX;
  r->ny = p->NY;
  if (p->bc_fac >= 0) { r->nx -= 1; r->ny -= 1; }
  r->nl = p->nl;
  r->nxp2 = r->nx + 2;
  r->nyp2 = r->ny + 2;
  r->X = calloc(r->nxp2, sizeof(double));
  r->Y = calloc(r->nyp2, sizeof(double));
  r->K = calloc(r->nyp2 > r->nxp2 ? r->nyp2 : r->nxp2, sizeof(double));
  r->L = calloc(r->nxp2, sizeof(double));
  const int periodic = p->bc_fac == -1;
  /* periodic: the zero of X and Y is at the second grid point (:144-148) */
  const int off = periodic ? -1 : 0;
  for (int i = 0; i < r->nxp2; ++i) r->X[i] = (i + off) * r->Delta;
  for (int j = 0; j < r->nyp2; ++j) r->Y[j] = (j + off) * r->Delta;
  if (periodic) {
    /* src/domain.h:163-168 (serial: K0 = 0, Nk = NXp2/2) */
    for (int j = 0; j < r->nx; ++j) r->L[j] = 2 * PORT_PI / p->Lx * (((j + r->nx / 2) % r->nx) - r->nx / 2);
    for (int i = 0; i < (r->nx + 2) / 2; ++i) r->K[i] = 2 * PORT_PI * i / p->Lx;
  } else {
    for (int j = 1; j < r->ny + 1; ++j) r->K[j] = PORT_PI * j / p->Lx;
    for (int i = 1; i < r->nx + 1; ++i) r->L[i] = PORT_PI * i / p->Lx;
  }
  /* init_elliptic, src/elliptic.h:29-74: periodic rows of Nx+2 doubles
   * (the in-place r2c layout), bounded rows of Nx */
  r->norm = periodic ? (double)p->NX * p->NY : 4.0 * (r->nx + 1) * (r->ny + 1);
  r->wrk = calloc((size_t)(r->nx + 2) * r->ny, sizeof(double));
  r->cl2m = calloc((size_t)r->nl * r->nl, sizeof(double));
  r->cm2l = calloc((size_t)r->nl * r->nl, sizeof(double));
  r->iRd2 = calloc(r->nl, sizeof(double));
  port_eigmode(r);
  /* init_vars, src/domain.h:178-212 */
  const size_t n3 = (size_t)r->nxp2 * r->nyp2 * r->nl;
  r->psi = calloc(n3, sizeof(double));
  r->q = calloc(n3, sizeof(double));
  r->diff = calloc(n3, sizeof(double));
  r->lapn = calloc(n3, sizeof(double));
  r->topo = calloc((size_t)r->nxp2 * r->nyp2, sizeof(double));
  for (int j = 0; j < r->nyp2; ++j)
    for (int i = 0; i < r->nxp2; ++i) {
#define SHELF(x, d) (1 - exp(-sq(x) / (2 * sq(d))))
      r->topo[IDX(r, i, j, 0)] = p->h_topo * (1 - SHELF(r->X[i], p->w_topo) * SHELF(p->Lx - r->X[i], p->w_topo) *
                                                  SHELF(r->Y[j], p->w_topo) * SHELF(r->Ly - r->Y[j], p->w_topo));
#undef SHELF
    }
  r->nu_hyper = pow(-1, p->n_hyper / 2 - 1) * fabs(p->nu_hyper);
  /* init_timestep, src/timestep.h:56-67 */
  for (int s = 0; s < 3; ++s) r->fab[s] = calloc(n3, sizeof(double));
  port_check_timestep(r);
  r->dt0 = r->dt;
  r->dt1 = r->dt;
  r->t = 0;
  r->t_out = 0;
  port_init_forcing(r);
  srand(1); /* the sequence a fresh reference process draws from */
  return r;
}

/* init_stoch_forc, src/forcing.h:67-168 (serial): the thin ring of
 * wavenumbers |k| ~ k_f (in cycles per unit length, dk = 1/Lx) of the
 * N_F x (N_F/2+1) half spectrum, N_F = NX (the unreduced grid size). */
static void port_init_forcing(port_run* r) {
  const qgw_params* p = &r->p;
  if (p->k_f == 0) return;
  r->kf = p->k_f / (2 * PORT_PI);
  /* N_F = NX (periodic) or NXp1, which after init_domain's NX -= 1 is the
   * unreduced NX as well (src/forcing.h:78-82) */
  r->NF = p->NX;
  r->NKf = r->NF / 2 + 1;
  r->forc = calloc((size_t)r->nxp2 * r->nyp2, sizeof(double));
  r->forc_f = calloc((size_t)2 * r->NKf * r->NF, sizeof(double));
  r->forc_p = calloc((size_t)r->NF * r->NF, sizeof(double));
  const double dk = 1. / p->Lx;
  /* room for every entry of the half spectrum (the reference sizes these
   * 4 pi k_f / dk, src/forcing.h:131-133, which the ring never exceeds in
   * the configurations tested) */
  const int N_ind = r->NF * r->NKf;
  r->ind_i = calloc(N_ind, sizeof(int));
  r->ind_j = calloc(N_ind, sizeof(int));
  r->NP = 0;
  r->Np = 0;
  for (int j = 0; j < r->NF; j++)
    for (int i = 0; i < r->NKf; i++) {
      double l = (((j + r->NF / 2) % r->NF) - r->NF / 2) * dk;
      double k = (i)*dk;
      double dist_k = fabs(k - sqrt(sq(r->kf) - sq(l)));
      double a = fabs(l - sqrt(sq(r->kf) - sq(k))), b = fabs(l + sqrt(sq(r->kf) - sq(k)));
      double dist_l = (a < b) ? a : b; /* the min macro of src/qg.c:40 */
      if (dist_k < dk / 2 || dist_l < dk / 2) {
        r->NP += 1;
        if (r->Np < N_ind) {
          r->ind_i[r->Np] = i;
          r->ind_j[r->Np] = j;
        }
        r->Np += 1;
      }
    }
}

/* calc_forc, src/forcing.h:170-201, with normal_noise / noise of :62-63;
 * rand() is the C library's (seeded at port_create, like a fresh reference
 * process).  C leaves the order of the two rand() calls of normal_noise
 * unspecified; the reference compiled in place (gcc) makes the logarithm's
 * first, which the golden fixtures pin (bit-identical results). */
static void port_calc_forc(port_run* r) {
  if (r->NP <= 1) return;
  memset(r->forc_f, 0, sizeof(double) * 2 * (size_t)r->NKf * r->NF);
  for (int ii = 0; ii < r->Np; ii++) {
    const int i = r->ind_i[ii], j = r->ind_j[ii];
    const double envelope = sqrt((double)8 / ((r->NP - 1) * 2)) * PORT_PI * r->kf;
    const double rl = (double)rand(); /* log argument */
    const double rc = (double)rand(); /* cos argument */
    const double nn = sqrt(-2. * log((rl + 1.) / ((double)(RAND_MAX) + 2.))) * cos(2 * PORT_PI * rc / (double)RAND_MAX);
    const double magnitude = r->p.sigma_f * nn;
    const double phase = ((double)rand() / RAND_MAX) * 2 * PORT_PI;
    r->forc_f[2 * ((size_t)j * r->NKf + i)] = envelope * magnitude * cos(phase);
    r->forc_f[2 * ((size_t)j * r->NKf + i) + 1] = envelope * magnitude * sin(phase);
  }
  /* out-of-place c2r of the N_F x N_F plan */
  const size_t ld = 2 * (size_t)r->NKf;
  double* t = malloc(sizeof(double) * ld * r->NF);
  memcpy(t, r->forc_f, sizeof(double) * ld * r->NF);
  om_dft_c2r_2d_any(r->NF, r->NF, t, r->fast);
  for (int j = 0; j < r->NF; j++)
    for (int i = 0; i < r->NF; i++) r->forc_p[(size_t)j * r->NF + i] = t[(size_t)j * ld + i];
  free(t);
  for (int j = 0; j < r->NF; j++)
    for (int i = 0; i < r->NF; i++)
      if (i + 1 < r->nxp2 && j + 1 < r->nyp2) r->forc[IDX(r, i + 1, j + 1, 0)] = r->forc_p[(size_t)j * r->NF + i];
}

void port_destroy(port_run* r) {
  if (!r) return;
  free(r->ind_i); free(r->ind_j); free(r->forc); free(r->forc_f); free(r->forc_p); free(r->frec);
  free(r->X); free(r->Y); free(r->K); free(r->L); free(r->wrk);
  free(r->cl2m); free(r->cm2l); free(r->iRd2);
  free(r->psi); free(r->q); free(r->diff); free(r->lapn); free(r->topo);
  for (int s = 0; s < 3; ++s) free(r->fab[s]);
  free(r);
}

/* ---------------------------------------------------- boundary values */

/* adjust_bc, periodic branch, src/domain.h:225-256: South, North, West,
 * East copies in that order (the corners end up periodic). */
static void port_adjust_bc_periodic(port_run* r, double* f) {
  for (int k = 0; k < r->nl; ++k) {
    for (int i = 0; i < r->nxp2; ++i) f[IDX(r, i, 0, k)] = f[IDX(r, i, r->ny, k)];
    for (int i = 0; i < r->nxp2; ++i) f[IDX(r, i, r->ny + 1, k)] = f[IDX(r, i, 1, k)];
    for (int j = 0; j < r->nyp2; ++j) f[IDX(r, 0, j, k)] = f[IDX(r, r->nx, j, k)];
    for (int j = 0; j < r->nyp2; ++j) f[IDX(r, r->nx + 1, j, k)] = f[IDX(r, 1, j, k)];
  }
}

/* adjust_bc, bounded branch, src/domain.h:308-348. */
static void port_adjust_bc(port_run* r, double* f, int field_type) {
  if (r->p.bc_fac == -1) {
    port_adjust_bc_periodic(r, f);
    return;
  }
  const double psi_bc = 0.0, c = 2 * r->p.bc_fac / sq(r->Delta);
  const double* psi = r->psi;
  for (int k = 0; k < r->nl; ++k) {
    for (int i = 0; i < r->nxp2; ++i) {
      int j = 0;
      f[IDX(r, i, j, k)] = field_type ? c * (psi[IDX(r, i, j + 1, k)] - psi_bc) : psi_bc;
    }
    for (int i = 0; i < r->nxp2; ++i) {
      int j = r->ny + 1;
      f[IDX(r, i, j, k)] = field_type ? c * (psi[IDX(r, i, j - 1, k)] - psi_bc) : psi_bc;
    }
    for (int j = 0; j < r->nyp2; ++j) {
      int i = 0;
      f[IDX(r, i, j, k)] = field_type ? c * (psi[IDX(r, i + 1, j, k)] - psi_bc) : psi_bc;
    }
    for (int j = 0; j < r->nyp2; ++j) {
      int i = r->nx + 1;
      f[IDX(r, i, j, k)] = field_type ? c * (psi[IDX(r, i - 1, j, k)] - psi_bc) : psi_bc;
    }
  }
}

/* ------------------------------------------------------- PV inversion */

/* invert_pv, src/elliptic.h:76-155, periodic branch: rows of Nx+2 doubles
 * (idx_fft with N_fft = Nxp2, :21), in-place r2c / c2r with the (Nx, Ny)
 * plan shape of :41-42, the division of :103-117 and the /norm of :131. */
static void port_invert_periodic(port_run* r) {
  const int nl = r->nl, nx = r->nx, ny = r->ny, ld = nx + 2, nk = (nx + 2) / 2;
  double *q = r->q, *psi = r->psi, *w = r->wrk;
  memset(psi, 0, sizeof(double) * (size_t)r->nxp2 * r->nyp2 * nl);
  for (int m = 0; m < nl; ++m) {
    for (int j = 1; j < ny + 1; ++j)
      for (int i = 1; i < nx + 1; ++i) {
        double acc = 0;
        for (int l = 0; l < nl; ++l) acc += r->cl2m[m * nl + l] * q[IDX(r, i, j, l)];
        w[(size_t)(j - 1) * ld + (i - 1)] = acc;
      }
    om_dft_r2c_2d_any(nx, ny, w, r->fast);
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nk; ++i) {
        double fact = -(sq(r->L[j]) + sq(r->K[i]) + r->iRd2[m]);
        if (fact != 0) {
          w[(size_t)j * ld + 2 * i] = w[(size_t)j * ld + 2 * i] / fact;
          w[(size_t)j * ld + 2 * i + 1] = w[(size_t)j * ld + 2 * i + 1] / fact;
        }
      }
    w[0] = 0;
    w[1] = 0;
    om_dft_c2r_2d_any(nx, ny, w, r->fast);
    for (int j = 1; j < ny + 1; ++j)
      for (int i = 1; i < nx + 1; ++i) w[(size_t)(j - 1) * ld + (i - 1)] = w[(size_t)(j - 1) * ld + (i - 1)] / r->norm;
    for (int j = 1; j < ny + 1; ++j)
      for (int i = 1; i < nx + 1; ++i)
        for (int l = 0; l < nl; ++l) psi[IDX(r, i, j, l)] += r->cm2l[l * nl + m] * w[(size_t)(j - 1) * ld + (i - 1)];
  }
  port_adjust_bc(r, psi, 0);
  port_adjust_bc(r, q, 1);
}

/* invert_pv, src/elliptic.h:76-155 (bounded branch). */
void port_invert(port_run* r) {
  const int nl = r->nl, nx = r->nx, ny = r->ny;
  double *q = r->q, *psi = r->psi, *w = r->wrk;
  if (r->p.bc_fac == -1) {
    port_invert_periodic(r);
    return;
  }
  memset(psi, 0, sizeof(double) * (size_t)r->nxp2 * r->nyp2 * nl);
  for (int m = 0; m < nl; ++m) {
    for (int j = 1; j < ny + 1; ++j)
      for (int i = 1; i < nx + 1; ++i) {
        double acc = 0;
        for (int l = 0; l < nl; ++l) acc += r->cl2m[m * nl + l] * q[IDX(r, i, j, l)];
        w[(size_t)(j - 1) * nx + (i - 1)] = acc;
      }
    om_dst2(ny, nx, w, r->fast);
    for (int j = 1; j < ny + 1; ++j)
      for (int i = 1; i < nx + 1; ++i) {
        double fact = -(sq(r->L[i]) + sq(r->K[j]) + r->iRd2[m]);
        w[(size_t)(j - 1) * nx + (i - 1)] = w[(size_t)(j - 1) * nx + (i - 1)] / fact;
      }
    om_dst2(ny, nx, w, r->fast);
    for (size_t s = 0; s < (size_t)nx * ny; ++s) w[s] = w[s] / r->norm;
    for (int j = 1; j < ny + 1; ++j)
      for (int i = 1; i < nx + 1; ++i)
        for (int l = 0; l < nl; ++l)
          psi[IDX(r, i, j, l)] += r->cm2l[l * nl + m] * w[(size_t)(j - 1) * nx + (i - 1)];
  }
  port_adjust_bc(r, psi, 0);
  port_adjust_bc(r, q, 1);
}

/* ---------------------------------------------------------------- RHS */

#define P_(f, di, dj, k) (f)[IDX(r, i + (di), j + (dj), k)]
/* laplacian, src/domain.h:12: the macro's numerator; callers divide by
 * sq(Delta) after any coefficient, as the macro expansion does. */
static double port_lapnum(const port_run* r, const double* f, int i, int j, int k) {
  return P_(f, 1, 0, k) + P_(f, -1, 0, k) + P_(f, 0, 1, k) + P_(f, 0, -1, k) - 4 * P_(f, 0, 0, k);
}
static double port_lap(const port_run* r, const double* f, int i, int j, int k) {
  return port_lapnum(r, f, i, j, k) / (sq(r->Delta));
}
/* jacobian_lev, src/domain.h:17-27 */
static double port_jac(const port_run* r, const double* p, const double* q, int i, int j, int k1, int k2) {
  return ((P_(p, 1, 0, k1) - P_(p, -1, 0, k1)) * (P_(q, 0, 1, k2) - P_(q, 0, -1, k2))
          + (P_(p, 0, -1, k1) - P_(p, 0, 1, k1)) * (P_(q, 1, 0, k2) - P_(q, -1, 0, k2))
          + P_(p, 1, 0, k1) * (P_(q, 1, 1, k2) - P_(q, 1, -1, k2))
          - P_(p, -1, 0, k1) * (P_(q, -1, 1, k2) - P_(q, -1, -1, k2))
          - P_(p, 0, 1, k1) * (P_(q, 1, 1, k2) - P_(q, -1, 1, k2))
          + P_(p, 0, -1, k1) * (P_(q, 1, -1, k2) - P_(q, -1, -1, k2))
          + P_(q, 0, 1, k2) * (P_(p, 1, 1, k1) - P_(p, -1, 1, k1))
          - P_(q, 0, -1, k2) * (P_(p, 1, -1, k1) - P_(p, -1, -1, k1))
          - P_(q, 1, 0, k2) * (P_(p, 1, 1, k1) - P_(p, 1, -1, k1))
          + P_(q, -1, 0, k2) * (P_(p, -1, 1, k1) - P_(p, -1, -1, k1)))
         / (12. * r->Delta * r->Delta);
}

/* calc_diff, src/dynamics.h:13-44. */
static void port_calc_diff(port_run* r) {
  const size_t n3 = (size_t)r->nxp2 * r->nyp2 * r->nl;
  memcpy(r->diff, r->psi, sizeof(double) * n3);
  for (int n = 0; n <= r->p.n_hyper; n += 2) {
    for (int k = 0; k < r->nl; ++k)
      for (int j = 1; j < r->ny + 1; ++j)
        for (int i = 1; i < r->nx + 1; ++i) r->lapn[IDX(r, i, j, k)] = port_lap(r, r->diff, i, j, k);
    port_adjust_bc(r, r->lapn, 1);
    memcpy(r->diff, r->lapn, sizeof(double) * n3);
  }
}

/* rhs, src/dynamics.h:47-73. */
static void port_rhs(port_run* r, double* f) {
  const qgw_params* p = &r->p;
  const double *psi = r->psi, *q = r->q;
  port_invert(r);
  port_calc_diff(r);
  for (int k = 0; k < r->nl; ++k)
    for (int j = 1; j < r->ny + 1; ++j)
      for (int i = 1; i < r->nx + 1; ++i)
        f[IDX(r, i, j, k)] = -port_jac(r, psi, q, i, j, k, k)
                             - (p->beta * (P_(psi, 1, 0, k) - P_(psi, -1, 0, k)) / (2 * r->Delta))
                             + p->nu * port_lapnum(r, q, i, j, k) / (sq(r->Delta))
                             + r->nu_hyper * r->lapn[IDX(r, i, j, k)];
  const int kb = r->nl - 1;
  for (int j = 1; j < r->ny + 1; ++j)
    for (int i = 1; i < r->nx + 1; ++i) {
      /* forcing_q, src/domain.h:33 */
      f[IDX(r, i, j, 0)] += (-p->tau0 / p->dh[0] * p->forc_mode * PORT_PI / r->Ly *
                             sin(p->forc_mode * PORT_PI * (r->Y[j]) / r->Ly));
      f[IDX(r, i, j, kb)] += -p->hEkb * p->f0 / (2 * p->dh[kb]) * port_lapnum(r, psi, i, j, kb) / (sq(r->Delta))
                             - port_jac(r, psi, r->topo, i, j, kb, 0) * p->f0 / p->dh[kb];
    }
}
#undef P_

/* ----------------------------------------------------------- time step */

/* adjust_timestep, src/timestep.h:69-111. */
static double port_adjust_timestep(port_run* r) {
  double dt_max = PORT_HUGE;
  const double* psi = r->psi;
  for (int k = 0; k < r->nl; ++k)
    for (int j = 1; j < r->ny + 1; ++j)
      for (int i = 1; i < r->nx + 1; ++i) {
        double u = -(psi[IDX(r, i + 1, j, k)] - psi[IDX(r, i, j, k)]) / r->Delta;
        double v = (psi[IDX(r, i, j + 1, k)] - psi[IDX(r, i, j, k)]) / r->Delta;
        u = (fabs(u) < fabs(v)) ? fabs(v) : fabs(u);
        if (u != 0.) {
          double dt_loc = r->p.cfl * r->Delta / u;
          if (dt_loc < dt_max) dt_max = dt_loc;
        }
      }
  double dt = r->dt;
  if (dt < dt_max) dt = 2. * dt;
  if (dt > r->DT_max) dt = r->DT_max;
  if (dt > dt_max) dt = dt_max;
  if (r->t_out > r->t + PORT_TEPS) {
    unsigned int n_step = (unsigned int)((r->t_out - r->t) / dt);
    if (n_step == 0)
      dt = r->t_out - r->t;
    else {
      double dt1 = (r->t_out - r->t) / n_step;
      if (dt1 > dt * (1. + PORT_TEPS))
        dt = (r->t_out - r->t) / (n_step + 1);
      else if (dt1 < dt)
        dt = dt1;
    }
  }
  return dt;
}

/* timestep, src/timestep.h:114-167, with the stochastic and 4-D forcing
 * add-ons. */
void port_timestep(port_run* r) {
  double* swap = r->fab[2];
  r->fab[2] = r->fab[1];
  r->fab[1] = r->fab[0];
  r->fab[0] = swap;
  port_rhs(r, r->fab[0]);
  r->dt1 = r->dt0;
  r->dt0 = r->dt;
  r->dt = port_adjust_timestep(r);
  const double dt = r->dt, dt0 = r->dt0, dt1 = r->dt1;
  const double c0 = dt * (2 * sq(dt) + 3 * dt * (2 * dt0 + dt1) + 6 * dt0 * (dt0 + dt1)) / (6 * dt0 * (dt0 + dt1));
  const double c1 = sq(dt) * (-dt / 3 - dt0 / 2 - dt1 / 2) / (dt0 * dt1);
  const double c2 = sq(dt) * (dt / 3 + dt0 / 2) / (dt1 * (dt0 + dt1));
  const double *f0 = r->fab[0], *f1 = r->fab[1], *f2 = r->fab[2];
  for (int k = 0; k < r->nl; ++k)
    for (int j = 1; j < r->ny + 1; ++j)
      for (int i = 1; i < r->nx + 1; ++i) {
        const size_t s = IDX(r, i, j, k);
        r->q[s] = r->q[s] + c0 * f0[s] + c1 * f1[s] + c2 * f2[s];
      }
  if (r->p.k_f != 0) { /* src/timestep.h:143-150 */
    port_calc_forc(r);
    for (int j = 1; j < r->ny + 1; ++j)
      for (int i = 1; i < r->nx + 1; ++i) r->q[IDX(r, i, j, 0)] += r->forc[IDX(r, i, j, 0)] * sqrt(dt);
  }
  if (r->p.dt_forc_period != 0 && r->nrec > 0) { /* src/timestep.h:152-163 */
    /* calc_4d_forcing, src/forcing.h:259-287: linear interpolation in t
     * (the time before this step's increment) between records irec1, irec2 */
    const int n_rec = (int)floor(r->p.dt_forc_period / r->p.dt_forc);
    const int irec1 = ((int)floor(r->t / r->p.dt_forc)) % n_rec;
    const int irec2 = (irec1 + 1) % n_rec;
    const double w2 = r->t / r->p.dt_forc - (int)floor(r->t / r->p.dt_forc);
    const double w1 = 1 - w2;
    const size_t n3 = (size_t)r->nxp2 * r->nyp2 * r->nl;
    const double *t1 = r->frec + (size_t)irec1 * n3, *t2 = r->frec + (size_t)irec2 * n3;
    for (int k = 0; k < r->nl; ++k)
      for (int j = 1; j < r->ny + 1; ++j)
        for (int i = 1; i < r->nx + 1; ++i) {
          const size_t s = IDX(r, i, j, k);
          const double qf = w1 * t1[s] + w2 * t2[s];
          r->q[s] += qf * dt;
        }
  }
  r->t = r->t + dt;
}

int port_run_steps(port_run* r, int nsteps, int snap) {
  int it = 0;
  for (; it < nsteps; ++it) {
    if (r->p.tend > 0 && !(r->t < r->p.tend)) break;
    if (snap && fabs(r->t - r->t_out) < PORT_TEPS * r->dt) r->t_out += r->p.dt_out;
    port_timestep(r);
  }
  return it;
}

/* ------------------------------------------------------------ accessors */

void port_sizes(const port_run* r, int* nx, int* ny, int* nl) { *nx = r->nx; *ny = r->ny; *nl = r->nl; }

void port_set_q(port_run* r, const double* q) {
  memcpy(r->q, q, sizeof(double) * (size_t)r->nxp2 * r->nyp2 * r->nl);
}

void port_set_forcing_records(port_run* r, const double* rec, int nrec) {
  const size_t n3 = (size_t)r->nxp2 * r->nyp2 * r->nl;
  free(r->frec);
  r->frec = (double*)malloc(sizeof(double) * n3 * (nrec > 0 ? nrec : 1));
  memcpy(r->frec, rec, sizeof(double) * n3 * nrec);
  r->nrec = nrec;
}

void port_set_topo(port_run* r, const double* topo) {
  memcpy(r->topo, topo, sizeof(double) * (size_t)r->nxp2 * r->nyp2);
}

void port_get(const port_run* r, double* psi, double* q) {
  const size_t n3 = (size_t)r->nxp2 * r->nyp2 * r->nl;
  if (psi) memcpy(psi, r->psi, sizeof(double) * n3);
  if (q) memcpy(q, r->q, sizeof(double) * n3);
}

void port_get_modes(const port_run* r, double* cl2m, double* cm2l, double* iRd2) {
  memcpy(cl2m, r->cl2m, sizeof(double) * r->nl * r->nl);
  memcpy(cm2l, r->cm2l, sizeof(double) * r->nl * r->nl);
  memcpy(iRd2, r->iRd2, sizeof(double) * r->nl);
}

void port_get_time(const port_run* r, qgw_time* tm, double* t_out) {
  tm->t = r->t; tm->dt = r->dt; tm->dt0 = r->dt0; tm->dt1 = r->dt1; tm->DT_max = r->DT_max;
  if (t_out) *t_out = r->t_out;
}

void port_set_time(port_run* r, const qgw_time* tm, double t_out) {
  r->t = tm->t; r->dt = tm->dt; r->dt0 = tm->dt0; r->dt1 = tm->dt1; r->DT_max = tm->DT_max;
  r->t_out = t_out;
}

void port_dst1(int n, int howmany, double* data, int fast) {
  if (fast) om_dst1(n, howmany, data, n, 1);
  else om_dst1_direct(n, howmany, data, n, 1);
}
