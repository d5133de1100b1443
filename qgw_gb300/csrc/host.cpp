// host.cpp -- host-side set-up of a qgw run: params.in parsing, vertical
// modes, initial time step, topography.  Plain C++, no CUDA.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/qgw_gpu.h"
#include "host.h"

namespace {
const double kPi = 3.141592653589793;  // the reference's pi, src/qg.c:44
}

extern "C" void qgw_params_default(qgw_params* p) {
  std::memset(p, 0, sizeof(*p));
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

// Array values `[a, b, c]`: tokens split on '[', ',' and ']' for the first
// token and on ',' afterwards, parsed with atof (src/extra.h:98-115).
static void parse_array(char* v, double* out) {
  if (char* nl = std::strchr(v, '\n')) *nl = 0;
  int n = 0;
  char* save = nullptr;
  char* tok = strtok_r(v, "[,]", &save);
  while (tok) {
    if (n < QGW_NL_MAX) out[n] = std::atof(tok);
    ++n;
    tok = strtok_r(nullptr, ",", &save);
  }
}

extern "C" int qgw_params_read(qgw_params* p, const char* path) {
  if (!p || !path) return QGW_ERR_PARAM;
  FILE* fp = std::fopen(path, "rt");
  if (!fp) return QGW_ERR_FILE;
  char line[300];
  while (std::fgets(line, sizeof line, fp)) {
    // remove spaces (only ' ', as trim_whitespace, src/extra.h:26-33)
    char* d = line;
    for (char* c = line; *c; ++c)
      if (*c != ' ') *d++ = *c;
    *d = 0;
    char* save = nullptr;
    char* key = strtok_r(line, "=", &save);
    char* val = strtok_r(nullptr, "=", &save);
    if (!key) continue;
    const char* v = val ? val : "";
    struct { const char* name; int* iv; double* dv; double* av; } tab[] = {
        {"NX", &p->NX, nullptr, nullptr}, {"NY", &p->NY, nullptr, nullptr},
        {"nl", &p->nl, nullptr, nullptr}, {"n_hyper", &p->n_hyper, nullptr, nullptr},
        {"Lx", nullptr, &p->Lx, nullptr}, {"dh", nullptr, nullptr, p->dh},
        {"tau0", nullptr, &p->tau0, nullptr}, {"forc_mode", nullptr, &p->forc_mode, nullptr},
        {"f0", nullptr, &p->f0, nullptr}, {"beta", nullptr, &p->beta, nullptr},
        {"nu", nullptr, &p->nu, nullptr}, {"nu_hyper", nullptr, &p->nu_hyper, nullptr},
        {"hEkb", nullptr, &p->hEkb, nullptr}, {"N2", nullptr, nullptr, p->N2},
        {"Ld", nullptr, &p->Ld, nullptr}, {"h_topo", nullptr, &p->h_topo, nullptr},
        {"w_topo", nullptr, &p->w_topo, nullptr}, {"bc_fac", nullptr, &p->bc_fac, nullptr},
        {"tend", nullptr, &p->tend, nullptr}, {"dt_out", nullptr, &p->dt_out, nullptr},
        {"dt_forc", nullptr, &p->dt_forc, nullptr},
        {"dt_forc_period", nullptr, &p->dt_forc_period, nullptr},
        {"sigma_f", nullptr, &p->sigma_f, nullptr}, {"k_f", nullptr, &p->k_f, nullptr},
        {"cfl", nullptr, &p->cfl, nullptr}, {"dt", nullptr, &p->dt, nullptr},
    };
    for (auto& e : tab) {
      if (std::strcmp(e.name, key) != 0) continue;
      if (e.iv) *e.iv = std::atoi(v);
      else if (e.dv) *e.dv = std::atof(v);
      else if (val) parse_array(val, e.av);
      break;
    }
  }
  std::fclose(fp);
  return QGW_OK;
}

namespace qgw_host {

// Eigen-decomposition of a real symmetric tridiagonal matrix by the
// implicit QL algorithm with Wilkinson shifts (a published method:
// Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11 (1968), the
// "tql2" procedure).  d: diagonal (n), e: sub-diagonal e[1..n-1];
// z starts as the identity and returns the eigenvectors in its columns.
static int tql2(int n, double* d, double* e, double* z) {
  for (int i = 1; i < n; ++i) e[i - 1] = e[i];
  e[n - 1] = 0.0;
  double f = 0.0, tst1 = 0.0;
  for (int l = 0; l < n; ++l) {
    tst1 = std::fmax(tst1, std::fabs(d[l]) + std::fabs(e[l]));
    int m = l;
    while (m < n) {
      if (std::fabs(e[m]) <= 2.2e-16 * tst1) break;
      ++m;
    }
    if (m == n) m = n - 1;
    if (m > l) {
      int iter = 0;
      do {
        if (++iter > 60) return -1;
        double g = d[l];
        double p = (d[l + 1] - g) / (2.0 * e[l]);
        double r = std::hypot(p, 1.0);
        if (p < 0) r = -r;
        d[l] = e[l] / (p + r);
        d[l + 1] = e[l] * (p + r);
        const double dl1 = d[l + 1];
        double h = g - d[l];
        for (int i = l + 2; i < n; ++i) d[i] -= h;
        f += h;
        p = d[m];
        double c = 1.0, c2 = 1.0, c3 = 1.0, s = 0.0, s2 = 0.0;
        const double el1 = e[l + 1];
        for (int i = m - 1; i >= l; --i) {
          c3 = c2;
          c2 = c;
          s2 = s;
          g = c * e[i];
          h = c * p;
          r = std::hypot(p, e[i]);
          e[i + 1] = s * r;
          s = e[i] / r;
          c = p / r;
          p = c * d[i] - s * g;
          d[i + 1] = h + s * (c * g + s * d[i]);
          for (int k = 0; k < n; ++k) {
            h = z[k * n + i + 1];
            z[k * n + i + 1] = s * z[k * n + i] + c * h;
            z[k * n + i] = c * z[k * n + i] - s * h;
          }
        }
        p = -s * s2 * c3 * el1 * e[l] / dl1;
        e[l] = s * p;
        d[l] = c * p;
      } while (std::fabs(e[l]) > 2.2e-16 * tst1);
    }
    d[l] = d[l] + f;
    e[l] = 0.0;
  }
  return 0;
}

}  // namespace qgw_host

// Vertical modes, following compute_eigmode (src/eigmode.h:87-271).  The
// stretching matrix G is tridiagonal with dh_l G[l][l+1] = dh_{l+1} G[l+1][l]
// (src/eigmode.h:107-118), so D^{1/2} G D^{-1/2} (D = diag dh) is symmetric;
// its eigenvectors U give the right vectors D^{-1/2} U and the left vectors
// D^{1/2} U.  Sorting, the Flierl (1978) normalisation and the surface-sign
// convention (src/eigmode.h:153-223) then make the result independent of the
// eigensolver.
extern "C" int qgw_eigmode(const qgw_params* p, double* cl2m, double* cm2l, double* iRd2) {
  if (!p || !cl2m || !cm2l || !iRd2) return QGW_ERR_PARAM;
  const int nl = p->nl;
  if (nl < 1 || nl > QGW_NL_MAX) return QGW_ERR_PARAM;
  if (nl == 1) {
    cl2m[0] = 1.0;
    cm2l[0] = 1.0;
    iRd2[0] = (p->Ld != 0) ? 1 / (p->Ld * p->Ld) : 0.0;
    return QGW_OK;
  }
  std::vector<double> dhc(nl), G((size_t)nl * nl, 0.0);
  for (int l = 0; l < nl - 1; ++l) dhc[l] = 0.5 * (p->dh[l] + p->dh[l + 1]);
  double htotal = 0;
  for (int k = 0; k < nl; ++k) htotal += p->dh[k];
  const double f2 = p->f0 * p->f0;
  for (int l = 0; l < nl; ++l) {
    if (l > 0) G[nl * l + l - 1] = -f2 / p->N2[l - 1] / (dhc[l - 1] * p->dh[l]);
    if (l < nl - 1) G[nl * l + l + 1] = -f2 / p->N2[l] / (dhc[l] * p->dh[l]);
  }
  for (int l = 0; l < nl; ++l) {
    double s = 0;
    if (l > 0) s -= G[nl * l + l - 1];
    if (l < nl - 1) s -= G[nl * l + l + 1];
    G[nl * l + l] = s;
  }
  // symmetrise
  std::vector<double> sd(nl), d(nl), e(nl, 0.0), z((size_t)nl * nl, 0.0);
  for (int l = 0; l < nl; ++l) {
    if (!(p->dh[l] > 0)) return QGW_ERR_PARAM;
    sd[l] = std::sqrt(p->dh[l]);
    d[l] = G[nl * l + l];
    z[(size_t)l * nl + l] = 1.0;
  }
  for (int l = 1; l < nl; ++l) {
    const double up = G[nl * (l - 1) + l], lo = G[nl * l + l - 1];
    if (!(up * lo > 0)) return QGW_ERR_EIGEN;
    e[l] = (up < 0 ? -1.0 : 1.0) * std::sqrt(up * lo);
  }
  // The QL iteration keeps its accuracy on a strongly graded matrix only
  // with the large entries last.  Thin, strongly stratified upper layers put
  // them first (many stretched layers: couplings falling by 1e6..1e10 from
  // top to bottom), so where the couplings fall by more than 1e3 the matrix
  // is solved in reversed layer order and the vectors are mapped back.
  const bool reverse = std::fabs(e[1]) > 1e3 * std::fabs(e[nl - 1]);
  if (reverse) {
    std::vector<double> dr(nl), er(nl, 0.0);
    for (int i = 0; i < nl; ++i) dr[i] = d[nl - 1 - i];
    for (int i = 1; i < nl; ++i) er[i] = e[nl - i];
    if (qgw_host::tql2(nl, dr.data(), er.data(), z.data())) return QGW_ERR_EIGEN;
    d = dr;
    std::vector<double> zr(z);
    for (int k = 0; k < nl; ++k)
      for (int m = 0; m < nl; ++m) z[(size_t)k * nl + m] = zr[(size_t)(nl - 1 - k) * nl + m];
  } else if (qgw_host::tql2(nl, d.data(), e.data(), z.data())) {
    return QGW_ERR_EIGEN;
  }
  // ascending order
  std::vector<int> ord(nl);
  for (int m = 0; m < nl; ++m) ord[m] = m;
  for (int a = 1; a < nl; ++a) {
    int v = ord[a], b = a - 1;
    while (b >= 0 && d[ord[b]] > d[v]) { ord[b + 1] = ord[b]; --b; }
    ord[b + 1] = v;
  }
  std::vector<double> vr((size_t)nl * nl), vl((size_t)nl * nl);
  for (int m = 0; m < nl; ++m)
    for (int k = 0; k < nl; ++k) {
      const double u = z[(size_t)k * nl + ord[m]];
      vr[(size_t)k * nl + m] = u / sd[k];
      vl[(size_t)k * nl + m] = u * sd[k];
    }
  for (int m = 0; m < nl; ++m) {
    double dotp = 0;
    for (int k = 0; k < nl; ++k) dotp += p->dh[k] * vr[(size_t)k * nl + m] * vr[(size_t)k * nl + m];
    const double flfac = (vr[m] > 0 ? 1 : -1) * std::sqrt(htotal / dotp);
    for (int k = 0; k < nl; ++k) vr[(size_t)k * nl + m] *= flfac;
  }
  for (int m = 0; m < nl; ++m) {
    double dotp = 0;
    for (int k = 0; k < nl; ++k) dotp += vr[(size_t)k * nl + m] * vl[(size_t)k * nl + m];
    for (int k = 0; k < nl; ++k) vl[(size_t)k * nl + m] /= dotp;
  }
  for (int m = 0; m < nl; ++m)
    for (int k = 0; k < nl; ++k) {
      cl2m[k * nl + m] = vl[(size_t)m * nl + k];
      cm2l[k * nl + m] = vr[(size_t)k * nl + m];
    }
  iRd2[0] = 0.0;
  for (int k = 1; k < nl; ++k) iRd2[k] = d[ord[k]];
  return QGW_OK;
}

static void interior(const qgw_params* p, int* nx, int* ny) {
  *nx = p->NX;
  *ny = p->NY;
  if (p->bc_fac >= 0) { *nx -= 1; *ny -= 1; }
}

double qgw_host_nu_hyper(const qgw_params* p) {
  // init_vars, src/domain.h:210
  return std::pow(-1, p->n_hyper / 2 - 1) * std::fabs(p->nu_hyper);
}

// check_timestep, src/timestep.h:18-54.  Its min/max come from the
// unparenthesised macros of src/qg.c:40-41, so
//   max(max(a,b),c) == (a < b) ? b : ((a < c) ? c : a)
//   1e-3*min(A,B)   == (1e-3*A > B) ? B : A
extern "C" int qgw_check_timestep(const qgw_params* p, double* DT_max, double* dt_out) {
  if (!p || !DT_max || !dt_out) return QGW_ERR_PARAM;
  int nx, ny;
  interior(p, &nx, &ny);
  if (nx < 1 || p->NX < 1 || p->NY < 1) return QGW_ERR_PARAM;
  const double Delta = p->Lx / p->NX;
  const double Ly = p->NY * Delta;
  const double nuh = qgw_host_nu_hyper(p);
  const double a = nuh * 20. / std::pow(p->Lx / nx, p->n_hyper);
  const double b = p->nu * 20. / std::pow(p->Lx / nx, 2);
  const double c = 2. * p->beta * p->Lx;
  const double mx = (a < b) ? b : ((a < c) ? c : a);
  const double DT = std::pow(mx, -1.);
  double dt = 0.0;
  if (p->tau0 != 0 && p->sigma_f != 0) {
    const double A = std::sqrt(p->cfl * Delta / (p->tau0 / p->dh[0] * p->forc_mode * kPi / Ly * Ly));
    const double B = std::pow((Delta * p->cfl) * (Delta * p->cfl) / p->sigma_f, 1. / 3.);
    dt = (1e-3 * A > B) ? B : A;
  } else if (p->tau0 != 0 && p->sigma_f == 0) {
    dt = 1e-3 * std::sqrt(p->cfl * Delta / (p->tau0 / p->dh[0] * p->forc_mode * kPi / Ly * Ly));
  } else if (p->tau0 == 0 && p->sigma_f != 0) {
    dt = 1e-3 * std::pow((Delta * p->cfl) * (Delta * p->cfl) / p->sigma_f, 1. / 3.);
  }
  if (DT != 0 && dt > DT) dt = DT;
  *DT_max = DT;
  *dt_out = dt;
  return QGW_OK;
}

// Topography of init_vars, src/domain.h:200-207, on the (ny+2, nx+2) grid.
extern "C" int qgw_topo(const qgw_params* p, double* topo) {
  if (!p || !topo) return QGW_ERR_PARAM;
  int nx, ny;
  interior(p, &nx, &ny);
  const double Delta = p->Lx / p->NX;
  const double Ly = p->NY * Delta;
  auto shelf = [](double x, double d) { return 1 - std::exp(-(x * x) / (2 * (d * d))); };
  for (int j = 0; j < ny + 2; ++j)
    for (int i = 0; i < nx + 2; ++i) {
      const int off = p->bc_fac == -1 ? -1 : 0;  // src/domain.h:144-148
      const double X = (i + off) * Delta, Y = (j + off) * Delta;
      topo[(size_t)j * (nx + 2) + i] =
          p->h_topo * (1 - shelf(X, p->w_topo) * shelf(p->Lx - X, p->w_topo) * shelf(Y, p->w_topo) *
                               shelf(Ly - Y, p->w_topo));
    }
  return QGW_OK;
}

// forcing_q (src/domain.h:33) on interior row j (1-based), written with the
// reference's operator order.
int qgw_host_forcing_ring(const qgw_params* p, std::vector<int>* ij) {
  if (p->k_f == 0) return 0;
  const double kf = p->k_f / (2 * kPi);  // k_f /= 2*pi (src/forcing.h:72)
  const int NF = p->NX;                   // N_F = NX, or NXp1 of the reduced NX
  const int NK = NF / 2 + 1;
  const double dk = 1. / p->Lx;
  int NP = 0;
  for (int j = 0; j < NF; j++)
    for (int i = 0; i < NK; i++) {
      const double l = (((j + NF / 2) % NF) - NF / 2) * dk;
      const double k = (i)*dk;
      const double dist_k = std::fabs(k - std::sqrt(kf * kf - l * l));
      const double a = std::fabs(l - std::sqrt(kf * kf - k * k)), b = std::fabs(l + std::sqrt(kf * kf - k * k));
      const double dist_l = (a < b) ? a : b;  // the min macro of src/qg.c:40
      if (dist_k < dk / 2 || dist_l < dk / 2) {
        ++NP;
        ij->push_back(i);
        ij->push_back(j);
      }
    }
  return NP;
}

double qgw_host_wind(const qgw_params* p, int j) {
  const double Delta = p->Lx / p->NX;
  const double Ly = p->NY * Delta;
  // periodic runs put the zero of Y at the second grid point (src/domain.h:144-148)
  const double Y = (j + (p->bc_fac == -1 ? -1 : 0)) * Delta;
  return (-p->tau0 / p->dh[0] * p->forc_mode * kPi / Ly * std::sin(p->forc_mode * kPi * (Y) / Ly));
}
