/*
 * oracle_math.c -- CPU numerics of the oracle (test infrastructure only;
 * see oracle_math.h).  Plain C99, no external libraries.
 */
#include "oracle_math.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double OM_PI = 3.14159265358979323846;

/* ---------------------------------------------------------------- tables */

/* sin(pi*m/M) for m = 0..2M-1, with m reduced exactly before the libm call
 * so that the table is accurate to one rounding. */
static double* sin_table(int M) {
  double* s = (double*)malloc(sizeof(double) * 2 * (size_t)M);
  for (int m = 0; m < 2 * M; ++m) {
    /* reduce to [0, M/2] by symmetry: sin(pi - x) = sin x, sin(pi + x) = -sin x */
    int r = m, sg = 1;
    if (r >= M) { r -= M; sg = -1; }
    if (2 * r > M) r = M - r;
    s[m] = sg * sin(OM_PI * (double)r / (double)M);
  }
  return s;
}

/* ----------------------------------------------------------- direct DST-I */

void om_dst1_direct(int n, int howmany, double* data, int stride, int dist) {
  const int M = n + 1;
  double* s = sin_table(M);
  double* tmp = (double*)malloc(sizeof(double) * (size_t)n);
  for (int h = 0; h < howmany; ++h) {
    double* x = data + (size_t)h * stride;
    for (int k = 0; k < n; ++k) {
      double acc = 0.0;
      for (int j = 0; j < n; ++j)
        acc += x[(size_t)j * dist] * s[((long)(j + 1) * (k + 1)) % (2 * M)];
      tmp[k] = 2.0 * acc;
    }
    for (int k = 0; k < n; ++k) x[(size_t)k * dist] = tmp[k];
  }
  free(tmp);
  free(s);
}

/* ------------------------------------------------------ 2-D real DFT pair */

/* cos and sin of 2 pi m / N, m = 0..N-1, from the exactly reduced sine
 * table: sin(2 pi m / N) = sin(pi (2m) / N) and, for even N,
 * cos(2 pi m / N) = sin(pi (2m + N/2) / N); odd N falls back to libm. */
static void trig_table_any(int N, double* c, double* s) {
  if (N % 2 == 0) {
    double* t = sin_table(N);  /* sin(pi m' / N), m' < 2N */
    for (int m = 0; m < N; ++m) {
      s[m] = t[(2 * (long)m) % (2 * N)];
      c[m] = t[(2 * (long)m + N / 2) % (2 * N)];
    }
    free(t);
    return;
  }
  for (int m = 0; m < N; ++m) {
    c[m] = cos(2.0 * OM_PI * (double)m / (double)N);
    s[m] = sin(2.0 * OM_PI * (double)m / (double)N);
  }
}

/* complex DFT of length n along a strided sequence (sign -1 forward, +1
 * backward), unnormalised, in place through a scratch copy */
static void cdft_strided(int n, double* re, double* im, int dist, int sign, const double* c, const double* s,
                         double* tr, double* ti) {
  for (int k = 0; k < n; ++k) {
    double ar = 0.0, ai = 0.0;
    for (int j = 0; j < n; ++j) {
      const long m = ((long)j * k) % n;
      const double xr = re[(size_t)j * dist], xi = im[(size_t)j * dist];
      const double wr = c[m], wi = sign * s[m];
      ar += xr * wr - xi * wi;
      ai += xr * wi + xi * wr;
    }
    tr[k] = ar;
    ti[k] = ai;
  }
  for (int k = 0; k < n; ++k) {
    re[(size_t)k * dist] = tr[k];
    im[(size_t)k * dist] = ti[k];
  }
}

void om_dft_r2c_2d(int n0, int n1, double* data) {
  const int h = n1 / 2 + 1, ld = 2 * h;
  double *c1 = malloc(sizeof(double) * n1), *s1 = malloc(sizeof(double) * n1);
  double *c0 = malloc(sizeof(double) * n0), *s0 = malloc(sizeof(double) * n0);
  trig_table_any(n1, c1, s1);
  trig_table_any(n0, c0, s0);
  double* row = malloc(sizeof(double) * (size_t)n1);
  double *tr = malloc(sizeof(double) * (size_t)(n0 > n1 ? n0 : n1)), *ti = malloc(sizeof(double) * (size_t)(n0 > n1 ? n0 : n1));
  /* rows: real -> half spectrum */
  for (int r = 0; r < n0; ++r) {
    double* d = data + (size_t)r * ld;
    memcpy(row, d, sizeof(double) * (size_t)n1);
    for (int k = 0; k < h; ++k) {
      double ar = 0.0, ai = 0.0;
      for (int j = 0; j < n1; ++j) {
        const long m = ((long)j * k) % n1;
        ar += row[j] * c1[m];
        ai -= row[j] * s1[m];
      }
      d[2 * k] = ar;
      d[2 * k + 1] = ai;
    }
  }
  /* columns: complex forward DFT of length n0 */
  for (int k = 0; k < h; ++k) cdft_strided(n0, data + 2 * k, data + 2 * k + 1, ld, -1, c0, s0, tr, ti);
  free(c1); free(s1); free(c0); free(s0); free(row); free(tr); free(ti);
}

void om_dft_c2r_2d(int n0, int n1, double* data) {
  const int h = n1 / 2 + 1, ld = 2 * h;
  double *c1 = malloc(sizeof(double) * n1), *s1 = malloc(sizeof(double) * n1);
  double *c0 = malloc(sizeof(double) * n0), *s0 = malloc(sizeof(double) * n0);
  trig_table_any(n1, c1, s1);
  trig_table_any(n0, c0, s0);
  double *tr = malloc(sizeof(double) * (size_t)(n0 > n1 ? n0 : n1)), *ti = malloc(sizeof(double) * (size_t)(n0 > n1 ? n0 : n1));
  double* spec = malloc(sizeof(double) * (size_t)ld);
  /* columns: complex backward DFT of length n0 */
  for (int k = 0; k < h; ++k) cdft_strided(n0, data + 2 * k, data + 2 * k + 1, ld, +1, c0, s0, tr, ti);
  /* rows: half spectrum -> real, x_j = sum_k Y_k e^{+2 pi i jk/n1} over the
   * Hermitian completion Y_{n1-k} = conj(Y_k); the k = 0 and (even n1)
   * k = n1/2 terms contribute their real parts only */
  for (int r = 0; r < n0; ++r) {
    double* d = data + (size_t)r * ld;
    memcpy(spec, d, sizeof(double) * (size_t)ld);
    for (int j = 0; j < n1; ++j) {
      double acc = spec[0];
      for (int k = 1; k < h; ++k) {
        const long m = ((long)j * k) % n1;
        const double term = spec[2 * k] * c1[m] - spec[2 * k + 1] * s1[m];
        acc += (n1 % 2 == 0 && k == n1 / 2) ? term : 2.0 * term;
      }
      d[j] = acc;
    }
  }
  free(c1); free(s1); free(c0); free(s0); free(tr); free(ti); free(spec);
}

/* ------------------------------------------------------- radix-2 complex FFT */

typedef struct {
  int N;          /* complex length (power of two)            */
  int* rev;       /* bit-reversal permutation                 */
  double* wr;     /* cos(2 pi k / N), k < N/2                 */
  double* wi;     /* -sin(2 pi k / N)                          */
} om_fft_plan;

static int ilog2(int N) { int l = 0; while ((1 << l) < N) ++l; return l; }

static om_fft_plan* fft_plan_make(int N) {
  om_fft_plan* p = (om_fft_plan*)calloc(1, sizeof(om_fft_plan));
  p->N = N;
  p->rev = (int*)malloc(sizeof(int) * (size_t)N);
  p->wr = (double*)malloc(sizeof(double) * (size_t)(N / 2 + 1));
  p->wi = (double*)malloc(sizeof(double) * (size_t)(N / 2 + 1));
  const int lg = ilog2(N);
  for (int i = 0; i < N; ++i) {
    int r = 0;
    for (int b = 0; b < lg; ++b) if (i & (1 << b)) r |= 1 << (lg - 1 - b);
    p->rev[i] = r;
  }
  double* s = sin_table(N / 2 > 0 ? N / 2 : 1); /* sin(pi m/(N/2)) = sin(2 pi m / N) */
  for (int k = 0; k <= N / 2; ++k) {
    /* cos(2 pi k/N) = sin(2 pi (k + N/4)/N) */
    int H = N / 2 > 0 ? N / 2 : 1;
    p->wr[k] = s[(k + N / 4) % (2 * H)];
    p->wi[k] = -s[k % (2 * H)];
  }
  if (N < 4) { /* tiny sizes: direct evaluation */
    for (int k = 0; k <= N / 2; ++k) {
      p->wr[k] = cos(2.0 * OM_PI * k / N);
      p->wi[k] = -sin(2.0 * OM_PI * k / N);
    }
  }
  free(s);
  return p;
}

/* Forward transform Z_k = sum_m z_m exp(-2 pi i m k / N), in place. */
static void fft_exec(const om_fft_plan* p, double* re, double* im) {
  const int N = p->N;
  for (int i = 0; i < N; ++i) {
    int r = p->rev[i];
    if (r > i) {
      double t = re[i]; re[i] = re[r]; re[r] = t;
      t = im[i]; im[i] = im[r]; im[r] = t;
    }
  }
  for (int len = 2; len <= N; len <<= 1) {
    const int half = len >> 1, step = N / len;
    for (int b = 0; b < N; b += len) {
      for (int k = 0; k < half; ++k) {
        const double cr = p->wr[k * step], ci = p->wi[k * step];
        const int a = b + k, c = a + half;
        const double tr = re[c] * cr - im[c] * ci;
        const double ti = re[c] * ci + im[c] * cr;
        re[c] = re[a] - tr; im[c] = im[a] - ti;
        re[a] += tr; im[a] += ti;
      }
    }
  }
}

/* Small cache of plans keyed by length (the oracle is single-threaded per
 * process). */
#define OM_CACHE 8
static om_fft_plan* g_plans[OM_CACHE];
static double* g_sin[OM_CACHE];
static int g_sinM[OM_CACHE];

static om_fft_plan* fft_plan_get(int N) {
  for (int i = 0; i < OM_CACHE; ++i)
    if (g_plans[i] && g_plans[i]->N == N) return g_plans[i];
  for (int i = 0; i < OM_CACHE; ++i)
    if (!g_plans[i]) return g_plans[i] = fft_plan_make(N);
  return g_plans[0]; /* not reached for the sizes the oracle uses */
}

static const double* sin_get(int M) {
  for (int i = 0; i < OM_CACHE; ++i)
    if (g_sin[i] && g_sinM[i] == M) return g_sin[i];
  for (int i = 0; i < OM_CACHE; ++i)
    if (!g_sin[i]) { g_sinM[i] = M; return g_sin[i] = sin_table(M); }
  return NULL;
}

/* ------------------------------------------------ fast 2-D real DFT pair */
/* Same transforms as om_dft_r2c_2d / om_dft_c2r_2d for power-of-two sizes,
 * through the radix-2 complex FFT (rows as complex sequences with zero
 * imaginary part; the backward transform as conj(FFT(conj))). */
static int pow2_ok(int n) { return n >= 2 && (n & (n - 1)) == 0; }

static void r2c_2d_fast(int n0, int n1, double* data) {
  const int h = n1 / 2 + 1, ld = 2 * h;
  const om_fft_plan* p1 = fft_plan_get(n1);
  const om_fft_plan* p0 = fft_plan_get(n0);
  const int nmax = n0 > n1 ? n0 : n1;
  double *re = malloc(sizeof(double) * (size_t)nmax), *im = malloc(sizeof(double) * (size_t)nmax);
  for (int r = 0; r < n0; ++r) {
    double* d = data + (size_t)r * ld;
    for (int j = 0; j < n1; ++j) { re[j] = d[j]; im[j] = 0.0; }
    fft_exec(p1, re, im);
    for (int k = 0; k < h; ++k) { d[2 * k] = re[k]; d[2 * k + 1] = im[k]; }
  }
  for (int k = 0; k < h; ++k) {
    for (int r = 0; r < n0; ++r) { re[r] = data[(size_t)r * ld + 2 * k]; im[r] = data[(size_t)r * ld + 2 * k + 1]; }
    fft_exec(p0, re, im);
    for (int r = 0; r < n0; ++r) { data[(size_t)r * ld + 2 * k] = re[r]; data[(size_t)r * ld + 2 * k + 1] = im[r]; }
  }
  free(re); free(im);
}

static void c2r_2d_fast(int n0, int n1, double* data) {
  const int h = n1 / 2 + 1, ld = 2 * h;
  const om_fft_plan* p1 = fft_plan_get(n1);
  const om_fft_plan* p0 = fft_plan_get(n0);
  const int nmax = n0 > n1 ? n0 : n1;
  double *re = malloc(sizeof(double) * (size_t)nmax), *im = malloc(sizeof(double) * (size_t)nmax);
  for (int k = 0; k < h; ++k) {
    for (int r = 0; r < n0; ++r) { re[r] = data[(size_t)r * ld + 2 * k]; im[r] = -data[(size_t)r * ld + 2 * k + 1]; }
    fft_exec(p0, re, im);
    for (int r = 0; r < n0; ++r) { data[(size_t)r * ld + 2 * k] = re[r]; data[(size_t)r * ld + 2 * k + 1] = -im[r]; }
  }
  for (int r = 0; r < n0; ++r) {
    double* d = data + (size_t)r * ld;
    /* Hermitian completion; k = 0 and k = n1/2 by their real parts */
    re[0] = d[0]; im[0] = 0.0;
    for (int k = 1; k < n1 / 2; ++k) {
      re[k] = d[2 * k]; im[k] = -d[2 * k + 1];
      re[n1 - k] = d[2 * k]; im[n1 - k] = d[2 * k + 1];
    }
    re[n1 / 2] = d[n1]; im[n1 / 2] = 0.0;
    fft_exec(p1, re, im);
    for (int j = 0; j < n1; ++j) d[j] = re[j];
  }
  free(re); free(im);
}

void om_dft_r2c_2d_any(int n0, int n1, double* data, int fast) {
  if (fast && pow2_ok(n0) && pow2_ok(n1)) r2c_2d_fast(n0, n1, data);
  else om_dft_r2c_2d(n0, n1, data);
}

void om_dft_c2r_2d_any(int n0, int n1, double* data, int fast) {
  if (fast && pow2_ok(n0) && pow2_ok(n1)) c2r_2d_fast(n0, n1, data);
  else om_dft_c2r_2d(n0, n1, data);
}

/* ------------------------------------------------------------- fast DST-I */
/*
 * DST-I of length n = M-1 through a real DFT of length M (a published
 * method: the "sine transform via a real FFT" pre-/post-processing, e.g.
 * Press et al., Numerical Recipes, section 12.3):
 *   y_0 = 0, y_j = sin(pi j/M)(x_j + x_{M-j}) + (x_j - x_{M-j})/2   (1-based x)
 *   F_k = sum_j y_j exp(-2 pi i j k/M) = R_k + i I_k
 *   Y_{2k} = -2 I_k,   Y_1 = R_0,   Y_{2k+1} = Y_{2k-1} + 2 R_k.
 * The real DFT of length M is one complex FFT of length M/2 on
 * z_m = y_{2m} + i y_{2m+1} followed by the usual split.
 */
void om_dst1_fast(int n, int howmany, double* data, int stride, int dist) {
  const int M = n + 1;
  if (M < 4 || (M & (M - 1))) { om_dst1_direct(n, howmany, data, stride, dist); return; }
  const int H = M / 2;
  const om_fft_plan* p = fft_plan_get(H);
  const double* s = sin_get(M); /* s[m] = sin(pi m / M) */
  double* y = (double*)malloc(sizeof(double) * (size_t)M);
  double* zr = (double*)malloc(sizeof(double) * (size_t)H);
  double* zi = (double*)malloc(sizeof(double) * (size_t)H);
  for (int h = 0; h < howmany; ++h) {
    double* x = data + (size_t)h * stride;
#define X1(j) x[(size_t)((j) - 1) * dist] /* 1-based access, 1 <= j <= n */
    y[0] = 0.0;
    for (int j = 1; j < M; ++j) {
      const double a = X1(j), b = X1(M - j);
      y[j] = s[j] * (a + b) + 0.5 * (a - b);
    }
    for (int m = 0; m < H; ++m) { zr[m] = y[2 * m]; zi[m] = y[2 * m + 1]; }
    fft_exec(p, zr, zi);
    /* split: F_k = (Z_k + conj Z_{H-k})/2 - i/2 e^{-2 pi i k/M} (Z_k - conj Z_{H-k}) */
    /* twiddle e^{-2 pi i k / M}: cos = s[(2k + H)... ] use sin table of M:   */
    /* cos(2 pi k/M) = sin(pi (2k + M/2)/M), sin(2 pi k/M) = sin(pi 2k/M)     */
    double run = 0.0;
    for (int k = 0; k < H; ++k) {
      const int kk = (H - k) % H;
      const double ar = zr[k], ai = zi[k];
      const double br = zr[kk], bi = -zi[kk];        /* conj Z_{H-k} */
      const double er = 0.5 * (ar + br), ei = 0.5 * (ai + bi);
      const double dr = ar - br, di = ai - bi;
      const double c = s[(2 * k + H) % (2 * M)];      /* cos(2 pi k/M) */
      const double sn = s[(2 * k) % (2 * M)];         /* sin(2 pi k/M) */
      /* -i/2 (c - i sn)(dr + i di) = -i/2 [(c dr + sn di) + i (c di - sn dr)]
       *                           = 1/2 (c di - sn dr) - i/2 (c dr + sn di) */
      const double Rk = er + 0.5 * (c * di - sn * dr);
      const double Ik = ei - 0.5 * (c * dr + sn * di);
      if (k == 0) run = Rk; else run += 2.0 * Rk;
      X1(2 * k + 1) = run;                             /* Y_{2k+1} */
      if (k > 0) X1(2 * k) = -2.0 * Ik;                /* Y_{2k}   */
    }
#undef X1
  }
  free(y); free(zr); free(zi);
}

void om_dst1(int n, int howmany, double* data, int stride, int dist) {
  const int M = n + 1;
  if (M >= 4 && !(M & (M - 1))) om_dst1_fast(n, howmany, data, stride, dist);
  else om_dst1_direct(n, howmany, data, stride, dist);
}

void om_dst2(int n0, int n1, double* data, int fast) {
  if (fast) {
    om_dst1(n1, n0, data, n1, 1);   /* rows    */
    om_dst1(n0, n1, data, 1, n1);   /* columns */
  } else {
    om_dst1_direct(n1, n0, data, n1, 1);
    om_dst1_direct(n0, n1, data, 1, n1);
  }
}

/* ------------------------------------------------------------ eigensolver */

/* Cyclic Jacobi on a symmetric n x n matrix s (row-major, destroyed):
 * eigenvalues to w, orthonormal eigenvectors to the columns of u. */
static void jacobi_sym(int n, double* s, double* w, double* u) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) u[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += s[i * n + j] * s[i * n + j];
        if (i != j) off += s[i * n + j] * s[i * n + j];
      }
    if (off <= 1e-300 || off <= 1e-34 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = s[p * n + q];
        if (apq == 0.0) continue;
        const double app = s[p * n + p], aqq = s[q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) /
                         (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; ++k) { /* columns p,q */
          const double skp = s[k * n + p], skq = s[k * n + q];
          s[k * n + p] = c * skp - sn * skq;
          s[k * n + q] = sn * skp + c * skq;
        }
        for (int k = 0; k < n; ++k) { /* rows p,q */
          const double spk = s[p * n + k], sqk = s[q * n + k];
          s[p * n + k] = c * spk - sn * sqk;
          s[q * n + k] = sn * spk + c * sqk;
        }
        for (int k = 0; k < n; ++k) {
          const double ukp = u[k * n + p], ukq = u[k * n + q];
          u[k * n + p] = c * ukp - sn * ukq;
          u[k * n + q] = sn * ukp + c * ukq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = s[i * n + i];
}

int om_tridiag_eig(int n, const double* a, double* w, double* vl, double* vr) {
  /* check the tridiagonal form */
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if ((j > i + 1 || j < i - 1) && a[i * n + j] != 0.0) return -1;
  double* d = (double*)malloc(sizeof(double) * (size_t)n);
  double* s = (double*)calloc((size_t)n * n, sizeof(double));
  double* u = (double*)malloc(sizeof(double) * (size_t)n * n);
  d[0] = 1.0;
  for (int i = 0; i + 1 < n; ++i) {
    const double up = a[i * n + i + 1], lo = a[(i + 1) * n + i];
    const double pr = up * lo;
    if (pr > 0.0) {
      d[i + 1] = d[i] * sqrt(up / lo); /* d_i^2 up = d_{i+1}^2 lo */
      const double off = (up > 0 ? 1.0 : -1.0) * sqrt(pr);
      s[i * n + i + 1] = off;
      s[(i + 1) * n + i] = off;
    } else if (up == 0.0 && lo == 0.0) {
      d[i + 1] = d[i];
    } else {
      free(d); free(s); free(u);
      return -1;
    }
  }
  for (int i = 0; i < n; ++i) s[i * n + i] = a[i * n + i];
  jacobi_sym(n, s, w, u);
  /* A = D^-1 S D: right vectors D^-1 u, left vectors D u */
  for (int m = 0; m < n; ++m) {
    double nr = 0.0, nl = 0.0;
    for (int k = 0; k < n; ++k) {
      vr[k * n + m] = u[k * n + m] / d[k];
      vl[k * n + m] = u[k * n + m] * d[k];
      nr += vr[k * n + m] * vr[k * n + m];
      nl += vl[k * n + m] * vl[k * n + m];
    }
    nr = sqrt(nr); nl = sqrt(nl);
    for (int k = 0; k < n; ++k) { vr[k * n + m] /= nr; vl[k * n + m] /= nl; }
  }
  free(d); free(s); free(u);
  return 0;
}
