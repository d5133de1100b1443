/*
 * fftw3.h (oracle shim) -- declares the subset of the FFTW 3 API that the
 * reference calls (src/elliptic.h:29-74,76-155,157-169, src/forcing.h:67-219), so
 * that the reference compiles unchanged when FFTW is not installed.  The
 * implementation in shim.c is project code (oracle_math.c); it is test
 * infrastructure only.  Names and signatures follow FFTW's public API.
 */
#ifndef QGW_SHIM_FFTW3_H
#define QGW_SHIM_FFTW3_H
#include <stddef.h>

typedef double fftw_complex[2];
typedef struct shim_fftw_plan_s* fftw_plan;
typedef enum {
  FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2,
  FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6,
  FFTW_RODFT00 = 7, FFTW_RODFT01 = 8, FFTW_RODFT10 = 9, FFTW_RODFT11 = 10
} fftw_r2r_kind;

#define FFTW_MEASURE (0U)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_r2r_2d(int n0, int n1, double* in, double* out,
                           fftw_r2r_kind kind0, fftw_r2r_kind kind1, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);
double* fftw_alloc_real(size_t n);
fftw_complex* fftw_alloc_complex(size_t n);
void fftw_free(void* p);
#endif
