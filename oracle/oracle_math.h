/*
 * oracle_math.h -- CPU numerics shared by the oracle (test infrastructure
 * only: used by tests/, the smoke check and the CPU baseline of bench.py,
 * never by the product library).
 *
 * - DST-I (FFTW's RODFT00 definition, the transform the reference plans at
 *   src/elliptic.h:63-66):  Y_k = 2 sum_{j=0}^{n-1} X_j sin(pi (j+1)(k+1)/(n+1)).
 *   Two implementations: a direct O(n^2) sum with an exactly reduced sine
 *   table, and an O(n log n) one through a half-length complex FFT (used when
 *   n+1 is a power of two).
 * - eigen-decomposition of a real tridiagonal matrix whose off-diagonal
 *   products are positive (the reference's stretching matrix,
 *   src/eigmode.h:105-119), by diagonal similarity to a symmetric matrix and
 *   cyclic Jacobi rotations.
 */
#ifndef QGW_ORACLE_MATH_H
#define QGW_ORACLE_MATH_H

#ifdef __cplusplus
extern "C" {
#endif

/* In-place DST-I of `howmany` rows of length n, rows `stride` doubles apart,
 * elements `dist` doubles apart within a row. */
void om_dst1_direct(int n, int howmany, double* data, int stride, int dist);
void om_dst1_fast(int n, int howmany, double* data, int stride, int dist);
/* Fast when n+1 is a power of two, direct otherwise. */
void om_dst1(int n, int howmany, double* data, int stride, int dist);

/* 2-D DST-I of a row-major (n0 rows, n1 columns) array in place. */
void om_dst2(int n0, int n1, double* data, int fast);

/* 2-D real DFT pair with FFTW's conventions (fftw_plan_dft_r2c_2d /
 * fftw_plan_dft_c2r_2d, in place, the layout the reference's periodic
 * inversion uses, src/elliptic.h:32-47,103-118): data holds n0 rows of
 * 2*(n1/2+1) doubles; r2c reads n1 reals per row and writes n1/2+1 complex
 * values per row,
 *     Y[k0][k1] = sum_{j0,j1} x[j0][j1] exp(-2 pi i (j0 k0/n0 + j1 k1/n1));
 * c2r is the unnormalised inverse (c2r(r2c(x)) = n0 n1 x) for Hermitian
 * input: after the backward transform along the first dimension, the
 * k1 = 0 and k1 = n1/2 entries of each row enter by their real parts.
 * Direct O(n^2) sums per dimension with exactly reduced twiddle tables
 * (accurate to a few ulp). */
void om_dft_r2c_2d(int n0, int n1, double* data);
void om_dft_c2r_2d(int n0, int n1, double* data);
/* The same, through a radix-2 FFT when fast != 0 and both sizes are powers
 * of two (agrees with the direct sums to round-off). */
void om_dft_r2c_2d_any(int n0, int n1, double* data, int fast);
void om_dft_c2r_2d_any(int n0, int n1, double* data, int fast);

/* Eigen-decomposition of a row-major n x n matrix a that is tridiagonal
 * with a[i][i+1]*a[i+1][i] > 0 (or both zero).  Outputs as LAPACK dgeev with
 * row-major storage: eigenvalues w (unsorted), right eigenvectors in the
 * columns of vr, left eigenvectors in the columns of vl, each column of unit
 * 2-norm.  Returns 0, or -1 when a is not of that form. */
int om_tridiag_eig(int n, const double* a, double* w, double* vl, double* vr);

#ifdef __cplusplus
}
#endif
#endif
