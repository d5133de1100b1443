/*
 * lapacke.h (oracle shim) -- declares LAPACKE_dgeev, the only LAPACK routine
 * the reference calls (src/eigmode.h:145-146).  shim.c implements it for the
 * matrices the reference builds (real tridiagonal with positive off-diagonal
 * products) with project code; test infrastructure only.
 */
#ifndef QGW_SHIM_LAPACKE_H
#define QGW_SHIM_LAPACKE_H
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int LAPACKE_dgeev(int matrix_layout, char jobvl, char jobvr, lapack_int n,
                         double* a, lapack_int lda, double* wr, double* wi,
                         double* vl, lapack_int ldvl, double* vr, lapack_int ldvr);
#endif
