/* Declarations of the four LAPACKE routines the reference calls.  The
 * definitions in lapacke_shim.c are small dense solvers written for the oracle
 * build (row-major only). */
#ifndef GLASS_ORACLE_SHIM_LAPACKE_H
#define GLASS_ORACLE_SHIM_LAPACKE_H
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
int LAPACKE_dgeev(int layout, char jobvl, char jobvr, int n, double *a, int lda,
                  double *wr, double *wi, double *vl, int ldvl, double *vr, int ldvr);
int LAPACKE_dgetrf(int layout, int m, int n, double *a, int lda, int *ipiv);
int LAPACKE_dgetri(int layout, int n, double *a, int lda, const int *ipiv);
int LAPACKE_dpotrf(int layout, char uplo, int n, double *a, int lda);
#endif
