/* Test-infrastructure shim (oracle build only).
 *
 * LAPACKE subset used by lyspeq, forwarded to the `scipy_LAPACKE_*` exports
 * of scipy's bundled OpenBLAS (LP64: lapack_int is a 32-bit int).
 */
#ifndef LQG_ORACLE_SHIM_LAPACKE_H
#define LQG_ORACLE_SHIM_LAPACKE_H

typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

#ifdef __cplusplus
extern "C" {
#endif

lapack_int scipy_LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double *a,
                                lapack_int lda, lapack_int *ipiv);
lapack_int scipy_LAPACKE_dgetri(int layout, lapack_int n, double *a, lapack_int lda,
                                const lapack_int *ipiv);
lapack_int scipy_LAPACKE_dpotrf(int layout, char uplo, lapack_int n, double *a,
                                lapack_int lda);
lapack_int scipy_LAPACKE_dpotri(int layout, char uplo, lapack_int n, double *a,
                                lapack_int lda);
lapack_int scipy_LAPACKE_dgesv(int layout, lapack_int n, lapack_int nrhs, double *a,
                               lapack_int lda, lapack_int *ipiv, double *b,
                               lapack_int ldb);
lapack_int scipy_LAPACKE_dposv(int layout, char uplo, lapack_int n, lapack_int nrhs,
                               double *a, lapack_int lda, double *b, lapack_int ldb);
lapack_int scipy_LAPACKE_dgesvd(int layout, char jobu, char jobvt, lapack_int m,
                                lapack_int n, double *a, lapack_int lda, double *s,
                                double *u, lapack_int ldu, double *vt,
                                lapack_int ldvt, double *superb);
lapack_int scipy_LAPACKE_dsyevr(int layout, char jobz, char range, char uplo,
                                lapack_int n, double *a, lapack_int lda, double vl,
                                double vu, lapack_int il, lapack_int iu,
                                double abstol, lapack_int *m, double *w, double *z,
                                lapack_int ldz, lapack_int *isuppz);

#ifdef __cplusplus
}
#endif

#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_dgetri scipy_LAPACKE_dgetri
#define LAPACKE_dpotrf scipy_LAPACKE_dpotrf
#define LAPACKE_dpotri scipy_LAPACKE_dpotri
#define LAPACKE_dgesv scipy_LAPACKE_dgesv
#define LAPACKE_dposv scipy_LAPACKE_dposv
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_dsyevr scipy_LAPACKE_dsyevr

#endif
