/* Test-infrastructure shim (oracle build only).
 *
 * Declares the CBLAS subset that lyspeq's hot path calls and forwards each
 * call to the `scipy_cblas_*` exports of the OpenBLAS copy bundled with scipy
 * (LP64 interface).  Enum values follow the CBLAS standard.  Nothing in the
 * product links against this header.
 */
#ifndef LQG_ORACLE_SHIM_CBLAS_H
#define LQG_ORACLE_SHIM_CBLAS_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;

double scipy_cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
double scipy_cblas_dnrm2(int n, const double *x, int incx);
void scipy_cblas_daxpy(int n, double a, const double *x, int incx, double *y, int incy);
void scipy_cblas_dscal(int n, double a, double *x, int incx);
void scipy_cblas_dcopy(int n, const double *x, int incx, double *y, int incy);
void scipy_cblas_dgemv(int order, int trans, int m, int n, double alpha,
                       const double *a, int lda, const double *x, int incx,
                       double beta, double *y, int incy);
void scipy_cblas_dsymv(int order, int uplo, int n, double alpha,
                       const double *a, int lda, const double *x, int incx,
                       double beta, double *y, int incy);
void scipy_cblas_dger(int order, int m, int n, double alpha, const double *x,
                      int incx, const double *y, int incy, double *a, int lda);
void scipy_cblas_dsyr(int order, int uplo, int n, double alpha, const double *x,
                      int incx, double *a, int lda);
void scipy_cblas_dgemm(int order, int ta, int tb, int m, int n, int k,
                       double alpha, const double *a, int lda, const double *b,
                       int ldb, double beta, double *c, int ldc);
void scipy_cblas_dsymm(int order, int side, int uplo, int m, int n,
                       double alpha, const double *a, int lda, const double *b,
                       int ldb, double beta, double *c, int ldc);

#ifdef __cplusplus
}
#endif

static inline double cblas_ddot(int n, const double *x, int incx, const double *y, int incy)
{ return scipy_cblas_ddot(n, x, incx, y, incy); }
static inline double cblas_dnrm2(int n, const double *x, int incx)
{ return scipy_cblas_dnrm2(n, x, incx); }
static inline void cblas_daxpy(int n, double a, const double *x, int incx, double *y, int incy)
{ scipy_cblas_daxpy(n, a, x, incx, y, incy); }
static inline void cblas_dscal(int n, double a, double *x, int incx)
{ scipy_cblas_dscal(n, a, x, incx); }
static inline void cblas_dcopy(int n, const double *x, int incx, double *y, int incy)
{ scipy_cblas_dcopy(n, x, incx, y, incy); }
static inline void cblas_dgemv(int order, int trans, int m, int n, double alpha,
                               const double *a, int lda, const double *x, int incx,
                               double beta, double *y, int incy)
{ scipy_cblas_dgemv(order, trans, m, n, alpha, a, lda, x, incx, beta, y, incy); }
static inline void cblas_dsymv(int order, int uplo, int n, double alpha,
                               const double *a, int lda, const double *x, int incx,
                               double beta, double *y, int incy)
{ scipy_cblas_dsymv(order, uplo, n, alpha, a, lda, x, incx, beta, y, incy); }
static inline void cblas_dger(int order, int m, int n, double alpha, const double *x,
                              int incx, const double *y, int incy, double *a, int lda)
{ scipy_cblas_dger(order, m, n, alpha, x, incx, y, incy, a, lda); }
static inline void cblas_dsyr(int order, int uplo, int n, double alpha, const double *x,
                              int incx, double *a, int lda)
{ scipy_cblas_dsyr(order, uplo, n, alpha, x, incx, a, lda); }
static inline void cblas_dgemm(int order, int ta, int tb, int m, int n, int k,
                               double alpha, const double *a, int lda, const double *b,
                               int ldb, double beta, double *c, int ldc)
{ scipy_cblas_dgemm(order, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc); }
static inline void cblas_dsymm(int order, int side, int uplo, int m, int n,
                               double alpha, const double *a, int lda, const double *b,
                               int ldb, double beta, double *c, int ldc)
{ scipy_cblas_dsymm(order, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc); }

#endif
