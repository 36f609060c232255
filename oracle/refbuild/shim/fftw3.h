/* Test-infrastructure shim (oracle build only).
 *
 * FFTW is not installed in this image.  lyspeq uses FFTs to build the
 * signal lookup table (not reached here) and to deconvolve resolution-matrix
 * rows (RealField::deconvolveSinc).  gsl_fftw_stubs.cpp defines the 1-D
 * real-to-complex and complex-to-real transforms by their definition.
 */
#ifndef LQG_ORACLE_SHIM_FFTW3_H
#define LQG_ORACLE_SHIM_FFTW3_H
typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;
#define FFTW_MEASURE 0U
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_REDFT00 3
typedef int fftw_r2r_kind;
fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out, fftw_r2r_kind kind, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
