// Test-infrastructure shim (oracle build only): definitions for the GSL and
// FFTW entry points declared in gsl/gsl_shim_common.h and fftw3.h.  None of
// them is reached on the per-chunk QMLE path with precomputed lookup tables;
// each throws so that an unexpected call is loud instead of silently wrong.
#include "gsl/gsl_shim_common.h"
#include "fftw3.h"

#include <stdexcept>
#include <string>

namespace {
[[noreturn]] void unavailable(const char *what) {
    throw std::runtime_error(std::string("oracle build: ") + what + " is not available");
}
const gsl_interp_type linear_t{"linear", 2}, cspline_t{"cspline", 3};
const gsl_interp2d_type bilinear_t{"bilinear", 2}, bicubic_t{"bicubic", 4};
}  // namespace

const gsl_interp_type *gsl_interp_linear = &linear_t;
const gsl_interp_type *gsl_interp_cspline = &cspline_t;
const gsl_interp2d_type *gsl_interp2d_bilinear = &bilinear_t;
const gsl_interp2d_type *gsl_interp2d_bicubic = &bicubic_t;

gsl_error_handler_t *gsl_set_error_handler_off(void) { return nullptr; }
const char *gsl_strerror(int) { return "gsl error (oracle build)"; }

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t) { unavailable("gsl_integration"); }
void gsl_integration_workspace_free(gsl_integration_workspace *) {}
gsl_integration_qawo_table *gsl_integration_qawo_table_alloc(double, double, gsl_integration_qawo_enum, size_t)
{ unavailable("gsl_integration_qawo"); }
int gsl_integration_qawo_table_set(gsl_integration_qawo_table *, double, double, gsl_integration_qawo_enum)
{ unavailable("gsl_integration_qawo"); }
int gsl_integration_qawo_table_set_length(gsl_integration_qawo_table *, double) { unavailable("gsl_integration_qawo"); }
void gsl_integration_qawo_table_free(gsl_integration_qawo_table *) {}
int gsl_integration_qawo(gsl_function *, double, double, double, size_t, gsl_integration_workspace *,
                         gsl_integration_qawo_table *, double *, double *) { unavailable("gsl_integration_qawo"); }
int gsl_integration_qawf(gsl_function *, double, double, size_t, gsl_integration_workspace *,
                         gsl_integration_workspace *, gsl_integration_qawo_table *, double *, double *)
{ unavailable("gsl_integration_qawf"); }

gsl_interp_accel *gsl_interp_accel_alloc(void) { unavailable("gsl_interp"); }
int gsl_interp_accel_reset(gsl_interp_accel *) { unavailable("gsl_interp"); }
void gsl_interp_accel_free(gsl_interp_accel *) {}
gsl_interp *gsl_interp_alloc(const gsl_interp_type *, size_t) { unavailable("gsl_interp"); }
int gsl_interp_init(gsl_interp *, const double[], const double[], size_t) { unavailable("gsl_interp"); }
double gsl_interp_eval(const gsl_interp *, const double[], const double[], double, gsl_interp_accel *)
{ unavailable("gsl_interp"); }
void gsl_interp_free(gsl_interp *) {}
gsl_spline *gsl_spline_alloc(const gsl_interp_type *, size_t) { unavailable("gsl_spline"); }
int gsl_spline_init(gsl_spline *, const double[], const double[], size_t) { unavailable("gsl_spline"); }
double gsl_spline_eval(const gsl_spline *, double, gsl_interp_accel *) { unavailable("gsl_spline"); }
double gsl_spline_eval_deriv(const gsl_spline *, double, gsl_interp_accel *) { unavailable("gsl_spline"); }
void gsl_spline_free(gsl_spline *) {}

gsl_spline2d *gsl_spline2d_alloc(const gsl_interp2d_type *, size_t, size_t) { unavailable("gsl_spline2d"); }
int gsl_spline2d_init(gsl_spline2d *, const double[], const double[], const double[], size_t, size_t)
{ unavailable("gsl_spline2d"); }
void gsl_spline2d_free(gsl_spline2d *) {}
double gsl_spline2d_eval(const gsl_spline2d *, const double, const double, gsl_interp_accel *, gsl_interp_accel *)
{ unavailable("gsl_spline2d"); }
int gsl_spline2d_eval_e(const gsl_spline2d *, const double, const double, gsl_interp_accel *, gsl_interp_accel *,
                        double *) { unavailable("gsl_spline2d"); }
double gsl_spline2d_eval_deriv_x(const gsl_spline2d *, const double, const double, gsl_interp_accel *,
                                 gsl_interp_accel *) { unavailable("gsl_spline2d"); }
int gsl_spline2d_eval_deriv_x_e(const gsl_spline2d *, const double, const double, gsl_interp_accel *,
                                gsl_interp_accel *, double *) { unavailable("gsl_spline2d"); }
double gsl_spline2d_eval_deriv_y(const gsl_spline2d *, const double, const double, gsl_interp_accel *,
                                 gsl_interp_accel *) { unavailable("gsl_spline2d"); }
int gsl_spline2d_eval_deriv_y_e(const gsl_spline2d *, const double, const double, gsl_interp_accel *,
                                gsl_interp_accel *, double *) { unavailable("gsl_spline2d"); }

fftw_plan fftw_plan_dft_r2c_1d(int, double *, fftw_complex *, unsigned) { return nullptr; }
fftw_plan fftw_plan_dft_c2r_1d(int, fftw_complex *, double *, unsigned) { return nullptr; }
fftw_plan fftw_plan_r2r_1d(int, double *, double *, fftw_r2r_kind, unsigned) { return nullptr; }
void fftw_execute(const fftw_plan) { unavailable("fftw_execute"); }
void fftw_destroy_plan(fftw_plan) {}
