// Test-infrastructure shim (oracle build only): definitions for the GSL and
// FFTW entry points declared in gsl/gsl_shim_common.h and fftw3.h.
//
// Two families are reached by lyspeq's resolution-matrix preprocessing and
// are implemented here from their mathematical definitions:
//  * gsl_interp with gsl_interp_cspline: the natural cubic spline (second
//    derivative zero at both ends), used by Resolution::oversample
//    (mathtools/matrix_helper.cpp:1008-1073); gsl_interp_linear as well.
//    Outside [x_0, x_{n-1}] the evaluation returns NaN, as GSL does with its
//    error handler off.  gsl_spline (value and first derivative) on top of
//    it, for the mean flux F-bar(z) of a MeanFluxFile (conv::setMeanFlux,
//    core/fiducial_cosmology.cpp:131-165).
//  * fftw_plan_dft_r2c_1d / fftw_plan_dft_c2r_1d with fftw_execute: the
//    unnormalised discrete Fourier transform of FFTW's definition, evaluated
//    as a direct O(n^2) sum (RealField::deconvolveSinc transforms 21 points
//    per resolution-matrix row, mathtools/real_field.cpp:78-110).
// Everything else (QAWO integration, 2-D splines, r2r transforms) is used only
// to build lookup tables and throws if it is ever reached.
#include "gsl/gsl_shim_common.h"
#include "fftw3.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

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

gsl_interp_accel *gsl_interp_accel_alloc(void) { return new gsl_interp_accel{0, 0, 0}; }
int gsl_interp_accel_reset(gsl_interp_accel *a) {
    if (a) *a = gsl_interp_accel{0, 0, 0};
    return GSL_SUCCESS;
}
void gsl_interp_accel_free(gsl_interp_accel *a) { delete a; }

namespace {
// State of a natural cubic spline: the second derivatives M_i at the knots.
struct CsplineState { std::vector<double> m; };

// Index i with xa[i] <= x < xa[i+1] (the last interval for x == xa[n-1]).
size_t find_interval(const double xa[], size_t n, double x) {
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        size_t mid = (lo + hi) / 2;
        if (xa[mid] > x) hi = mid; else lo = mid;
    }
    return lo;
}
}  // namespace

gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n) {
    if (T != gsl_interp_cspline && T != gsl_interp_linear) unavailable("this gsl_interp type");
    if (n < T->min_size) throw std::invalid_argument("gsl_interp_alloc: too few points");
    auto *g = new gsl_interp{T, 0.0, 0.0, n, nullptr};
    if (T == gsl_interp_cspline) g->state = new CsplineState{std::vector<double>(n, 0.0)};
    return g;
}

// Natural cubic spline: for the interior knots
//   h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1}
//     = 6 ((y_{i+1} - y_i) / h_i - (y_i - y_{i-1}) / h_{i-1}),  M_0 = M_{n-1} = 0,
// solved by forward elimination and back substitution (the system is
// diagonally dominant).
int gsl_interp_init(gsl_interp *g, const double xa[], const double ya[], size_t n) {
    if (!g || n != g->size) throw std::invalid_argument("gsl_interp_init: size mismatch");
    for (size_t i = 1; i < n; ++i)
        if (!(xa[i] > xa[i - 1])) throw std::invalid_argument("gsl_interp_init: x not increasing");
    g->xmin = xa[0];
    g->xmax = xa[n - 1];
    if (g->type != gsl_interp_cspline) return GSL_SUCCESS;
    std::vector<double> &m = static_cast<CsplineState *>(g->state)->m;
    std::fill(m.begin(), m.end(), 0.0);
    if (n < 3) return GSL_SUCCESS;
    const size_t k = n - 2;                       // unknowns M_1 .. M_{n-2}
    std::vector<double> diag(k), upper(k), rhs(k);
    for (size_t j = 0; j < k; ++j) {
        const size_t i = j + 1;
        const double h0 = xa[i] - xa[i - 1], h1 = xa[i + 1] - xa[i];
        diag[j] = 2.0 * (h0 + h1);
        upper[j] = h1;
        rhs[j] = 6.0 * ((ya[i + 1] - ya[i]) / h1 - (ya[i] - ya[i - 1]) / h0);
    }
    for (size_t j = 1; j < k; ++j) {
        const double lower = xa[j + 1] - xa[j];   // h_{i-1} of row j (i = j + 1)
        const double f = lower / diag[j - 1];
        diag[j] -= f * upper[j - 1];
        rhs[j] -= f * rhs[j - 1];
    }
    m[k] = rhs[k - 1] / diag[k - 1];
    for (size_t j = k - 1; j-- > 0;) m[j + 1] = (rhs[j] - upper[j] * m[j + 2]) / diag[j];
    return GSL_SUCCESS;
}

double gsl_interp_eval(const gsl_interp *g, const double xa[], const double ya[], double x,
                       gsl_interp_accel *a) {
    if (!(x >= g->xmin && x <= g->xmax)) return std::numeric_limits<double>::quiet_NaN();
    const size_t i = find_interval(xa, g->size, x);
    if (a) a->cache = i;
    const double h = xa[i + 1] - xa[i];
    if (g->type == gsl_interp_linear) return ya[i] + (ya[i + 1] - ya[i]) * ((x - xa[i]) / h);
    const std::vector<double> &m = static_cast<const CsplineState *>(g->state)->m;
    // Cubic on [x_i, x_{i+1}] with second derivatives M_i, M_{i+1} at the ends.
    const double t1 = xa[i + 1] - x, t0 = x - xa[i];
    return (m[i] * t1 * t1 * t1 + m[i + 1] * t0 * t0 * t0) / (6.0 * h)
         + (ya[i] / h - m[i] * h / 6.0) * t1 + (ya[i + 1] / h - m[i + 1] * h / 6.0) * t0;
}

void gsl_interp_free(gsl_interp *g) {
    if (!g) return;
    if (g->type == gsl_interp_cspline) delete static_cast<CsplineState *>(g->state);
    delete g;
}
// gsl_spline: a gsl_interp that keeps its own copy of the knots, as GSL's
// does; lyspeq's Interpolation (mathtools/interpolation.cpp) reads the mean
// flux F-bar(z) of a MeanFluxFile through it, and its first derivative to
// continue the curve past the ends.
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n) {
    return new gsl_spline{gsl_interp_alloc(T, n), new double[n], new double[n], n};
}
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n) {
    if (!s || n != s->size) throw std::invalid_argument("gsl_spline_init: size mismatch");
    std::copy(xa, xa + n, s->x);
    std::copy(ya, ya + n, s->y);
    return gsl_interp_init(s->interp, s->x, s->y, n);
}
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a) {
    return gsl_interp_eval(s->interp, s->x, s->y, x, a);
}
// d/dx of the cubic above: the derivatives of t1^3 and t0^3 are -3 t1^2 and
// 3 t0^2, of t1 and t0 -1 and 1.
double gsl_spline_eval_deriv(const gsl_spline *s, double x, gsl_interp_accel *a) {
    const gsl_interp *g = s->interp;
    const double *xa = s->x, *ya = s->y;
    if (!(x >= g->xmin && x <= g->xmax)) return std::numeric_limits<double>::quiet_NaN();
    const size_t i = find_interval(xa, g->size, x);
    if (a) a->cache = i;
    const double h = xa[i + 1] - xa[i];
    if (g->type == gsl_interp_linear) return (ya[i + 1] - ya[i]) / h;
    const std::vector<double> &m = static_cast<const CsplineState *>(g->state)->m;
    const double t1 = xa[i + 1] - x, t0 = x - xa[i];
    return (3.0 * m[i + 1] * t0 * t0 - 3.0 * m[i] * t1 * t1) / (6.0 * h)
         - (ya[i] / h - m[i] * h / 6.0) + (ya[i + 1] / h - m[i + 1] * h / 6.0);
}
void gsl_spline_free(gsl_spline *s) {
    if (!s) return;
    gsl_interp_free(s->interp);
    delete[] s->x;
    delete[] s->y;
    delete s;
}

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

// A plan remembers the transform, its length and the two arrays, as FFTW's does.
struct fftw_plan_s {
    int kind;   // 0: r2c, 1: c2r
    int n;
    double *real;
    fftw_complex *cplx;
};

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned) {
    return new fftw_plan_s{0, n, in, out};
}
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex *in, double *out, unsigned) {
    return new fftw_plan_s{1, n, out, in};
}
fftw_plan fftw_plan_r2r_1d(int, double *, double *, fftw_r2r_kind, unsigned) { return nullptr; }

// r2c: X_k = sum_j x_j exp(-2 pi i j k / n), k = 0 .. n/2.
// c2r: x_j = sum_{k=0}^{n-1} X_k exp(+2 pi i j k / n) with X_{n-k} = conj(X_k),
//      unnormalised; the imaginary parts of X_0 and X_{n/2} are ignored.
void fftw_execute(const fftw_plan p) {
    if (!p) unavailable("fftw_execute of this plan");
    const int n = p->n;
    const double w = 2.0 * M_PI / n;
    if (p->kind == 0) {
        std::vector<double> x(p->real, p->real + n);
        for (int k = 0; k <= n / 2; ++k) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < n; ++j) {
                const double ang = w * (double) ((long long) j * k % n);
                re += x[j] * std::cos(ang);
                im -= x[j] * std::sin(ang);
            }
            p->cplx[k][0] = re;
            p->cplx[k][1] = im;
        }
    } else {
        const int nh = n / 2 + 1;
        std::vector<double> re(nh), im(nh);
        for (int k = 0; k < nh; ++k) { re[k] = p->cplx[k][0]; im[k] = p->cplx[k][1]; }
        for (int j = 0; j < n; ++j) {
            double s = re[0];
            for (int k = 1; k < nh; ++k) {
                const double ang = w * (double) ((long long) j * k % n);
                if (2 * k == n) s += re[k] * std::cos(ang);
                else s += 2.0 * (re[k] * std::cos(ang) - im[k] * std::sin(ang));
            }
            p->real[j] = s;
        }
    }
}
void fftw_destroy_plan(fftw_plan p) { delete p; }
