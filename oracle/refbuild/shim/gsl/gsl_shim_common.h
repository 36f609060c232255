/* Test-infrastructure shim (oracle build only).
 *
 * GSL is not installed in this image.  Most GSL routines that lyspeq calls
 * are off the per-chunk QMLE path (QAWO integration and FFTs build the S/Q
 * lookup tables).  This header declares the types and prototypes those
 * translation units use so that they compile.  gsl_fftw_stubs.cpp implements
 * the 1-D interpolators (natural cubic spline, linear), which oversample
 * resolution matrices, and throws for everything else.
 */
#ifndef LQG_ORACLE_SHIM_GSL_COMMON_H
#define LQG_ORACLE_SHIM_GSL_COMMON_H
#include <cstddef>
#include <math.h>  /* real GSL headers pull in math.h; lyspeq relies on it */

#define GSL_SUCCESS 0
#define GSL_EDOM 1
#define GSL_EROUND 18
#define GSL_ETABLE 26
#define GSL_EDIVERGE 22

typedef void gsl_error_handler_t(const char *, const char *, int, int);
gsl_error_handler_t *gsl_set_error_handler_off(void);
const char *gsl_strerror(int gsl_errno);

typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;

typedef struct gsl_integration_workspace_s gsl_integration_workspace;
typedef struct gsl_integration_qawo_table_s gsl_integration_qawo_table;
typedef enum { GSL_INTEG_COSINE, GSL_INTEG_SINE } gsl_integration_qawo_enum;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
gsl_integration_qawo_table *gsl_integration_qawo_table_alloc(
    double omega, double L, gsl_integration_qawo_enum sine, size_t n);
int gsl_integration_qawo_table_set(gsl_integration_qawo_table *t, double omega,
                                   double L, gsl_integration_qawo_enum sine);
int gsl_integration_qawo_table_set_length(gsl_integration_qawo_table *t, double L);
void gsl_integration_qawo_table_free(gsl_integration_qawo_table *t);
int gsl_integration_qawo(gsl_function *f, double a, double epsabs, double epsrel,
                         size_t limit, gsl_integration_workspace *w,
                         gsl_integration_qawo_table *wf, double *result, double *abserr);
int gsl_integration_qawf(gsl_function *f, double a, double epsabs, size_t limit,
                         gsl_integration_workspace *w, gsl_integration_workspace *wc,
                         gsl_integration_qawo_table *wf, double *result, double *abserr);

typedef struct { const char *name; unsigned int min_size; } gsl_interp_type;
extern const gsl_interp_type *gsl_interp_linear;
extern const gsl_interp_type *gsl_interp_cspline;
typedef struct { size_t cache; size_t miss_count; size_t hit_count; } gsl_interp_accel;
typedef struct { const gsl_interp_type *type; double xmin, xmax; size_t size; void *state; } gsl_interp;
typedef struct { gsl_interp *interp; double *x; double *y; size_t size; } gsl_spline;

gsl_interp_accel *gsl_interp_accel_alloc(void);
int gsl_interp_accel_reset(gsl_interp_accel *a);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n);
int gsl_interp_init(gsl_interp *obj, const double xa[], const double ya[], size_t size);
double gsl_interp_eval(const gsl_interp *obj, const double xa[], const double ya[],
                       double x, gsl_interp_accel *a);
void gsl_interp_free(gsl_interp *interp);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size);
int gsl_spline_init(gsl_spline *spline, const double xa[], const double ya[], size_t size);
double gsl_spline_eval(const gsl_spline *spline, double x, gsl_interp_accel *a);
double gsl_spline_eval_deriv(const gsl_spline *spline, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *spline);

typedef struct { const char *name; unsigned int min_size; } gsl_interp2d_type;
extern const gsl_interp2d_type *gsl_interp2d_bilinear;
extern const gsl_interp2d_type *gsl_interp2d_bicubic;
typedef struct { const gsl_interp2d_type *type; double xmin, xmax, ymin, ymax;
                 size_t xsize, ysize; void *state; } gsl_interp2d;
typedef struct { gsl_interp2d interp_object; double *xarr; double *yarr; double *zarr; } gsl_spline2d;
gsl_spline2d *gsl_spline2d_alloc(const gsl_interp2d_type *T, size_t xsize, size_t ysize);
int gsl_spline2d_init(gsl_spline2d *interp, const double xa[], const double ya[],
                      const double za[], size_t xsize, size_t ysize);
void gsl_spline2d_free(gsl_spline2d *interp);
double gsl_spline2d_eval(const gsl_spline2d *interp, const double x, const double y,
                         gsl_interp_accel *xa, gsl_interp_accel *ya);
int gsl_spline2d_eval_e(const gsl_spline2d *interp, const double x, const double y,
                        gsl_interp_accel *xa, gsl_interp_accel *ya, double *z);
double gsl_spline2d_eval_deriv_x(const gsl_spline2d *interp, const double x, const double y,
                                 gsl_interp_accel *xa, gsl_interp_accel *ya);
int gsl_spline2d_eval_deriv_x_e(const gsl_spline2d *interp, const double x, const double y,
                                gsl_interp_accel *xa, gsl_interp_accel *ya, double *z);
double gsl_spline2d_eval_deriv_y(const gsl_spline2d *interp, const double x, const double y,
                                 gsl_interp_accel *xa, gsl_interp_accel *ya);
int gsl_spline2d_eval_deriv_y_e(const gsl_spline2d *interp, const double x, const double y,
                                gsl_interp_accel *xa, gsl_interp_accel *ya, double *z);
#endif
