/* Stand-in for the GSL spline API (test infrastructure only): a natural cubic spline (shim.c). The
 * periodic path builds the redshift-distance table in create_grids (main.c:1233-1248) and never
 * evaluates it; the survey path evaluates it and the number-density spline. */
#ifndef CAPOW_SHIM_GSL_SPLINE_H
#define CAPOW_SHIM_GSL_SPLINE_H
#include <stddef.h>
typedef struct { int unused; } gsl_interp_type;
typedef struct { int unused; } gsl_interp_accel;
typedef struct { size_t n; double *x, *y, *m; } gsl_spline;
extern const gsl_interp_type *gsl_interp_cspline;
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *t, size_t n);
int gsl_spline_init(gsl_spline *s, const double *x, const double *y, size_t n);
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *s);
#endif
