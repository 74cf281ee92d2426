/* Stand-in for the GSL integration API (test infrastructure only): adaptive Gauss-Kronrod (shim.c). */
#ifndef CAPOW_SHIM_GSL_INTEGRATION_H
#define CAPOW_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel, size_t limit,
                         gsl_integration_workspace *w, double *result, double *abserr);
#endif
