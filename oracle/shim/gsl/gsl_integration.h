// Build shim: the subset of GSL's integration API used by Curve::Length.
// The stand-in (oracle/shim/shim_support.c) is a composite Gauss-Legendre
// rule, not GSL's adaptive QAG; curve lengths are outside the parity path.
#ifndef ORACLE_SHIM_GSL_INTEGRATION_H
#define ORACLE_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { int unused; } gsl_integration_workspace;
typedef struct {
  double (*function)(double x, void* params);
  void* params;
} gsl_function;
enum { GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21, GSL_INTEG_GAUSS31,
       GSL_INTEG_GAUSS41, GSL_INTEG_GAUSS51, GSL_INTEG_GAUSS61 };
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace* w);
int gsl_integration_qag(const gsl_function* f, double a, double b,
                        double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace* w, double* result,
                        double* abserr);
#ifdef __cplusplus
}
#endif
#endif
