// Build shim: the subset of GSL's ODE API used by AnalyticCurve's
// arc-length parametrisation.  The stand-in integrates with fixed-size
// classical RK4 sub-steps; arc-length partitions are outside the parity path.
#ifndef ORACLE_SHIM_GSL_ODEIV_H
#define ORACLE_SHIM_GSL_ODEIV_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
  int (*function)(double t, const double y[], double dydt[], void* params);
  int (*jacobian)(double t, const double y[], double* dfdy, double dfdt[],
                  void* params);
  size_t dimension;
  void* params;
} gsl_odeiv_system;
typedef struct { int unused; } gsl_odeiv_step_type;
typedef struct { size_t dim; } gsl_odeiv_step;
typedef struct { double eps; } gsl_odeiv_control;
typedef struct { size_t dim; } gsl_odeiv_evolve;
extern const gsl_odeiv_step_type* gsl_odeiv_step_rk2;
gsl_odeiv_step* gsl_odeiv_step_alloc(const gsl_odeiv_step_type* T, size_t dim);
void gsl_odeiv_step_free(gsl_odeiv_step* s);
gsl_odeiv_control* gsl_odeiv_control_y_new(double eps_abs, double eps_rel);
void gsl_odeiv_control_free(gsl_odeiv_control* c);
gsl_odeiv_evolve* gsl_odeiv_evolve_alloc(size_t dim);
void gsl_odeiv_evolve_free(gsl_odeiv_evolve* e);
int gsl_odeiv_evolve_apply(gsl_odeiv_evolve* e, gsl_odeiv_control* con,
                           gsl_odeiv_step* step, const gsl_odeiv_system* dydt,
                           double* t, double t1, double* h, double y[]);
#ifdef __cplusplus
}
#endif
#endif
