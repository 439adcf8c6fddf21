// Build shim: GSL's real-argument Bessel functions J0, J1, Y0, Y1.  The
// oracle maps them onto the POSIX libm functions j0/j1/y0/y1 (definitions
// in oracle/shim/shim_support.c).
#ifndef ORACLE_SHIM_GSL_SF_BESSEL_H
#define ORACLE_SHIM_GSL_SF_BESSEL_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_J0(double x);
double gsl_sf_bessel_J1(double x);
double gsl_sf_bessel_Y0(double x);
double gsl_sf_bessel_Y1(double x);
#ifdef __cplusplus
}
#endif
#endif
