// Build shim: GSL status code used by the reference's arc-length ODE.
#ifndef ORACLE_SHIM_GSL_ERRNO_H
#define ORACLE_SHIM_GSL_ERRNO_H
#define GSL_SUCCESS 0
#endif
