// Build shim: included by the reference's basis header; nothing is used.
#ifndef ORACLE_SHIM_GSL_SF_LEGENDRE_H
#define ORACLE_SHIM_GSL_SF_LEGENDRE_H
#endif
