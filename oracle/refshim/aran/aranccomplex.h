/* aran/aranccomplex.h -- TEST INFRASTRUCTURE: what configure makes of the
 * reference's aran/aranccomplex.h.in for a C build: C99 complex numbers. */
#ifndef ORACLE_SHIM_ARANCCOMPLEX_H
#define ORACLE_SHIM_ARANCCOMPLEX_H
#include <complex.h>
#endif
