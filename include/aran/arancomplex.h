/* arancomplex.h -- complex types of LibAran (aran/arancomplex.h:31-35). */
#ifndef ARAN_COMPLEX_COMPAT_H
#define ARAN_COMPLEX_COMPAT_H

#ifdef __cplusplus
#include <complex>
typedef std::complex<float> gcomplex64;
typedef std::complex<double> gcomplex128;
#else
#include <complex.h>
typedef float _Complex gcomplex64;
typedef double _Complex gcomplex128;
#endif

#endif
