/*
 * aranlaurentseriesd.h -- LibAran's Laurent series (aran/aranlaurentseriesd.h:
 * 41-80) on the GPU library.
 *
 * A series of degrees (posdeg, negdeg) holds the complex coefficients of
 * z^posdeg .. z^0 .. z^-negdeg; aran_laurent_seriesd_get_term (als, i)
 * returns the coefficient of z^i.  The containers live in host memory.
 * evaluate, translate and to_taylor run on the GPU (one small launch per
 * call, FP64, the reference's term-by-term loops); when no GPU is usable
 * they leave their outputs untouched, return 0 where they return a value,
 * and set aran_gpu_last_error().
 */
#ifndef ARAN_COMPAT_LAURENT_SERIESD_H
#define ARAN_COMPAT_LAURENT_SERIESD_H

#include <stdio.h>

#include <aran/aran.h>

G_BEGIN_DECLS

typedef struct _AranLaurentSeriesd AranLaurentSeriesd;

AranLaurentSeriesd *aran_laurent_seriesd_new (guint8 posdeg, guint8 negdeg);
void aran_laurent_seriesd_free (AranLaurentSeriesd *als);
void aran_laurent_seriesd_copy (const AranLaurentSeriesd *src, AranLaurentSeriesd *dst);
AranLaurentSeriesd *aran_laurent_seriesd_clone (AranLaurentSeriesd *src);
gcomplex128 *aran_laurent_seriesd_get_term (AranLaurentSeriesd *als, gint i);
guint8 aran_laurent_seriesd_get_posdeg (AranLaurentSeriesd *als);
guint8 aran_laurent_seriesd_get_negdeg (AranLaurentSeriesd *als);
void aran_laurent_seriesd_set_zero (AranLaurentSeriesd *als);
void aran_laurent_seriesd_add (AranLaurentSeriesd *one, AranLaurentSeriesd *other,
                               AranLaurentSeriesd *result);
void aran_laurent_seriesd_write (AranLaurentSeriesd *als, FILE *file);

gcomplex128 aran_laurent_seriesd_evaluate (AranLaurentSeriesd *als, gcomplex128 z);
void aran_laurent_seriesd_translate (AranLaurentSeriesd *src, gcomplex128 zsrc,
                                     AranLaurentSeriesd *dst, gcomplex128 zdst);
void aran_laurent_seriesd_to_taylor (AranLaurentSeriesd *src, gcomplex128 zsrc,
                                     AranLaurentSeriesd *dst, gcomplex128 zdst);

G_END_DECLS

#endif
