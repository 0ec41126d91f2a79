/* aran.h -- LibAran entry header (aran/aran.h:27-29). */
#ifndef ARAN_COMPAT_ARAN_H
#define ARAN_COMPAT_ARAN_H

#include <aran/aranglib.h>
#include <aran/arancomplex.h>

G_BEGIN_DECLS

typedef void (*AranZeroFunc) (gpointer devel);

/* aran_init (aran/aran.c:60-69): one-time initialisation; selects the
 * current CUDA device for later solvers. */
void aran_init (void);

G_END_DECLS

#endif
