/* glib/gprintf.h -- TEST INFRASTRUCTURE (see glib.h of this directory) */
#ifndef ORACLE_SHIM_GPRINTF_H
#define ORACLE_SHIM_GPRINTF_H
#include <stdio.h>
#define g_fprintf fprintf
#endif
