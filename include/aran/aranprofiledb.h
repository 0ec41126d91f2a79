/*
 * aranprofiledb.h -- LibAran's operator cost database (aran/aranprofiledb.h).
 *
 * A profiledb.ini file (GKeyFile syntax: [group] headers, key=value lines,
 * '#' comments) holds, per operator symbol, the ascending coefficients of a
 * polynomial in the order ("name=c0;c1;...;") and measured samples
 * ("samples-name=p:seconds;...").  The file is the given one, else
 * $ARAN_PROFILE_DB, else profiledb.ini beside libaran_gpu.so; the group the
 * given one, else $ARAN_PROFILE_GROUP, else "aran-profile"
 * (aran/aranprofiledb.c:158-200).  Keys are resolved to the addresses of the
 * functions of that name in the process (the reference resolves them with
 * g_module_symbol), so lookups by name and by operator address agree.
 * Evaluation returns the sample at exactly x when there is one, else the
 * polynomial's value, else NaN (aran/aranprofiledb.c:276-318).
 */
#ifndef ARAN_COMPAT_PROFILE_DB_H
#define ARAN_COMPAT_PROFILE_DB_H

#include <aran/aran.h>
#include <aran/aranpoly1d.h>

G_BEGIN_DECLS

#define ARAN_PROFILE_DB_DEFAULT_GROUP "aran-profile"
#define ARAN_PROFILE_DB_SAMPLES_PREFIX "samples-"

void aran_profile_db_set_verbose (gboolean verbose);
gboolean aran_profile_db_read_file (const gchar *filename, const gchar *group);
AranPoly1d *aran_profile_db_get_by_name (gchar *name);
AranPoly1d *aran_profile_db_get_by_address (gpointer address);
void aran_profile_db_set_value (gchar *name, gpointer address, AranPoly1d *value);
gdouble aran_profile_db_name_eval (gchar *name, gdouble x);
gdouble aran_profile_db_address_eval (gpointer address, gdouble x);

G_END_DECLS

#endif
