// profiledb.cpp -- LibAran's operator cost database (aran/aranprofiledb.c)
// and its polynomial type (aran/aranpoly1d.c), host code of libaran_gpu.so.
//
// The file format, the lookup rules (sample at exactly x, else polynomial,
// else NaN) and the environment variables follow the reference; the
// key-file reader, the name -> address resolution (dlsym on this library,
// then on the whole process) and the storage are this library's own.
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <aran/aranprofiledb.h>

namespace {

struct Db {
  std::mutex mu;
  bool verbose = true;
  std::map<std::string, AranPoly1d *> by_name;
  std::map<const void *, AranPoly1d *> by_addr;
  std::map<std::string, std::map<double, double>> samples_by_name;
  std::map<const void *, std::map<double, double>> samples_by_addr;
};

Db &db() {
  static Db d;
  return d;
}

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// the function of that name in this library, else anywhere in the process
void *symbol_address(const std::string &name) {
  static void *self = nullptr;
  if (!self) {
    Dl_info info;
    if (dladdr((void *)&aran_profile_db_read_file, &info) && info.dli_fname)
      self = dlopen(info.dli_fname, RTLD_LAZY | RTLD_NOLOAD);
  }
  void *p = self ? dlsym(self, name.c_str()) : nullptr;
  return p ? p : dlsym(RTLD_DEFAULT, name.c_str());
}

std::string default_path() {
  Dl_info info;
  if (dladdr((void *)&aran_profile_db_read_file, &info) && info.dli_fname) {
    std::string f = info.dli_fname;
    size_t k = f.rfind('/');
    return (k == std::string::npos ? std::string(".") : f.substr(0, k)) + "/profiledb.ini";
  }
  return "profiledb.ini";
}

std::vector<std::string> split(const std::string &s, char sep) {
  std::vector<std::string> out;
  std::string cur;
  std::istringstream in(s);
  while (std::getline(in, cur, sep)) {
    cur = trim(cur);
    if (!cur.empty()) out.push_back(cur);
  }
  return out;
}

double eval_locked(AranPoly1d *p, const std::map<double, double> *smp, double x) {
  if (smp) {
    auto it = smp->find(x);
    if (it != smp->end()) return it->second;
  }
  if (!p) return NAN;
  return aran_poly1d_eval(p, x);
}

}  // namespace

extern "C" {

AranPoly1d *aran_poly1d_new(guint deg) {
  AranPoly1d *p = (AranPoly1d *)std::malloc(sizeof(AranPoly1d));
  p->degree = deg;
  p->terms = (gdouble *)std::calloc(deg + 1, sizeof(gdouble));
  return p;
}

AranPoly1d *aran_poly1d_new_with_terms(int degree, const double *terms) {
  AranPoly1d *p = aran_poly1d_new(degree < 0 ? 0 : (guint)degree);
  for (int i = 0; i <= degree; ++i) p->terms[i] = terms[i];
  return p;
}

void aran_poly1d_free(AranPoly1d *p) {
  if (!p) return;
  std::free(p->terms);
  std::free(p);
}

void aran_poly1d_write(AranPoly1d *p, FILE *file) {
  if (!p || !file) return;
  for (guint i = 0; i <= p->degree; ++i) std::fprintf(file, "%s%.17g", i ? ";" : "", p->terms[i]);
}

static void poly_combine(AranPoly1d *one, AranPoly1d *other, AranPoly1d *ret, double sign) {
  if (!one || !other || !ret) return;
  for (guint i = 0; i <= ret->degree; ++i) {
    double a = i <= one->degree ? one->terms[i] : 0., b = i <= other->degree ? other->terms[i] : 0.;
    ret->terms[i] = a + sign * b;
  }
}

void aran_poly1d_add(AranPoly1d *one, AranPoly1d *other, AranPoly1d *ret) {
  poly_combine(one, other, ret, 1.);
}

void aran_poly1d_sub(AranPoly1d *one, AranPoly1d *other, AranPoly1d *ret) {
  poly_combine(one, other, ret, -1.);
}

void aran_poly1d_scalp(AranPoly1d *p, gdouble factor, AranPoly1d *ret) {
  if (!p || !ret) return;
  for (guint i = 0; i <= ret->degree; ++i) ret->terms[i] = (i <= p->degree ? p->terms[i] : 0.) * factor;
}

gdouble aran_poly1d_eval(AranPoly1d *p, gdouble x) {
  double r = p->terms[p->degree];
  for (int i = (int)p->degree - 1; i >= 0; --i) r = r * x + p->terms[i];
  return r;
}

void aran_profile_db_set_verbose(gboolean verbose) {
  std::lock_guard<std::mutex> lk(db().mu);
  db().verbose = verbose != 0;
}

gboolean aran_profile_db_read_file(const gchar *filename, const gchar *group) {
  Db &d = db();
  std::string path;
  if (filename) path = filename;
  else if (const char *e = std::getenv("ARAN_PROFILE_DB")) path = e;
  else path = default_path();
  std::string grp;
  if (group) grp = group;
  else if (const char *e = std::getenv("ARAN_PROFILE_GROUP")) grp = e;
  else grp = ARAN_PROFILE_DB_DEFAULT_GROUP;
  std::ifstream in(path);
  if (!in) {
    if (d.verbose || filename) std::fprintf(stderr, "Unable to open profile_db file \"%s\"\n", path.c_str());
    return FALSE;
  }
  std::string line, cur;
  bool found = false;
  std::vector<std::pair<std::string, std::string>> kv;
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    if (t[0] == '[') {
      size_t e = t.find(']');
      cur = t.substr(1, e == std::string::npos ? std::string::npos : e - 1);
      if (cur == grp) found = true;
      continue;
    }
    size_t eq = t.find('=');
    if (eq == std::string::npos || cur != grp) continue;
    kv.emplace_back(trim(t.substr(0, eq)), trim(t.substr(eq + 1)));
  }
  if (!found) {
    if (d.verbose)
      std::fprintf(stderr, "Unable to locate group \"%s\" in profile_db file \"%s\"\n", grp.c_str(),
                   path.c_str());
    return FALSE;
  }
  std::lock_guard<std::mutex> lk(d.mu);
  const std::string pre = ARAN_PROFILE_DB_SAMPLES_PREFIX;
  for (auto &p : kv) {
    if (p.first.compare(0, pre.size(), pre) == 0) {
      std::string name = p.first.substr(pre.size());
      std::map<double, double> m;
      for (auto &item : split(p.second, ';')) {
        size_t c = item.find(':');
        if (c == std::string::npos) continue;
        m[std::strtod(item.substr(0, c).c_str(), nullptr)] =
            std::strtod(item.substr(c + 1).c_str(), nullptr);
      }
      d.samples_by_name[name] = m;
      if (void *a = symbol_address(name)) d.samples_by_addr[a] = m;
    } else {
      std::vector<double> c;
      for (auto &item : split(p.second, ';')) c.push_back(std::strtod(item.c_str(), nullptr));
      if (c.empty()) continue;
      AranPoly1d *poly = aran_poly1d_new_with_terms((int)c.size() - 1, c.data());
      auto old = d.by_name.find(p.first);
      if (old != d.by_name.end()) {
        for (auto it = d.by_addr.begin(); it != d.by_addr.end();)
          it = it->second == old->second ? d.by_addr.erase(it) : std::next(it);
        aran_poly1d_free(old->second);
      }
      d.by_name[p.first] = poly;
      if (void *a = symbol_address(p.first)) d.by_addr[a] = poly;
    }
  }
  return TRUE;
}

AranPoly1d *aran_profile_db_get_by_name(gchar *name) {
  if (!name) return nullptr;
  std::lock_guard<std::mutex> lk(db().mu);
  auto it = db().by_name.find(name);
  return it == db().by_name.end() ? nullptr : it->second;
}

AranPoly1d *aran_profile_db_get_by_address(gpointer address) {
  std::lock_guard<std::mutex> lk(db().mu);
  auto it = db().by_addr.find(address);
  return it == db().by_addr.end() ? nullptr : it->second;
}

void aran_profile_db_set_value(gchar *name, gpointer address, AranPoly1d *value) {
  if (!name) return;
  std::lock_guard<std::mutex> lk(db().mu);
  db().by_name[name] = value;
  if (address) db().by_addr[address] = value;
}

gdouble aran_profile_db_name_eval(gchar *name, gdouble x) {
  if (!name) return NAN;
  std::lock_guard<std::mutex> lk(db().mu);
  Db &d = db();
  auto s = d.samples_by_name.find(name);
  auto p = d.by_name.find(name);
  return eval_locked(p == d.by_name.end() ? nullptr : p->second,
                     s == d.samples_by_name.end() ? nullptr : &s->second, x);
}

gdouble aran_profile_db_address_eval(gpointer address, gdouble x) {
  std::lock_guard<std::mutex> lk(db().mu);
  Db &d = db();
  auto s = d.samples_by_addr.find(address);
  auto p = d.by_addr.find(address);
  return eval_locked(p == d.by_addr.end() ? nullptr : p->second,
                     s == d.samples_by_addr.end() ? nullptr : &s->second, x);
}

}  // extern "C"
