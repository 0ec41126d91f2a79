// tune.cu -- the autotuner of the 3D solve: times the leaf capacities and
// M2L kernels that serve a configuration on a sample and keeps the fastest,
// in the profile database file (profiledb.ini syntax) under the group
// [aran-gpu-tune].  LibAran's own profiling times its operators for the
// semifar cost model (aran/aranprofile.c:11-60, stored by
// aran/aranprofiledb.c:158-200); this tunes the GPU solve itself, and reads
// and writes its group without touching the operator-cost groups.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "internal.cuh"

namespace aran {
namespace {

const char *kTuneGroup = "aran-gpu-tune";

std::string tune_key(const AranGpuConfig3d *c) {
  const char *fl = c->flavour == ARAN_FLAVOUR_KKYLIN ? "kkylin"
                   : (c->flavour == ARAN_FLAVOUR_NORMAL ? "normal" : "rotate");
  return "p" + std::to_string(c->order) + "-" +
         (c->precision == ARAN_PRECISION_MIXED ? "mixed" : "fp64") + "-" + fl + "-" +
         (c->field ? "field" : "pot");
}

std::string db_path(const char *given) {
  if (given) return given;
  if (const char *e = std::getenv("ARAN_PROFILE_DB")) return e;
  Dl_info info;
  if (dladdr((void *)&aran_gpu_tune_lookup, &info) && info.dli_fname) {
    std::string f = info.dli_fname;
    size_t k = f.rfind('/');
    return (k == std::string::npos ? std::string(".") : f.substr(0, k)) + "/profiledb.ini";
  }
  return "profiledb.ini";
}

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// value of key in group of an INI file ("" and false when absent)
bool ini_get(const std::string &path, const std::string &group, const std::string &key,
             std::string &val) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line, cur;
  while (std::getline(in, line)) {
    const std::string t = trim(line);
    if (t.empty() || t[0] == '#' || t[0] == ';') continue;
    if (t.front() == '[' && t.back() == ']') {
      cur = t.substr(1, t.size() - 2);
      continue;
    }
    if (cur != group) continue;
    const size_t eq = t.find('=');
    if (eq == std::string::npos) continue;
    if (trim(t.substr(0, eq)) == key) {
      val = trim(t.substr(eq + 1));
      return true;
    }
  }
  return false;
}

// sets keys of group in an INI file, keeping every other line
void ini_set(const std::string &path, const std::string &group,
             const std::vector<std::pair<std::string, std::string>> &kv) {
  std::vector<std::string> lines;
  {
    std::ifstream in(path);
    std::string line;
    while (in && std::getline(in, line)) lines.push_back(line);
  }
  std::vector<bool> done(kv.size(), false);
  std::string cur;
  int group_end = -1;   // index after the group's last line
  for (size_t i = 0; i < lines.size(); ++i) {
    const std::string t = trim(lines[i]);
    if (!t.empty() && t.front() == '[' && t.back() == ']') {
      cur = t.substr(1, t.size() - 2);
      if (cur == group) group_end = (int)i + 1;
      continue;
    }
    if (cur != group) continue;
    group_end = (int)i + 1;
    const size_t eq = t.find('=');
    if (eq == std::string::npos || t[0] == '#') continue;
    const std::string k = trim(t.substr(0, eq));
    for (size_t j = 0; j < kv.size(); ++j)
      if (!done[j] && kv[j].first == k) {
        lines[i] = k + "=" + kv[j].second;
        done[j] = true;
      }
  }
  std::vector<std::string> add;
  for (size_t j = 0; j < kv.size(); ++j)
    if (!done[j]) add.push_back(kv[j].first + "=" + kv[j].second);
  if (group_end < 0) {
    if (!lines.empty() && !trim(lines.back()).empty()) lines.push_back("");
    lines.push_back("[" + group + "]");
    lines.insert(lines.end(), add.begin(), add.end());
  } else {
    lines.insert(lines.begin() + group_end, add.begin(), add.end());
  }
  std::ofstream out(path, std::ios::trunc);
  if (!out) throw std::runtime_error("cannot write the profile database " + path);
  for (const auto &l : lines) out << l << "\n";
}

struct Candidate {
  int maxbox, kernel, nst, g;
};

// merges "x:value;" into the samples string of a profile-database key
std::string merge_sample(const std::string &old, double x, double value) {
  std::vector<std::pair<double, std::string>> items;
  std::istringstream in(old);
  std::string item;
  while (std::getline(in, item, ';')) {
    item = trim(item);
    const size_t c = item.find(':');
    if (c == std::string::npos) continue;
    const double k = std::strtod(item.substr(0, c).c_str(), nullptr);
    if (k != x) items.push_back({k, item});
  }
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%g:%.6e", x, value);
  items.push_back({x, buf});
  std::sort(items.begin(), items.end(),
            [](const std::pair<double, std::string> &a, const std::pair<double, std::string> &b) {
              return a.first < b.first;
            });
  std::string out;
  for (const auto &it : items) out += it.second + ";";
  return out;
}

// amortised cost of one operator call on the GPU for the chosen
// configuration (a stage's CUDA-event time over the operations it ran),
// stored as samples at x = order under the reference's operator names in
// the operator-cost group, which aran_solver3d_db_profile_operators reads
// (aran/aransolver3d.c:687-740)
void write_operator_costs(const std::string &path, const AranGpuConfig3d *cfg,
                          const double ms[16], const int64_t st[11]) {
  const char *suffix = cfg->flavour == ARAN_FLAVOUR_KKYLIN ? "_kkylin"
                       : (cfg->flavour == ARAN_FLAVOUR_NORMAL ? "" : "_rotate");
  const char *group = std::getenv("ARAN_PROFILE_GROUP");
  const std::string grp = group ? group : "aran-profile";
  struct Op {
    std::string name;
    double ms;
    int64_t count;
  };
  const Op ops[] = {{"aran_development3d_p2m", ms[4], st[2]},
                    {std::string("aran_development3d_m2m") + suffix, ms[5], st[3]},
                    {std::string("aran_development3d_m2l") + suffix, ms[6], st[4]},
                    {std::string("aran_development3d_l2l") + suffix, ms[7], st[5]},
                    {"aran_development3d_l2p", ms[8], st[6]}};
  std::vector<std::pair<std::string, std::string>> kv;
  for (const Op &o : ops) {
    if (o.count <= 0 || !(o.ms > 0)) continue;
    std::string old;
    ini_get(path, grp, "samples-" + o.name, old);
    kv.push_back({"samples-" + o.name, merge_sample(old, cfg->order, o.ms * 1e-3 / (double)o.count)});
  }
  if (!kv.empty()) ini_set(path, grp, kv);
}

}  // namespace
}  // namespace aran

using namespace aran;

extern "C" {

int aran_gpu_tune_lookup(const char *path, const AranGpuConfig3d *cfg, AranGpuTuneResult *out) {
  if (!cfg || !out) return fail(ARAN_ERR_INVALID, "NULL argument");
  std::string v;
  if (!ini_get(db_path(path), kTuneGroup, tune_key(cfg), v)) return 0;
  AranGpuTuneResult r = {};
  // maxbox=..;m2l=..;nst=..;g=..;ms=..
  int got = 0;
  std::istringstream in(v);
  std::string item;
  while (std::getline(in, item, ';')) {
    const size_t eq = item.find('=');
    if (eq == std::string::npos) continue;
    const std::string k = trim(item.substr(0, eq));
    const std::string x = trim(item.substr(eq + 1));
    char *endp = nullptr;
    const double d = std::strtod(x.c_str(), &endp);
    if (endp == x.c_str()) return fail(ARAN_ERR_INVALID, "malformed tuning entry: " + v);
    if (k == "maxbox") { r.maxbox = (int)d; got |= 1; }
    else if (k == "m2l") { r.m2l_kernel = (int)d; got |= 2; }
    else if (k == "nst") r.m2l_nst = (int)d;
    else if (k == "g") r.m2l_g = (int)d;
    else if (k == "ms") r.ms = d;
  }
  if ((got & 3) != 3 || r.maxbox < 1 || r.m2l_kernel < ARAN_M2L_AUTO || r.m2l_kernel > ARAN_M2L_TENSOR ||
      r.m2l_nst < 0 || r.m2l_nst > 3 || r.m2l_g < 0 || r.m2l_g > 2)
    return fail(ARAN_ERR_INVALID, "malformed tuning entry: " + v);
  *out = r;
  return 1;
}

int aran_gpu_autotune3d(const AranGpuConfig3d *cfg, int64_t n, const double *xyz, const double *q,
                        int mem, const int *maxboxes, int nmaxbox, int reps, const char *path,
                        AranGpuTuneResult *out) {
  if (!cfg || !xyz || !q || !out) return fail(ARAN_ERR_INVALID, "NULL argument");
  if (n < 1) return fail(ARAN_ERR_INVALID, "n must be >= 1");
  if (reps < 1) reps = 3;
  static const int kDefault[] = {16, 24, 32, 48, 64, 96, 128};
  std::vector<int> mbs;
  if (maxboxes && nmaxbox > 0) mbs.assign(maxboxes, maxboxes + nmaxbox);
  else mbs.assign(kDefault, kDefault + 7);
  for (int m : mbs)
    if (m < 1) return fail(ARAN_ERR_INVALID, "candidate maxbox must be >= 1");
  const bool rot = cfg->flavour != ARAN_FLAVOUR_KKYLIN;
  const bool mixed = cfg->precision == ARAN_PRECISION_MIXED;
  std::vector<Candidate> cands;
  for (int m : mbs) {
    if (!mixed || !rot) {
      cands.push_back({m, ARAN_M2L_AUTO, 0, 0});
      continue;
    }
    if (m2l_lane_order(cfg->order)) cands.push_back({m, ARAN_M2L_LANES, 0, 0});
    cands.push_back({m, ARAN_M2L_SIBLING, 0, 0});
    int nst = 0, g = 0;
    const int nc = m2l_sibling_configs(cfg->order, &nst, &g, 0);
    for (int k = 0; k < nc; ++k) {
      m2l_sibling_configs(cfg->order, &nst, &g, k);
      cands.push_back({m, ARAN_M2L_SIBLING, nst, g});
    }
  }
  AranGpuTuneResult best = {};
  best.ms = INFINITY;
  std::string samples;
  for (const Candidate &c : cands) {
    AranGpuConfig3d cc = *cfg;
    cc.maxbox = c.maxbox;
    AranGpuSolver3d *s = nullptr;
    int rc = aran_gpu_solver3d_create(&cc, &s);
    if (rc) return rc;
    rc = aran_gpu_solver3d_set_m2l_kernel(s, c.kernel, c.nst, c.g);
    std::vector<double> t;
    for (int r = 0; !rc && r <= reps; ++r) {
      rc = aran_gpu_solver3d_solve(s, n, xyz, q, nullptr, nullptr, mem);
      double ms[16];
      if (!rc && r > 0 && aran_gpu_solver3d_timings(s, ms) == ARAN_OK) t.push_back(ms[0]);
    }
    aran_gpu_solver3d_destroy(s);
    if (rc) return rc;
    std::sort(t.begin(), t.end());
    const double med = t[t.size() / 2];
    char buf[96];
    std::snprintf(buf, sizeof(buf), "%s%d/%d/%d/%d:%.4f", samples.empty() ? "" : ";", c.maxbox,
                  c.kernel, c.nst, c.g, med);
    samples += buf;
    if (med < best.ms) {
      best.maxbox = c.maxbox;
      best.m2l_kernel = c.kernel;
      best.m2l_nst = c.nst;
      best.m2l_g = c.g;
      best.ms = med;
    }
  }
  best.candidates = (int)cands.size();
  *out = best;
  if (path) {
    // one more solve of the chosen configuration for the operator costs
    AranGpuConfig3d cc = *cfg;
    cc.maxbox = best.maxbox;
    AranGpuSolver3d *s = nullptr;
    int rc = aran_gpu_solver3d_create(&cc, &s);
    if (rc) return rc;
    double ms[16];
    int64_t st[11];
    rc = aran_gpu_solver3d_set_m2l_kernel(s, best.m2l_kernel, best.m2l_nst, best.m2l_g);
    if (!rc) rc = aran_gpu_solver3d_solve(s, n, xyz, q, nullptr, nullptr, mem);
    if (!rc) rc = aran_gpu_solver3d_timings(s, ms);
    if (!rc) rc = aran_gpu_solver3d_get_stats(s, st);
    aran_gpu_solver3d_destroy(s);
    if (rc) return rc;
    try {
      write_operator_costs(path, cfg, ms, st);
    } catch (const std::exception &e) {
      return fail(ARAN_ERR_INVALID, e.what());
    }
    char v[160];
    std::snprintf(v, sizeof(v), "maxbox=%d;m2l=%d;nst=%d;g=%d;ms=%.4f", best.maxbox,
                  best.m2l_kernel, best.m2l_nst, best.m2l_g, best.ms);
    const std::string key = tune_key(cfg);
    try {
      ini_set(path, kTuneGroup, {{key, v}, {"samples-" + key, samples}});
    } catch (const std::exception &e) {
      return fail(ARAN_ERR_INVALID, e.what());
    }
  }
  return ARAN_OK;
}

}  // extern "C"
