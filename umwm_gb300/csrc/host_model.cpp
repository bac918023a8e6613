// Host-side model set-up (see host_model.hpp).  All arithmetic is fp32 in
// the reference's evaluation order; this file is compiled without FMA
// contraction so that the unrolled grid is bit-identical and the tables
// are what an fp32 build of the reference computes.
#include "host_model.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>

namespace umwm {

// ---------------------------------------------------------------------------
// Namelist reader: '&group key = value[, value ...] /' with '!' comments,
// case-insensitive names, quoted strings and blank/comma separated lists.
// umwm_init.F90:67-92 (read order DOMAIN .. OUTPUT), umwm_stokes.F90:25-34.
// ---------------------------------------------------------------------------
namespace {
enum class Tok { Word, Eq, Slash, Amp, End };

struct Lexer {
  const std::string& s;
  size_t k = 0;
  explicit Lexer(const std::string& t) : s(t) {}
  void skip() {
    for (;;) {
      while (k < s.size() && (std::isspace((unsigned char)s[k]) || s[k] == ',')) ++k;
      if (k < s.size() && s[k] == '!') {
        while (k < s.size() && s[k] != '\n') ++k;
        continue;
      }
      return;
    }
  }
  Tok next(std::string& word) {
    skip();
    word.clear();
    if (k >= s.size()) return Tok::End;
    char c = s[k];
    if (c == '=') { ++k; return Tok::Eq; }
    if (c == '/') { ++k; return Tok::Slash; }
    if (c == '&') {
      ++k;
      while (k < s.size() && (std::isalnum((unsigned char)s[k]) || s[k] == '_')) word += (char)std::tolower((unsigned char)s[k++]);
      return Tok::Amp;
    }
    if (c == '\'' || c == '"') {
      size_t e = s.find(c, k + 1);
      if (e == std::string::npos) e = s.size();
      word = s.substr(k + 1, e - k - 1);
      k = e + 1;
      return Tok::Word;
    }
    while (k < s.size() && !std::isspace((unsigned char)s[k]) && s[k] != ',' && s[k] != '=' && s[k] != '/' &&
           s[k] != '!')
      word += s[k++];
    return Tok::Word;
  }
};
}  // namespace

bool parse_nml(const std::string& text, NmlGroups& out, std::string& err) {
  Lexer lx(text);
  std::string w, group, key;
  std::vector<std::string> pending;  // words seen since the last '='
  bool in_group = false;
  auto flush_values = [&](size_t keep_last) {
    // all pending words except the trailing keep_last belong to 'key'
    if (!key.empty())
      for (size_t q = 0; q + keep_last < pending.size(); ++q) out.g[group][key].push_back(pending[q]);
    pending.erase(pending.begin(), pending.end() - (long)keep_last);
  };
  for (;;) {
    Tok t = lx.next(w);
    if (t == Tok::End) break;
    if (!in_group) {
      if (t == Tok::Amp) { group = w; in_group = true; key.clear(); pending.clear(); out.g[group]; }
      continue;
    }
    if (t == Tok::Word) { pending.push_back(w); continue; }
    if (t == Tok::Eq) {
      if (pending.empty()) { err = "'=' without a name in &" + group; return false; }
      flush_values(1);
      key = pending.back();
      for (auto& c : key) c = (char)std::tolower((unsigned char)c);
      pending.clear();
      out.g[group][key].clear();
      continue;
    }
    if (t == Tok::Slash) {
      flush_values(0);
      in_group = false;
      continue;
    }
    if (t == Tok::Amp) { err = "group &" + group + " not closed with '/'"; return false; }
  }
  if (in_group) { err = "group &" + group + " not closed with '/'"; return false; }
  return true;
}

// ---------------------------------------------------------------------------
// Clock: proleptic Gregorian seconds (the reference uses datetime-fortran
// only for this, umwm_top.F90:59-75,157-158).
// ---------------------------------------------------------------------------
static int64_t days_since_epoch(int64_t y, int m, int d) {
  // count days with March-based years so that the leap day is last
  y -= (m <= 2);
  int64_t era = (y >= 0 ? y : y - 399) / 400;
  int64_t yoe = y - era * 400;
  int64_t mp = (m + 9) % 12;
  int64_t doy = (153 * mp + 2) / 5 + d - 1;
  int64_t doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 719468;
}

bool time_from_string(const std::string& s, int64_t& t) {
  if (s.size() < 19) return false;
  for (int q : {0, 1, 2, 3, 5, 6, 8, 9, 11, 12, 14, 15, 17, 18})
    if (!std::isdigit((unsigned char)s[q])) return false;
  auto num = [&](int a, int n) { return std::atoi(s.substr(a, n).c_str()); };
  int Y = num(0, 4), M = num(5, 2), D = num(8, 2), h = num(11, 2), mi = num(14, 2), se = num(17, 2);
  if (M < 1 || M > 12 || D < 1 || D > 31 || h > 23 || mi > 59 || se > 59) return false;
  t = days_since_epoch(Y, M, D) * 86400 + h * 3600 + mi * 60 + se;
  return true;
}

std::string time_to_string(int64_t t, char sep) {
  int64_t days = t / 86400, rem = t % 86400;
  if (rem < 0) { rem += 86400; days -= 1; }
  int64_t z = days + 719468;
  int64_t era = (z >= 0 ? z : z - 146096) / 146097;
  int64_t doe = z - era * 146097;
  int64_t yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  int64_t doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  int64_t mp = (5 * doy + 2) / 153;
  int d = (int)(doy - (153 * mp + 2) / 5 + 1);
  int m = (int)(mp < 10 ? mp + 3 : mp - 9);
  int64_t y = yoe + era * 400 + (m <= 2);
  char buf[64];
  std::snprintf(buf, sizeof buf, "%04d-%02d-%02d%c%02d:%02d:%02d", (int)y, m, d, sep, (int)(rem / 3600),
                (int)(rem / 60 % 60), (int)(rem % 60));
  return buf;
}

std::string time_key(const char* time19) {
  std::string k(time19 ? time19 : "");
  if (k.size() > 19) k.resize(19);
  if (k.size() >= 11) k[10] = '_';
  return k;
}

// ---------------------------------------------------------------------------
// nmlread, umwm_init.F90:56-193
// ---------------------------------------------------------------------------
bool HostModel::read_namelist(const std::string& text) {
  NmlGroups nl;
  if (!parse_nml(text, nl, err)) { err = "namelist: " + err; return false; }
  for (const char* gname : {"domain", "physics", "grid", "forcing", "forcing_constant", "output", "stokes"})
    if (!nl.g.count(gname)) { err = std::string("namelist: group &") + gname + " not found"; return false; }
  auto first = [&](const char* gname, const char* key) -> const std::string* {
    auto& grp = nl.g[gname];
    auto it = grp.find(key);
    return (it == grp.end() || it->second.empty()) ? nullptr : &it->second[0];
  };
  // A name missing from the file keeps the zero value of static storage.
  auto real = [&](const char* gname, const char* key, float& v) {
    const std::string* s = first(gname, key);
    if (!s) { v = 0.f; return; }
    std::string t = *s;
    for (auto& c : t) if (c == 'd' || c == 'D') c = 'e';
    v = std::strtof(t.c_str(), nullptr);
  };
  auto integer = [&](const char* gname, const char* key, int& v) {
    const std::string* s = first(gname, key);
    v = s ? std::atoi(s->c_str()) : 0;
  };
  auto logical = [&](const char* gname, const char* key, bool& v) {
    const std::string* s = first(gname, key);
    if (!s) { v = false; return; }
    size_t q = (!s->empty() && (*s)[0] == '.') ? 1 : 0;
    v = q < s->size() && (std::tolower((unsigned char)(*s)[q]) == 't');
  };
  auto str = [&](const char* gname, const char* key, std::string& v) {
    const std::string* s = first(gname, key);
    v = s ? *s : std::string();
  };
  logical("domain", "isglobal", isglobal);
  integer("domain", "mm", mm); integer("domain", "nm", nm); integer("domain", "om", om); integer("domain", "pm", pm);
  real("domain", "fmin", fmin); real("domain", "fmax", fmax); real("domain", "fprog", fprog);
  str("domain", "starttimestr", starttimestr); str("domain", "stoptimestr", stoptimestr);
  real("domain", "dtg", dtg); logical("domain", "restart", restart);
  real("physics", "g", g); real("physics", "nu_air", nu_air); real("physics", "nu_water", nu_water);
  real("physics", "sfct", sfct); real("physics", "kappa", kappa); real("physics", "z", z);
  real("physics", "gustiness", gustiness); real("physics", "dmin", dmin); real("physics", "explim", explim);
  real("physics", "sin_fac", sin_fac); real("physics", "sin_diss1", sin_diss1);
  real("physics", "sin_diss2", sin_diss2); real("physics", "sds_fac", sds_fac);
  real("physics", "sds_power", sds_power); real("physics", "mss_fac", mss_fac);
  real("physics", "snl_fac", snl_fac); real("physics", "sdt_fac", sdt_fac); real("physics", "sbf_fac", sbf_fac);
  real("physics", "sbp_fac", sbp_fac);
  logical("grid", "gridfromfile", gridfromfile); real("grid", "delx", delx); real("grid", "dely", dely);
  logical("grid", "topofromfile", topofromfile); real("grid", "dpt", dpt);
  logical("grid", "fillestuaries", fillestuaries); logical("grid", "filllakes", filllakes);
  logical("forcing", "winds", winds); logical("forcing", "currents", currents);
  logical("forcing", "air_density", air_density); logical("forcing", "water_density", water_density);
  logical("forcing", "seaice", seaice);
  real("forcing_constant", "wspd0", wspd0); real("forcing_constant", "wdir0", wdir0);
  real("forcing_constant", "uc0", uc0); real("forcing_constant", "vc0", vc0);
  real("forcing_constant", "rhoa0", rhoa0); real("forcing_constant", "rhow0", rhow0);
  real("forcing_constant", "fice0", fice0); real("forcing_constant", "fice_lth", fice_lth);
  real("forcing_constant", "fice_uth", fice_uth);
  integer("output", "outgrid", outgrid); integer("output", "outspec", outspec); integer("output", "outrst", outrst);
  integer("output", "xpl", xpl); integer("output", "ypl", ypl); logical("output", "stokes", stokes);
  depths_nml.assign(100, -1.f);
  {
    auto& grp = nl.g["stokes"];
    auto it = grp.find("depths");
    if (it != grp.end())
      for (size_t q = 0; q < it->second.size() && q < 100; ++q) depths_nml[q] = std::strtof(it->second[q].c_str(), nullptr);
  }
  // value checks, umwm_init.F90:95-185
  std::string bad;
  auto chk = [&](bool cond, const char* msg) { if (cond) bad += std::string(msg) + "; "; };
  const int allowed[10] = {-1, 0, 1, 2, 3, 4, 6, 8, 12, 24};
  auto ok_time = [&](int v) { return std::find(allowed, allowed + 10, v) != allowed + 10; };
  chk(mm < 3 || nm < 3, "mm and nm must be > 2");
  chk(pm % 4 != 0, "pm must be divisible by 4");
  chk(fmin <= 0 || fmax <= 0 || fprog <= 0, "fmin, fmax and fprog must be > 0");
  chk(fmin >= fmax, "fmin must be < fmax");
  chk(dtg <= 0, "dtg must be > 0");
  chk(z <= 0, "z must be > 0");
  chk(gustiness < 0, "gustiness must be positive");
  chk(dmin <= 0, "dmin must be > 0");
  chk(!gridfromfile && (delx <= 0 || dely <= 0), "delx and dely must be > 0");
  chk(!topofromfile && dpt <= 0, "dpt must be > 0");
  chk(!ok_time(outgrid), "outgrid must be -1, 0, 1, 2, 3, 4, 6, 8, 12 or 24");
  chk(!ok_time(outspec), "outspec must be -1, 0, 1, 2, 3, 4, 6, 8, 12 or 24");
  chk(!ok_time(outrst), "outrst must be -1, 0, 1, 2, 3, 4, 6, 8, 12 or 24");
  if (!bad.empty()) { err = "namelist: " + bad; return false; }
  return true;
}

// ---------------------------------------------------------------------------
// grid .. dispersion, umwm_init.F90:381-1658 (serial tiling)
// ---------------------------------------------------------------------------
namespace {
float gc_distance(float lon1, float lon2, float lat1, float lat2) {  // umwm_util.F90:211-235
  float dl = std::fabs(lon2 - lon1), dp = std::fabs(lat2 - lat1);
  float a = std::sin(0.5f * dp), b = std::sin(0.5f * dl);
  return 2 * std::asin(std::sqrt(a * a + std::cos(lat1) * std::cos(lat2) * (b * b)));
}

// The Newton solve for k and the per-(o,i) tables of dispersion(),
// umwm_init.F90:1444-1514, for wet points [a, b].
void tables_range(HostModel& M, int a, int b, float tol) {
  const int om = M.om;
  for (int i = a; i <= b; ++i) {
    const float d = M.d[i];
    const float bb = M.sfct / (M.rhow0 * M.g * (d * d));
    for (int o = 1; o <= om; ++o) {
      float c = M.twopi * std::sqrt(d / M.g);
      float fn = c * M.f[o - 1];
      float kk = fn * fn;
      float dk = 2.f * tol;
      int counter = 1;
      while (std::fabs(dk) > tol) {
        float t = std::tanh(kk);
        dk = -(fn * fn - kk * t * (1.f + bb * kk * kk)) / (3.f * bb * kk * kk * t + t + kk * (1.f + bb * kk * kk) * (1.f - t * t));
        kk = kk - dk;
        if (counter == 1000) break;
        counter++;
      }
      kk = std::fabs(kk) / d;
      const size_t q = M.oi(o, i);
      M.k[q] = kk;
      float kd = kk * d;
      if (kd > 20.f) kd = 20.f;
      float cp = M.twopi * M.f[o - 1] / kk;
      float cg = cp * (0.5f + kk * d / std::sinh(2.f * kd) + M.sfct * kk * kk / (M.rhow0 * M.g + M.sfct * kk * kk));
      M.cp0[q] = cp;
      M.cg0[q] = cg;
      float dwn = M.dom[o - 1] / std::fabs(cg);
      M.dwn[q] = dwn;
      float l2 = 0.5f * std::fabs(cp) / M.f[o - 1];
      M.k4[q] = std::pow(kk, 4.f);
      M.kdk[q] = kk * dwn;
      M.k3dk[q] = std::pow(kk, 3.f) * dwn;
      M.fkovg[q] = M.f[o - 1] * kk / M.g;
      M.cothkd[q] = std::cosh(0.2f * kd) / std::sinh(0.2f * kd);
      M.sbf[q] = M.sbf_fac * kk / (std::sinh(2.f * kd)) + M.sbp_fac * kk / (std::cosh(kd) * std::cosh(kd));
      M.sdv[q] = 4.f * M.nu_water * std::pow(kk, 2.f);
      M.logl2overz[q] = (l2 > 20.f) ? std::log(20.f / M.z) : std::log(l2 / M.z);
    }
    for (int o = 1; o <= om - 2; ++o) {
      M.bf1r[M.oi(o, i)] = M.snl_fac * M.bf1 * M.kdk[M.oi(o + 1, i)] / M.kdk[M.oi(o, i)];
      M.bf2r[M.oi(o, i)] = M.snl_fac * M.bf2 * M.kdk[M.oi(o + 2, i)] / M.kdk[M.oi(o, i)];
    }
  }
}

void fill_lake(HostModel& M, int m0, int n0) {  // umwm_init.F90:698-718, as an explicit stack
  auto edge = [&](int m, int n) { return m == 1 || m == M.mm || n == 1 || n == M.nm; };
  if (edge(m0, n0)) return;
  std::vector<std::pair<int, int>> st{{m0, n0}};
  M.mask[M.i2(m0, n0)] = 0;
  while (!st.empty()) {
    auto [m, n] = st.back();
    st.pop_back();
    const int dm[4] = {-1, 1, 0, 0}, dn[4] = {0, 0, -1, 1};
    for (int q = 0; q < 4; ++q) {
      int a = m + dm[q], b = n + dn[q];
      if (M.mask[M.i2(a, b)] == 1 && !edge(a, b)) { M.mask[M.i2(a, b)] = 0; st.push_back({a, b}); }
    }
  }
}
}  // namespace

bool HostModel::build(const Inputs& inp) {
  pi = 3.141592653589793f;
  twopi = 2 * pi;
  const size_t n2 = (size_t)mm * nm;
  // ---- grid, umwm_init.F90:381-568
  d_2d.assign(n2, 0); dx_2d.assign(n2, 0); dy_2d.assign(n2, 0); curv.assign(n2, 0);
  lon.assign(n2, 0); lat.assign(n2, 0);
  curvilinear = false;
  if (gridfromfile) {
    auto a = inp.gridtopo.find("lon"), b = inp.gridtopo.find("lat");
    if (a == inp.gridtopo.end() || b == inp.gridtopo.end() || a->second.size() != n2 || b->second.size() != n2) {
      err = "grid: gridFromFile needs 'lon' and 'lat' of size mm*nm staged with umwm_gpu_put_gridtopo";
      return false;
    }
    lon = a->second; lat = b->second;
    std::vector<float> rlon(n2), rlat(n2);
    for (size_t q = 0; q < n2; ++q) { rlon[q] = lon[q] * twopi / 360.f; rlat[q] = lat[q] * twopi / 360.f; }
    for (int n = 1; n <= nm; ++n)
      for (int m = 2; m <= mm - 1; ++m)
        dx_2d[i2(m, n)] = 6.371009e6f * gc_distance(0.5f * (rlon[i2(m - 1, n)] + rlon[i2(m, n)]),
                                                     0.5f * (rlon[i2(m, n)] + rlon[i2(m + 1, n)]),
                                                     0.5f * (rlat[i2(m - 1, n)] + rlat[i2(m, n)]),
                                                     0.5f * (rlat[i2(m, n)] + rlat[i2(m + 1, n)]));
    for (int n = 1; n <= nm; ++n) {
      dx_2d[i2(1, n)] = 2 * dx_2d[i2(2, n)] - dx_2d[i2(3, n)];
      dx_2d[i2(mm, n)] = 2 * dx_2d[i2(mm - 1, n)] - dx_2d[i2(mm - 2, n)];
    }
    for (int n = 2; n <= nm - 1; ++n)
      for (int m = 1; m <= mm; ++m)
        dy_2d[i2(m, n)] = 6.371009e6f * gc_distance(0.5f * (rlon[i2(m, n - 1)] + rlon[i2(m, n)]),
                                                     0.5f * (rlon[i2(m, n)] + rlon[i2(m, n + 1)]),
                                                     0.5f * (rlat[i2(m, n - 1)] + rlat[i2(m, n)]),
                                                     0.5f * (rlat[i2(m, n)] + rlat[i2(m, n + 1)]));
    for (int m = 1; m <= mm; ++m) {
      dy_2d[i2(m, 1)] = 2 * dy_2d[i2(m, 2)] - dy_2d[i2(m, 3)];
      dy_2d[i2(m, nm)] = 2 * dy_2d[i2(m, nm - 1)] - dy_2d[i2(m, nm - 2)];
    }
    auto heading = [&](int ma, int mb, int n) {
      float dl = rlon[i2(mb, n)] - rlon[i2(ma, n)];
      return std::atan2(std::sin(dl) * std::cos(rlat[i2(mb, n)]),
                        std::cos(rlat[i2(ma, n)]) * std::sin(rlat[i2(mb, n)]) -
                            std::sin(rlat[i2(ma, n)]) * std::cos(rlat[i2(mb, n)]) * std::cos(dl));
    };
    for (int n = 1; n <= nm; ++n)
      for (int m = 2; m <= mm - 1; ++m) curv[i2(m, n)] = heading(m - 1, m + 1, n);
    for (int n = 1; n <= nm; ++n) {
      if (isglobal) { curv[i2(1, n)] = heading(mm, 2, n); curv[i2(mm, n)] = heading(mm - 1, 1, n); }
      else { curv[i2(1, n)] = curv[i2(2, n)]; curv[i2(mm, n)] = curv[i2(mm - 1, n)]; }
    }
    for (auto& v : curv) v = v - 0.5f * pi;
    curvilinear = true;
  } else {
    std::fill(dx_2d.begin(), dx_2d.end(), delx);
    std::fill(dy_2d.begin(), dy_2d.end(), dely);
  }
  if (topofromfile) {
    auto a = inp.gridtopo.find("z");
    if (a == inp.gridtopo.end() || a->second.size() != n2) {
      err = "grid: topoFromFile needs 'z' of size mm*nm staged with umwm_gpu_put_gridtopo";
      return false;
    }
    d_2d = a->second;
  } else {
    std::fill(d_2d.begin(), d_2d.end(), dpt);
  }
  // ---- masks, umwm_init.F90:571-694
  mask.assign(n2, 1);
  for (int m = 1; m <= mm; ++m) { mask[i2(m, 1)] = 0; mask[i2(m, nm)] = 0; }
  if (!isglobal)
    for (int n = 1; n <= nm; ++n) { mask[i2(1, n)] = 0; mask[i2(mm, n)] = 0; }
  if (topofromfile) {
    for (size_t q = 0; q < n2; ++q) {
      if (d_2d[q] >= 0) { mask[q] = 0; d_2d[q] = dmin; }
      d_2d[q] = std::fabs(d_2d[q]);
      if (d_2d[q] < dmin) d_2d[q] = dmin;
    }
    if (fillestuaries) {
      for (bool again = true; again;) {
        again = false;
        for (int n = 2; n <= nm - 1; ++n)
          for (int m = 2; m <= mm - 1; ++m)
            if (mask[i2(m, n)] == 1) {
              int wet = mask[i2(m - 1, n)] + mask[i2(m + 1, n)] + mask[i2(m, n - 1)] + mask[i2(m, n + 1)];
              if (wet <= 1) { mask[i2(m, n)] = 0; again = true; }
            }
      }
    }
    if (filllakes)
      for (auto& s : inp.exclude) {
        if (s.first < 1 || s.first > mm || s.second < 1 || s.second > nm) {
          err = "masks: exclude point outside the domain";
          return false;
        }
        fill_lake(*this, s.first, s.second);
      }
  } else {
    for (size_t q = 0; q < n2; ++q) if (mask[q] == 0) d_2d[q] = dmin;
  }
  im = 0;
  for (int v : mask) im += v;
  imm = mm * nm;
  if (im < 1) { err = "masks: the domain has no sea point"; return false; }
  // ---- remap (serial: remap_dir='v', m outer, n inner), umwm_init.F90:875-1237
  ii.assign(n2, 0);
  for (auto* v : {&mi, &ni, &is, &in, &iw, &ie}) v->assign(imm + 1, 0);
  d.assign(imm + 1, 0); dx.assign(imm + 1, 0); dy.assign(imm + 1, 0);
  int cnt = 0;
  for (int pass = 1; pass >= 0; --pass)  // sea points first, then land points
    for (int m = 1; m <= mm; ++m)
      for (int n = 1; n <= nm; ++n)
        if (mask[i2(m, n)] == pass) {
          ++cnt;
          ii[i2(m, n)] = cnt;
          d[cnt] = d_2d[i2(m, n)]; dx[cnt] = dx_2d[i2(m, n)]; dy[cnt] = dy_2d[i2(m, n)];
        }
  for (int n = 1; n <= nm; ++n)
    for (int m = 1; m <= mm; ++m) { mi[ii[i2(m, n)]] = m; ni[ii[i2(m, n)]] = n; }
  auto link = [&](int m, int n, int mw, int me) {
    int q = ii[i2(m, n)];
    is[q] = ii[i2(m, n - 1)]; in[q] = ii[i2(m, n + 1)]; iw[q] = ii[i2(mw, n)]; ie[q] = ii[i2(me, n)];
  };
  for (int n = 2; n <= nm - 1; ++n)
    for (int m = 2; m <= mm - 1; ++m) link(m, n, m - 1, m + 1);
  if (isglobal)
    for (int n = 2; n <= nm - 1; ++n) { link(1, n, mm, 2); link(mm, n, mm - 1, 1); }
  iis = is; iin = in; iiw = iw; iie = ie;
  ar.assign(im + 1, 0); oneovar.assign(im + 1, 0); oneovdx.assign(im + 1, 0); oneovdy.assign(im + 1, 0);
  dxn.assign(im + 1, 0); dxs.assign(im + 1, 0); dye.assign(im + 1, 0); dyw.assign(im + 1, 0);
  curv_i.assign(im + 1, 0);
  for (int q = 1; q <= im; ++q) {
    dxn[q] = 0.5f * (dx[q] + dx[iin[q]]);
    dxs[q] = 0.5f * (dx[q] + dx[iis[q]]);
    dye[q] = 0.5f * (dy[q] + dy[iie[q]]);
    dyw[q] = 0.5f * (dy[q] + dy[iiw[q]]);
    // land neighbours are aliased to the ghost point 0 (iistart-1)
    for (auto* v : {&is, &in, &iw, &ie}) if ((*v)[q] < 1 || (*v)[q] > im) (*v)[q] = 0;
    curv_i[q] = curv[i2(mi[q], ni[q])];
  }
  // ---- init, umwm_init.F90:1240-1348
  dlnf = (std::log(fmax) - std::log(fmin)) / float(om - 1);
  f.assign(om, 0); dom.assign(om, 0);
  for (int o = 1; o <= om; ++o) f[o - 1] = std::exp(std::log(fmin) + float(o - 1) * dlnf);
  dth = twopi / float(pm);
  dthg = dth * g;
  oneovdth = 1.f / dth;
  twopisds_fac = twopi * sds_fac;
  fieldscale1 = sin_diss1 / sin_fac;
  fieldscale2 = sin_diss2 / sin_diss1;
  inv_sds_power = 1.f / sds_power;
  cfllim = (pm % 8 == 0) ? std::cos(0.25f * pi - 0.5f * dth) : 1.f / std::sqrt(2.f);
  for (int q = 1; q <= im; ++q) {
    ar[q] = dx[q] * dy[q];
    oneovdx[q] = 1.f / dx[q];
    oneovdy[q] = 1.f / dy[q];
    oneovar[q] = 1.f / ar[q];
  }
  {
    float b1 = std::exp(-16 * dlnf * dlnf), b2 = std::exp(-64 * dlnf * dlnf);
    bf1 = b1 / (b1 + b2);
    bf2 = b2 / (b1 + b2);
  }
  th.assign(pm, 0); cth.assign(pm, 0); sth.assign(pm, 0);
  for (int p = 1; p <= pm; ++p) {
    th[p - 1] = (float(p) - 0.5f * float(pm + 1)) * dth;
    cth[p - 1] = std::cos(th[p - 1]);
    sth[p - 1] = std::sin(th[p - 1]);
  }
  for (int o = 1; o <= om; ++o) dom[o - 1] = twopi * dlnf * f[o - 1];
  // ---- dispersion, umwm_init.F90:1422-1658
  const size_t noi = (size_t)om * (im + 1);
  for (auto* v : {&k, &cp0, &cg0, &dwn, &kdk, &k3dk, &k4, &fkovg, &cothkd, &sbf, &sdv, &bf1r, &bf2r, &logl2overz})
    v->assign(noi, 0.f);
  std::fill(cp0.begin(), cp0.end(), std::numeric_limits<float>::min());
  std::fill(cg0.begin(), cg0.end(), std::numeric_limits<float>::min());
  {
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if ((long)im < 4096) nt = 1;
    std::vector<std::thread> pool;
    int chunk = (im + (int)nt - 1) / (int)nt;
    for (unsigned t = 0; t < nt; ++t) {
      int a = 1 + (int)t * chunk, b = std::min(im, a + chunk - 1);
      if (a > b) break;
      pool.emplace_back([this, a, b] { tables_range(*this, a, b, 1e-2f); });
    }
    for (auto& th_ : pool) th_.join();
  }
  for (int o = 1; o <= om; ++o) {
    float mc = std::numeric_limits<float>::max(), mg = std::numeric_limits<float>::max();
    for (int q = 1; q <= im; ++q) { mc = std::min(mc, cp0[oi(o, q)]); mg = std::min(mg, cg0[oi(o, q)]); }
    cp0[oi(o, 0)] = mc;
    cg0[oi(o, 0)] = mg;
  }
  float mdx = std::numeric_limits<float>::max(), mdy = std::numeric_limits<float>::max();
  for (size_t q = 0; q < n2; ++q)
    if (mask[q] == 1) { mdx = std::min(mdx, dx_2d[q]); mdy = std::min(mdy, dy_2d[q]); }
  mindelx = std::min(mdx, mdy);
  cgmax = -std::numeric_limits<float>::max();
  for (int q = 1; q <= im; ++q)
    for (int o = 1; o <= om; ++o) cgmax = std::max(cgmax, cg0[oi(o, q)]);
  dtamin = 0.98f * cfllim * mindelx / cgmax;
  // ---- stokes depths, umwm_stokes.F90:36-39
  lm = 0;
  for (float v : depths_nml) lm += (v >= 0);
  depth.assign(lm, 0);
  for (int l = 0; l < lm; ++l) depth[l] = -depths_nml[l];
  eulerinv = 1.f / (float)std::exp(1.0);
  iip = (xpl >= 1 && xpl <= mm && ypl >= 1 && ypl <= nm) ? ii[i2(xpl, ypl)] : 0;
  return true;
}

}  // namespace umwm
