// UMWM oracle: a CPU restatement of the reference's per-time-step path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
// only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// reference legs load it.  The product path never links or calls it.
//
// PARITY UNPINNED: the reference (Fortran 90, umwm/umwm v2.0.0) ships no
// tests, golden vectors or fixtures, and it cannot be compiled here (no
// Fortran compiler, no netCDF).  This restatement follows the reference
// source line by line, keeping its array order (o fastest, then p, then the
// unrolled wet index i), its loop order and its left-to-right evaluation
// order, so that an fp32 instantiation is what a strict-IEEE fp32 build of
// the reference computes, and an fp64 instantiation is what an
// -fdefault-real-8 -DREAL64 build computes.  Every routine cites the
// reference file:line it restates.
//
// Inputs the reference reads from netCDF files (input/umwm.gridtopo,
// input/umwmin_<time>.nc, restart/umwmrst_<time>.nc) and from
// namelists/exclude.nml are handed over through in-memory stores keyed the
// same way (variable name, time string).

#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <limits>
#include <map>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Namelist text parser (Fortran namelist subset used by main.nml).
// umwm_init.F90:67-92 (groups DOMAIN..OUTPUT), umwm_stokes.F90:25,31-34 (STOKES)
// ---------------------------------------------------------------------------
struct Namelist {
  std::map<std::string, std::map<std::string, std::vector<std::string>>> groups;
  bool ok = true;
  std::string err;
};

static std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

static Namelist parse_namelist(const std::string& text) {
  Namelist nl;
  // strip comments (outside quotes)
  std::string t;
  bool inq = false;
  char q = 0;
  for (size_t k = 0; k < text.size(); ++k) {
    char c = text[k];
    if (inq) {
      t += c;
      if (c == q) inq = false;
      continue;
    }
    if (c == '\'' || c == '"') { inq = true; q = c; t += c; continue; }
    if (c == '!') { while (k < text.size() && text[k] != '\n') ++k; t += '\n'; continue; }
    t += c;
  }
  // tokenize: words, '=', ',', '/', '&NAME', quoted strings
  std::vector<std::string> tok;
  size_t k = 0;
  while (k < t.size()) {
    char c = t[k];
    if (std::isspace((unsigned char)c) || c == ',') {
      if (c == ',') tok.push_back(",");
      ++k; continue;
    }
    if (c == '=' || c == '/') { tok.push_back(std::string(1, c)); ++k; continue; }
    if (c == '\'' || c == '"') {
      size_t e = t.find(c, k + 1);
      if (e == std::string::npos) { nl.ok = false; nl.err = "unterminated string"; return nl; }
      tok.push_back(t.substr(k, e - k + 1));
      k = e + 1; continue;
    }
    size_t s = k;
    while (k < t.size() && !std::isspace((unsigned char)t[k]) && t[k] != ',' && t[k] != '=' && t[k] != '/') ++k;
    tok.push_back(t.substr(s, k - s));
  }
  std::string grp, key;
  for (size_t j = 0; j < tok.size(); ++j) {
    const std::string& w = tok[j];
    if (grp.empty()) {
      if (!w.empty() && w[0] == '&') { grp = lower(w.substr(1)); nl.groups[grp]; }
      continue;
    }
    if (w == "/") { grp.clear(); key.clear(); continue; }
    if (w == ",") continue;
    if (j + 1 < tok.size() && tok[j + 1] == "=") { key = lower(w); nl.groups[grp][key].clear(); ++j; continue; }
    if (key.empty()) { nl.ok = false; nl.err = "value without key in &" + grp; return nl; }
    nl.groups[grp][key].push_back(w);
  }
  return nl;
}

template <typename T> T parse_real(const std::string& s0) {
  std::string s = s0;
  for (auto& c : s) if (c == 'd' || c == 'D') c = 'e';
  if (sizeof(T) == 4) return (T)std::strtof(s.c_str(), nullptr);
  return (T)std::strtod(s.c_str(), nullptr);
}

static bool parse_logical(const std::string& s0) {
  std::string s = lower(s0);
  if (!s.empty() && s[0] == '.') s = s.substr(1);
  return !s.empty() && s[0] == 't';
}

// ---------------------------------------------------------------------------
// Civil time (stands in for datetime-fortran, used only for the clock):
// umwm_top.F90:59-75 (strptime/strftime/timedelta), :157-158 (getminute...)
// days_from_civil: H. Hinnant's published algorithm.
// ---------------------------------------------------------------------------
static int64_t days_from_civil(int64_t y, unsigned m, unsigned d) {
  y -= m <= 2;
  const int64_t era = (y >= 0 ? y : y - 399) / 400;
  const unsigned yoe = (unsigned)(y - era * 400);
  const unsigned doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
  const unsigned doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + (int64_t)doe - 719468;
}
static void civil_from_days(int64_t z, int64_t& y, unsigned& m, unsigned& d) {
  z += 719468;
  const int64_t era = (z >= 0 ? z : z - 146096) / 146097;
  const unsigned doe = (unsigned)(z - era * 146097);
  const unsigned yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  y = (int64_t)yoe + era * 400;
  const unsigned doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  const unsigned mp = (5 * doy + 2) / 153;
  d = doy - (153 * mp + 2) / 5 + 1;
  m = mp < 10 ? mp + 3 : mp - 9;
  y += m <= 2;
}
static bool parse_time(const std::string& s, int64_t& t) {
  int Y, M, D, h, mi, sec;
  if (s.size() < 19) return false;
  if (std::sscanf(s.c_str(), "%d-%d-%d%*c%d:%d:%d", &Y, &M, &D, &h, &mi, &sec) != 6) return false;
  t = days_from_civil(Y, (unsigned)M, (unsigned)D) * 86400 + h * 3600 + mi * 60 + sec;
  return true;
}
static std::string format_time(int64_t t, char sep) {
  int64_t days = t >= 0 ? t / 86400 : -((-t + 86399) / 86400);
  int64_t rem = t - days * 86400;
  int64_t y; unsigned m, d;
  civil_from_days(days, y, m, d);
  char buf[80];
  std::snprintf(buf, sizeof buf, "%04lld-%02u-%02u%c%02lld:%02lld:%02lld", (long long)y, m, d, sep,
                (long long)(rem / 3600), (long long)((rem / 60) % 60), (long long)(rem % 60));
  return buf;
}

// Fortran nint
static long long nint_d(double x) { return (long long)std::llround(x); }

// ---------------------------------------------------------------------------
// The model
// ---------------------------------------------------------------------------
template <typename T>
struct Model {
  std::string nml_text;
  std::string error;

  // namelist (umwm_module.F90:22-82)
  bool isglobal = false, restart = false, gridfromfile = false, topofromfile = false,
       fillestuaries = false, filllakes = false, winds = false, currents = false,
       air_density = false, water_density = false, seaice = false, stokes = false;
  int mm = 0, nm = 0, om = 0, pm = 0, outgrid = 0, outspec = 0, outrst = 0, xpl = 0, ypl = 0;
  T fmin = 0, fmax = 0, fprog = 0, dtg = 0, g = 0, nu_air = 0, nu_water = 0, sfct = 0, kappa = 0, z = 0,
    gustiness = 0, dmin = 0, explim = 0, sin_fac = 0, sin_diss1 = 0, sin_diss2 = 0, sds_fac = 0,
    sds_power = 0, mss_fac = 0, snl_fac = 0, sdt_fac = 0, sbf_fac = 0, sbp_fac = 0, delx = 0, dely = 0,
    dpt = 0, wspd0 = 0, wdir0 = 0, uc0 = 0, vc0 = 0, rhoa0 = 0, rhow0 = 0, fice0 = 0, fice_lth = 0,
    fice_uth = 0;
  std::string starttimestr, stoptimestr;
  std::vector<T> depths_nml = std::vector<T>(100, T(-1));

  // constants (umwm_module.F90:87-91)
  T pi = T(3.141592653589793);
  T twopi = 2 * pi;

  // scalars
  int im = 0, imm = 0, istart = 1, iend = 0, iistart = 1, iiend = 0, iip = 0, lm = 0;
  bool first = true, firstdtg = true, zerocurrents = true;
  T dta = 0, dtr = 0, dtamin = 0, bf1 = 0, bf1a = 0, bf2 = 0, cgmax = 0, cfllim = 0, dlnf = 0, dts = 0,
    dth = 0, dthg = 0, fieldscale1 = 0, fieldscale2 = 0, inv_sds_power = 0, log10overz = 0, mindelx = 0,
    oneovdth = 0, sumt = 0, twopisds_fac = 0, twonu = 0, dtr_temp = 0;
  long long substeps = 0, max_substeps = -1;
  long long cut_count = 0;  // bins whose negative ef was cut to 0 (see run)
  bool stopped = false;

  // 2-d (mm,nm), Fortran order
  std::vector<T> ar_2d, curv, d_2d, dx_2d, dy_2d, dlon, dlat, lat, lon, x, y, rhoa_2d, rhow_2d, wspd_2d,
      wdir_2d, fice_2d, ficeb, ficef, uwb, vwb, uw, vw, uwf, vwf, ucb, uc_2d, ucf, vcb, vc_2d, vcf;
  std::vector<int> ii, mask;
  // 1-d over imm (index 1..imm; [0] unused)
  std::vector<int> iw, ie, is, in, iiw, iie, iis, iin, mi, ni;
  std::vector<T> d, dx, dy, wspd, wdir, uc, vc, rhoa, rhoab, rhoaf, rhow, rhowb, rhowf, rhorat, fice;
  // 1-d over wet points (index 1..im)
  std::vector<int> oc;
  std::vector<T> ar, cd, dxn, dxs, dye, dyw, fcutoff, oneovar, oneovdx, oneovdy, shelt, physics_time_step,
      ustar, taux, tauy, taux_form, tauy_form, taux_skin, tauy_skin, taux_diag, tauy_diag, tailatmx,
      tailatmy, ht, mss, mwd, mwl, mwp, dwd, dwl, dwp, dcp0, dcp, dcg0, dcg, momx, momy, cgmxx, cgmxy, cgmyy;
  // spectral constants
  std::vector<int> pl, pr;
  std::vector<T> th, cth, sth, cth2, dom, f, cth_curv, sth_curv, cth2pp;
  // (om, i) tables; cp0/cg0 carry the ghost column i=0
  std::vector<T> cp0, cg0, k, bf1_renorm, bf2_renorm, cothkd, dwn, fkovg, invcp0, k4, kdk, k3dk, oneoverk4,
      sbf, sdt, sdv, snl_arg, l2, logl2overz, sice;
  // (om, pm, i); e carries the ghost i=0
  std::vector<T> e, ef, dummy, rotl, rotr, sds, snl, ssin;
  // stokes
  std::vector<T> depth, ds, us, vs, usmag, util;
  // stress('ocn') outputs over wet points (index 1..im)
  std::vector<T> taux_ocntop, tauy_ocntop, taux_ocnbot, tauy_ocnbot, taux_snl, tauy_snl, epsx_ocn, epsy_ocn,
      epsx_atm, epsy_atm, tailocnx, tailocny, taux1, tauy1, taux2, tauy2, taux3, tauy3;

  // inputs standing in for files
  std::map<std::string, std::vector<float>> gridtopo;                        // lon, lat, z
  std::map<std::string, std::map<std::string, std::vector<float>>> forcing;  // time -> var -> (mm,nm)
  std::map<std::string, std::pair<std::vector<float>, std::vector<float>>> restarts;
  std::vector<std::pair<int, int>> exclude;

  // screen line records (umwm_top.F90:143-148)
  std::vector<double> screen;
  bool verbose = false;

  // index helpers (1-based o, p, m, n; i as in the reference)
  inline size_t i2(int m, int n) const { return (size_t)(m - 1) + (size_t)(n - 1) * mm; }
  inline size_t oi(int o, int i) const { return (size_t)i * om + (o - 1); }
  inline size_t opi(int o, int p, int i) const { return ((size_t)i * pm + (p - 1)) * om + (o - 1); }
  inline size_t pi_(int p, int i) const { return (size_t)i * pm + (p - 1); }

  bool fail(const std::string& msg) { if (error.empty()) error = msg; return false; }

  // -------------------------------------------------------------------------
  // nmlread, umwm_init.F90:56-193
  // -------------------------------------------------------------------------
  bool nmlread() {
    Namelist nl = parse_namelist(nml_text);
    if (!nl.ok) return fail("namelist: " + nl.err);
    const char* need[] = {"domain", "physics", "grid", "forcing", "forcing_constant", "output"};
    for (auto g_ : need)
      if (!nl.groups.count(g_)) return fail(std::string("namelist: missing group &") + g_);
    auto val = [&](const char* g_, const char* k_) -> const std::vector<std::string>* {
      auto& grp = nl.groups[g_];
      auto it = grp.find(k_);
      if (it == grp.end() || it->second.empty()) return nullptr;
      return &it->second;
    };
    auto R = [&](const char* g_, const char* k_, T& out) { auto v = val(g_, k_); out = v ? parse_real<T>((*v)[0]) : T(0); };
    auto I = [&](const char* g_, const char* k_, int& out) { auto v = val(g_, k_); out = v ? std::atoi((*v)[0].c_str()) : 0; };
    auto L = [&](const char* g_, const char* k_, bool& out) { auto v = val(g_, k_); out = v ? parse_logical((*v)[0]) : false; };
    auto S = [&](const char* g_, const char* k_, std::string& out) {
      auto v = val(g_, k_);
      out = v ? (*v)[0] : std::string();
      if (out.size() >= 2 && (out[0] == '\'' || out[0] == '"')) out = out.substr(1, out.size() - 2);
    };
    L("domain", "isglobal", isglobal); I("domain", "mm", mm); I("domain", "nm", nm); I("domain", "om", om);
    I("domain", "pm", pm); R("domain", "fmin", fmin); R("domain", "fmax", fmax); R("domain", "fprog", fprog);
    S("domain", "starttimestr", starttimestr); S("domain", "stoptimestr", stoptimestr);
    R("domain", "dtg", dtg); L("domain", "restart", restart);
    R("physics", "g", g); R("physics", "nu_air", nu_air); R("physics", "nu_water", nu_water);
    R("physics", "sfct", sfct); R("physics", "kappa", kappa); R("physics", "z", z);
    R("physics", "gustiness", gustiness); R("physics", "dmin", dmin); R("physics", "explim", explim);
    R("physics", "sin_fac", sin_fac); R("physics", "sin_diss1", sin_diss1); R("physics", "sin_diss2", sin_diss2);
    R("physics", "sds_fac", sds_fac); R("physics", "sds_power", sds_power); R("physics", "mss_fac", mss_fac);
    R("physics", "snl_fac", snl_fac); R("physics", "sdt_fac", sdt_fac); R("physics", "sbf_fac", sbf_fac);
    R("physics", "sbp_fac", sbp_fac);
    L("grid", "gridfromfile", gridfromfile); R("grid", "delx", delx); R("grid", "dely", dely);
    L("grid", "topofromfile", topofromfile); R("grid", "dpt", dpt); L("grid", "fillestuaries", fillestuaries);
    L("grid", "filllakes", filllakes);
    L("forcing", "winds", winds); L("forcing", "currents", currents); L("forcing", "air_density", air_density);
    L("forcing", "water_density", water_density); L("forcing", "seaice", seaice);
    R("forcing_constant", "wspd0", wspd0); R("forcing_constant", "wdir0", wdir0); R("forcing_constant", "uc0", uc0);
    R("forcing_constant", "vc0", vc0); R("forcing_constant", "rhoa0", rhoa0); R("forcing_constant", "rhow0", rhow0);
    R("forcing_constant", "fice0", fice0); R("forcing_constant", "fice_lth", fice_lth);
    R("forcing_constant", "fice_uth", fice_uth);
    I("output", "outgrid", outgrid); I("output", "outspec", outspec); I("output", "outrst", outrst);
    I("output", "xpl", xpl); I("output", "ypl", ypl); L("output", "stokes", stokes);
    // &STOKES is read by stokes_drift('init'), umwm_stokes.F90:31-34
    if (!nl.groups.count("stokes")) return fail("namelist: missing group &stokes");
    if (auto v = val("stokes", "depths")) {
      for (size_t j = 0; j < v->size() && j < 100; ++j) depths_nml[j] = parse_real<T>((*v)[j]);
    }
    // checks, umwm_init.F90:95-185
    bool ok = true;
    std::string msg;
    auto bad = [&](const char* m_) { ok = false; msg += std::string(m_) + "; "; };
    const int allowed[10] = {-1, 0, 1, 2, 3, 4, 6, 8, 12, 24};
    auto allowedq = [&](int v) { for (int a : allowed) if (a == v) return true; return false; };
    if (mm < 3 || nm < 3) bad("mm and nm must be > 2");
    if (pm % 4 != 0) bad("pm must be divisible by 4");
    if (fmin <= 0 || fmax <= 0 || fprog <= 0) bad("fmin, fmax and fprog must be > 0");
    if (fmin >= fmax) bad("fmin must be < fmax");
    if (dtg <= 0) bad("dtg must be > 0");
    if (z <= 0) bad("z must be > 0");
    if (gustiness < 0) bad("gustiness must be positive");
    if (dmin <= 0) bad("dmin must be > 0");
    if (!gridfromfile && (delx <= 0 || dely <= 0)) bad("delx and dely must be > 0");
    if (!topofromfile && dpt <= 0) bad("dpt must be > 0");
    if (!allowedq(outgrid)) bad("bad outgrid");
    if (!allowedq(outspec)) bad("bad outspec");
    if (!allowedq(outrst)) bad("bad outrst");
    if (!ok) return fail("namelist: " + msg);
    return true;
  }

  // -------------------------------------------------------------------------
  // alloc(1), umwm_init.F90:202-221
  // -------------------------------------------------------------------------
  void alloc1() {
    size_t n2 = (size_t)mm * nm;
    for (auto* v : {&ar_2d, &curv, &d_2d, &dx_2d, &dy_2d, &dlon, &dlat, &lat, &lon, &x, &y, &rhoa_2d, &rhow_2d,
                    &wspd_2d, &wdir_2d, &fice_2d, &ficeb, &ficef, &uwb, &vwb, &uw, &vw, &uwf, &vwf, &ucb, &uc_2d,
                    &ucf, &vcb, &vc_2d, &vcf})
      v->assign(n2, T(0));
    ii.assign(n2, 0);
    mask.assign(n2, 0);
  }

  static T haversine(T lon1, T lon2, T lat1, T lat2) {  // umwm_util.F90:211-235
    T dlon_ = std::abs(lon2 - lon1), dlat_ = std::abs(lat2 - lat1);
    T s1 = std::sin(T(0.5) * dlat_), s2 = std::sin(T(0.5) * dlon_);
    return 2 * std::asin(std::sqrt(s1 * s1 + std::cos(lat1) * std::cos(lat2) * (s2 * s2)));
  }

  // -------------------------------------------------------------------------
  // grid, umwm_init.F90:381-568
  // -------------------------------------------------------------------------
  bool grid() {
    const T r_earth = T(6.371009e6);
    const T dr = pi / T(180.);
    if (gridfromfile) {
      if (!gridtopo.count("lon") || !gridtopo.count("lat")) return fail("grid: lon/lat not provided");
      for (size_t q = 0; q < lon.size(); ++q) { lon[q] = (T)gridtopo["lon"][q]; lat[q] = (T)gridtopo["lat"][q]; }
      bool loniscontinuous = true;
      T mn = *std::min_element(lon.begin(), lon.end()), mx = *std::max_element(lon.begin(), lon.end());
      if (mn < -175 && mx > 175) loniscontinuous = false;
      std::vector<T> lon_tmp = lon;
      if (!loniscontinuous) for (auto& v : lon) if (v < 0) v = v + 360;
      for (int n = 1; n <= nm; ++n)
        for (int m = 2; m <= mm - 1; ++m) dlon[i2(m, n)] = T(0.5) * (lon[i2(m + 1, n)] - lon[i2(m - 1, n)]);
      for (int n = 1; n <= nm; ++n) {
        dlon[i2(1, n)] = 2 * dlon[i2(2, n)] - dlon[i2(3, n)];
        dlon[i2(mm, n)] = 2 * dlon[i2(mm - 1, n)] - dlon[i2(mm - 2, n)];
      }
      for (int n = 2; n <= nm - 1; ++n)
        for (int m = 1; m <= mm; ++m) dlat[i2(m, n)] = T(0.5) * (lat[i2(m, n + 1)] - lat[i2(m, n - 1)]);
      for (int m = 1; m <= mm; ++m) {
        dlat[i2(m, 1)] = 2 * dlat[i2(m, 2)] - dlat[i2(m, 3)];
        dlat[i2(m, nm)] = 2 * dlat[i2(m, nm - 1)] - dlat[i2(m, nm - 2)];
      }
      (void)dr;
      lon = lon_tmp;
      std::vector<T> rlon(lon.size()), rlat(lat.size());
      for (size_t q = 0; q < lon.size(); ++q) { rlon[q] = lon[q] * twopi / T(360.); rlat[q] = lat[q] * twopi / T(360.); }
      for (int n = 1; n <= nm; ++n)
        for (int m = 2; m <= mm - 1; ++m)
          dx_2d[i2(m, n)] = r_earth * haversine(T(0.5) * (rlon[i2(m - 1, n)] + rlon[i2(m, n)]),
                                                T(0.5) * (rlon[i2(m, n)] + rlon[i2(m + 1, n)]),
                                                T(0.5) * (rlat[i2(m - 1, n)] + rlat[i2(m, n)]),
                                                T(0.5) * (rlat[i2(m, n)] + rlat[i2(m + 1, n)]));
      for (int n = 1; n <= nm; ++n) {
        dx_2d[i2(1, n)] = 2 * dx_2d[i2(2, n)] - dx_2d[i2(3, n)];
        dx_2d[i2(mm, n)] = 2 * dx_2d[i2(mm - 1, n)] - dx_2d[i2(mm - 2, n)];
      }
      for (int n = 2; n <= nm - 1; ++n)
        for (int m = 1; m <= mm; ++m)
          dy_2d[i2(m, n)] = r_earth * haversine(T(0.5) * (rlon[i2(m, n - 1)] + rlon[i2(m, n)]),
                                                T(0.5) * (rlon[i2(m, n)] + rlon[i2(m, n + 1)]),
                                                T(0.5) * (rlat[i2(m, n - 1)] + rlat[i2(m, n)]),
                                                T(0.5) * (rlat[i2(m, n)] + rlat[i2(m, n + 1)]));
      for (int m = 1; m <= mm; ++m) {
        dy_2d[i2(m, 1)] = 2 * dy_2d[i2(m, 2)] - dy_2d[i2(m, 3)];
        dy_2d[i2(m, nm)] = 2 * dy_2d[i2(m, nm - 1)] - dy_2d[i2(m, nm - 2)];
      }
      std::fill(curv.begin(), curv.end(), T(0));
      auto bearing = [&](int ma, int mb, int n) {  // atan2 expression of umwm_init.F90:493-495
        T dl = rlon[i2(mb, n)] - rlon[i2(ma, n)];
        return std::atan2(std::sin(dl) * std::cos(rlat[i2(mb, n)]),
                          std::cos(rlat[i2(ma, n)]) * std::sin(rlat[i2(mb, n)]) -
                              std::sin(rlat[i2(ma, n)]) * std::cos(rlat[i2(mb, n)]) * std::cos(dl));
      };
      for (int n = 1; n <= nm; ++n)
        for (int m = 2; m <= mm - 1; ++m) curv[i2(m, n)] = bearing(m - 1, m + 1, n);
      if (isglobal) {
        for (int n = 1; n <= nm; ++n) {
          curv[i2(1, n)] = bearing(mm, 2, n);
          curv[i2(mm, n)] = bearing(mm - 1, 1, n);
        }
      } else {
        for (int n = 1; n <= nm; ++n) { curv[i2(1, n)] = curv[i2(2, n)]; curv[i2(mm, n)] = curv[i2(mm - 1, n)]; }
      }
      for (auto& v : curv) v = v - T(0.5) * pi;
    } else {
      std::fill(dx_2d.begin(), dx_2d.end(), delx);
      std::fill(dy_2d.begin(), dy_2d.end(), dely);
      std::fill(curv.begin(), curv.end(), T(0));
      std::fill(lon.begin(), lon.end(), T(0));
      std::fill(lat.begin(), lat.end(), T(0));
      std::fill(dlon.begin(), dlon.end(), T(0));
      std::fill(dlat.begin(), dlat.end(), T(0));
      for (int n = 1; n <= nm; ++n) x[i2(1, n)] = 0;
      for (int m = 2; m <= mm; ++m)
        for (int n = 1; n <= nm; ++n)
          x[i2(m, n)] = x[i2(m - 1, n)] + T(0.5) * (dx_2d[i2(m - 1, n)] + dx_2d[i2(m, n)]);
      for (int m = 1; m <= mm; ++m) y[i2(m, 1)] = 0;
      for (int n = 2; n <= nm; ++n)
        for (int m = 1; m <= mm; ++m)
          y[i2(m, n)] = y[i2(m, n - 1)] + T(0.5) * (dy_2d[i2(m, n - 1)] + dy_2d[i2(m, n)]);
    }
    if (topofromfile) {
      if (!gridtopo.count("z")) return fail("grid: z not provided");
      for (size_t q = 0; q < d_2d.size(); ++q) d_2d[q] = (T)gridtopo["z"][q];
    } else {
      std::fill(d_2d.begin(), d_2d.end(), dpt);
    }
    for (size_t q = 0; q < ar_2d.size(); ++q) ar_2d[q] = dx_2d[q] * dy_2d[q];
    return true;
  }

  // -------------------------------------------------------------------------
  // masks + fill, umwm_init.F90:571-718
  // -------------------------------------------------------------------------
  void fill(int m, int n, int& fillcount) {  // recursive flood fill, umwm_init.F90:698-718
    // iterative form of the same depth-first recursion (identical visit order)
    std::vector<std::pair<int, int>> stack;
    std::vector<int> state;
    auto enter = [&](int mm_, int nn_) -> bool {
      if (mm_ == 1 || mm_ == mm || nn_ == 1 || nn_ == nm) return false;
      mask[i2(mm_, nn_)] = 0;
      fillcount++;
      return true;
    };
    if (!enter(m, n)) return;
    stack.push_back({m, n});
    state.push_back(0);
    while (!stack.empty()) {
      auto [cm, cn] = stack.back();
      int& st = state.back();
      int dm[4] = {-1, 1, 0, 0}, dn[4] = {0, 0, -1, 1};
      bool pushed = false;
      while (st < 4) {
        int tm = cm + dm[st], tn = cn + dn[st];
        st++;
        if (mask[i2(tm, tn)] == 1) {
          if (enter(tm, tn)) { stack.push_back({tm, tn}); state.push_back(0); pushed = true; break; }
        }
      }
      if (!pushed && st >= 4) { stack.pop_back(); state.pop_back(); }
    }
  }

  void masks() {
    std::fill(mask.begin(), mask.end(), 1);
    for (int m = 1; m <= mm; ++m) { mask[i2(m, 1)] = 0; mask[i2(m, nm)] = 0; }
    if (!isglobal)
      for (int n = 1; n <= nm; ++n) { mask[i2(1, n)] = 0; mask[i2(mm, n)] = 0; }
    if (topofromfile) {
      for (size_t q = 0; q < d_2d.size(); ++q)
        if (d_2d[q] >= 0) { mask[q] = 0; d_2d[q] = dmin; }
      for (auto& v : d_2d) v = std::abs(v);
      for (auto& v : d_2d) if (v < dmin) v = dmin;
      if (fillestuaries) {
        bool iterate = true;
        while (iterate) {
          iterate = false;
          for (int n = 2; n <= nm - 1; ++n)
            for (int m = 2; m <= mm - 1; ++m) {
              if (mask[i2(m, n)] == 1) {
                int cnt = 0;
                if (mask[i2(m - 1, n)] == 1) cnt++;
                if (mask[i2(m + 1, n)] == 1) cnt++;
                if (mask[i2(m, n - 1)] == 1) cnt++;
                if (mask[i2(m, n + 1)] == 1) cnt++;
                if (cnt <= 1) { mask[i2(m, n)] = 0; iterate = true; }
              }
            }
        }
      }
      if (filllakes) {
        for (auto& pr_ : exclude) { int fc = 0; fill(pr_.first, pr_.second, fc); }
      }
    } else {
      for (size_t q = 0; q < d_2d.size(); ++q) if (mask[q] == 0) d_2d[q] = dmin;
    }
    im = 0;
    for (int v : mask) im += (v == 1);
    imm = mm * nm;
  }

  // partition (serial), umwm_init.F90:734-738
  void partition() { istart = 1; iend = im; iistart = istart; iiend = iend; }

  // -------------------------------------------------------------------------
  // alloc(2) + remap, umwm_init.F90:224-376, 875-1237 (serial: remap_dir='v')
  // -------------------------------------------------------------------------
  void alloc2() {
    auto I1 = [&](std::vector<int>& v, size_t n) { v.assign(n, 0); };
    auto R1 = [&](std::vector<T>& v, size_t n) { v.assign(n, T(0)); };
    size_t nimm = imm + 1, nim = im + 1;
    dom.assign(om, 0); f.assign(om, 0);
    cth.assign(pm, 0); cth2.assign(pm, 0); sth.assign(pm, 0); th.assign(pm, 0);
    pl.assign(pm, 0); pr.assign(pm, 0);
    cth_curv.assign((size_t)pm * nim, 0); sth_curv.assign((size_t)pm * nim, 0);
    for (auto* v : {&iw, &ie, &is, &in, &iiw, &iie, &iis, &iin, &mi, &ni}) I1(*v, nimm);
    I1(oc, nim);
    for (auto* v : {&ar, &cd, &dxn, &dxs, &dye, &dyw, &fcutoff, &oneovar, &oneovdx, &oneovdy, &shelt,
                    &physics_time_step, &ustar, &taux, &tauy, &taux_form, &tauy_form, &taux_skin, &tauy_skin,
                    &taux_diag, &tauy_diag, &tailatmx, &tailatmy, &ht, &mss, &mwd, &mwl, &mwp, &dwd, &dwl, &dwp,
                    &dcp0, &dcp, &dcg0, &dcg, &momx, &momy, &cgmxx, &cgmxy, &cgmyy})
      R1(*v, nim);
    for (auto* v : {&d, &dx, &dy, &wspd, &wdir, &uc, &vc, &rhoa, &rhoab, &rhoaf, &rhow, &rhowb, &rhowf,
                    &rhorat, &fice})
      R1(*v, nimm);
    size_t n_oi = (size_t)om * nim;
    for (auto* v : {&cp0, &cg0, &k, &bf1_renorm, &bf2_renorm, &cothkd, &dwn, &fkovg, &invcp0, &k4, &kdk, &k3dk,
                    &oneoverk4, &sbf, &sdt, &sdv, &snl_arg, &l2, &logl2overz, &sice})
      R1(*v, n_oi);
    size_t n_opi = (size_t)om * pm * nim;
    for (auto* v : {&e, &ef, &dummy, &rotl, &rotr, &sds, &snl, &ssin}) R1(*v, n_opi);
  }

  void remap() {
    int i = 0;
    // remap_dir = 'v': m outer, n inner; sea points first, then land points
    for (int m = 1; m <= mm; ++m)
      for (int n = 1; n <= nm; ++n)
        if (mask[i2(m, n)] == 1) {
          ++i; ii[i2(m, n)] = i; dx[i] = dx_2d[i2(m, n)]; dy[i] = dy_2d[i2(m, n)]; d[i] = d_2d[i2(m, n)];
        }
    for (int m = 1; m <= mm; ++m)
      for (int n = 1; n <= nm; ++n)
        if (mask[i2(m, n)] == 0) {
          ++i; ii[i2(m, n)] = i; dx[i] = dx_2d[i2(m, n)]; dy[i] = dy_2d[i2(m, n)]; d[i] = d_2d[i2(m, n)];
        }
    for (int n = 1; n <= nm; ++n)
      for (int m = 1; m <= mm; ++m) { int q = ii[i2(m, n)]; mi[q] = m; ni[q] = n; }
    for (int n = 2; n <= nm - 1; ++n)
      for (int m = 2; m <= mm - 1; ++m) {
        int q = ii[i2(m, n)];
        is[q] = ii[i2(m, n - 1)]; in[q] = ii[i2(m, n + 1)]; iw[q] = ii[i2(m - 1, n)]; ie[q] = ii[i2(m + 1, n)];
      }
    if (isglobal) {
      for (int n = 2; n <= nm - 1; ++n) {
        int q = ii[i2(1, n)];
        is[q] = ii[i2(1, n - 1)]; in[q] = ii[i2(1, n + 1)]; iw[q] = ii[i2(mm, n)]; ie[q] = ii[i2(2, n)];
        q = ii[i2(mm, n)];
        is[q] = ii[i2(mm, n - 1)]; in[q] = ii[i2(mm, n + 1)]; iw[q] = ii[i2(mm - 1, n)]; ie[q] = ii[i2(1, n)];
      }
    }
    iis = is; iin = in; iiw = iw; iie = ie;
    for (int q = istart; q <= iend; ++q) {
      dxn[q] = T(0.5) * (dx[q] + dx[iin[q]]);
      dxs[q] = T(0.5) * (dx[q] + dx[iis[q]]);
      dye[q] = T(0.5) * (dy[q] + dy[iie[q]]);
      dyw[q] = T(0.5) * (dy[q] + dy[iiw[q]]);
    }
    // e = tiny(e) including the ghost column, umwm_init.F90:1182
    std::fill(e.begin(), e.end(), std::numeric_limits<T>::min());
    for (int q = istart; q <= iend; ++q) {
      if (is[q] < iistart || is[q] > iiend) is[q] = iistart - 1;
      if (in[q] < iistart || in[q] > iiend) in[q] = iistart - 1;
      if (ie[q] < iistart || ie[q] > iiend) ie[q] = iistart - 1;
      if (iw[q] < iistart || iw[q] > iiend) iw[q] = iistart - 1;
    }
  }

  std::vector<T> remap_mn2i(const std::vector<T>& fmn) {  // umwm_util.F90:46-64
    std::vector<T> out(imm + 1, T(0));
    for (int n = 1; n <= nm; ++n)
      for (int m = 1; m <= mm; ++m) out[ii[i2(m, n)]] = fmn[i2(m, n)];
    return out;
  }

  // -------------------------------------------------------------------------
  // input_nc, umwm_io.F90:13-93 (the netCDF file is an in-memory store here)
  // -------------------------------------------------------------------------
  bool readfile() const { return winds || currents || air_density || water_density || seaice; }

  bool input_nc(const std::string& timestr) {
    std::string key = timestr;
    if (key.size() >= 11) key[10] = '_';
    std::map<std::string, std::vector<float>>* snap = nullptr;
    if (readfile()) {
      auto it = forcing.find(key);
      if (it == forcing.end()) return fail("input_nc: no forcing for " + key);
      snap = &it->second;
    }
    auto get = [&](const char* var, std::vector<T>& dst) -> bool {
      auto it = snap->find(var);
      if (it == snap->end()) return fail(std::string("input_nc: missing variable ") + var + " for " + key);
      for (size_t q = 0; q < dst.size(); ++q) dst[q] = (T)it->second[q];
      return true;
    };
    if (winds) {
      if (!get("uw", uwf) || !get("vw", vwf)) return false;
    } else {
      std::fill(wspd.begin() + 1, wspd.end(), wspd0);
      std::fill(wdir.begin() + 1, wdir.end(), wdir0);
    }
    if (currents) {
      if (!get("uc", ucf) || !get("vc", vcf)) return false;
    } else {
      std::fill(ucf.begin(), ucf.end(), uc0); std::fill(vcf.begin(), vcf.end(), vc0);
      std::fill(uc.begin() + 1, uc.end(), uc0); std::fill(vc.begin() + 1, vc.end(), vc0);
    }
    if (seaice) {
      if (!get("fice", ficef)) return false;
    } else {
      std::fill(fice_2d.begin(), fice_2d.end(), fice0);
      std::fill(fice.begin() + 1, fice.end(), fice0);
    }
    for (size_t q = 0; q < mask.size(); ++q) if (mask[q] == 0) { ucf[q] = 0; vcf[q] = 0; }
    if (air_density) {
      if (!get("rhoa", rhoa_2d)) return false;
    } else {
      std::fill(rhoa_2d.begin(), rhoa_2d.end(), rhoa0); std::fill(rhoa.begin() + 1, rhoa.end(), rhoa0);
    }
    if (water_density) {
      if (!get("rhow", rhow_2d)) return false;
    } else {
      std::fill(rhow_2d.begin(), rhow_2d.end(), rhow0); std::fill(rhow.begin() + 1, rhow.end(), rhow0);
    }
    rhoaf = remap_mn2i(rhoa_2d);
    rhowf = remap_mn2i(rhow_2d);
    return true;
  }

  // -------------------------------------------------------------------------
  // init, umwm_init.F90:1240-1419
  // -------------------------------------------------------------------------
  void init() {
    dlnf = (std::log(fmax) - std::log(fmin)) / T(om - 1);
    for (int o = 1; o <= om; ++o) f[o - 1] = std::exp(std::log(fmin) + T(o - 1) * dlnf);
    dth = twopi / T(pm);
    dthg = dth * g;
    oneovdth = T(1.) / dth;
    log10overz = std::log(T(10.) / z);
    twopisds_fac = twopi * sds_fac;
    twonu = T(2.) * nu_water;
    fieldscale1 = sin_diss1 / sin_fac;
    fieldscale2 = sin_diss2 / sin_diss1;
    inv_sds_power = T(1.) / sds_power;
    if (pm % 8 == 0) cfllim = std::cos(T(0.25) * pi - T(0.5) * dth);
    else cfllim = T(1.) / std::sqrt(T(2.));
    for (int q = istart; q <= iend; ++q) {
      ar[q] = dx[q] * dy[q];
      oneovdx[q] = T(1.) / dx[q];
      oneovdy[q] = T(1.) / dy[q];
      oneovar[q] = T(1.) / ar[q];
    }
    bf1 = std::exp(T(-16) * dlnf * dlnf);
    bf2 = std::exp(T(-64) * dlnf * dlnf);
    bf1a = bf1 / (bf1 + bf2);
    bf2 = bf2 / (bf1 + bf2);
    bf1 = bf1a;
    for (int p = 1; p <= pm; ++p) th[p - 1] = (T(p) - T(0.5) * T(pm + 1)) * dth;
    for (int p = 1; p <= pm; ++p) { cth[p - 1] = std::cos(th[p - 1]); sth[p - 1] = std::sin(th[p - 1]); }
    for (int q = istart; q <= iend; ++q)
      for (int p = 1; p <= pm; ++p) {
        T cv = curv[i2(mi[q], ni[q])];
        cth_curv[pi_(p, q)] = std::cos(th[p - 1] + cv);
        sth_curv[pi_(p, q)] = std::sin(th[p - 1] + cv);
      }
    for (int p = 1; p <= pm; ++p) { pl[p - 1] = p + 1; pr[p - 1] = p - 1; }
    pl[pm - 1] = 1;
    pr[0] = pm;
    for (int o = 1; o <= om; ++o) dom[o - 1] = twopi * dlnf * f[o - 1];
    for (int p = 1; p <= pm; ++p) { T c = std::cos(dth * T(p - 1)); cth2[p - 1] = c * c; }
    cth2pp.assign((size_t)pm * pm, 0);
    for (int p = 1; p <= pm; ++p)
      for (int pp = 1; pp <= pm; ++pp) {
        int ind = pp - p + 1;
        if (ind <= 0) ind = pm + ind;
        cth2pp[(size_t)(p - 1) * pm + (pp - 1)] = cth2[ind - 1] * dth;
      }
    dispersion(T(1e-2));
    T mdx = std::numeric_limits<T>::max();
    for (size_t q = 0; q < mask.size(); ++q)
      if (mask[q] == 1) { mdx = std::min(mdx, dx_2d[q]); }
    T mdy = std::numeric_limits<T>::max();
    for (size_t q = 0; q < mask.size(); ++q)
      if (mask[q] == 1) { mdy = std::min(mdy, dy_2d[q]); }
    mindelx = std::min(mdx, mdy);
    cgmax = -std::numeric_limits<T>::max();
    for (int q = istart; q <= iend; ++q)
      for (int o = 1; o <= om; ++o) cgmax = std::max(cgmax, cg0[oi(o, q)]);
    dtamin = T(0.98) * cfllim * mindelx / cgmax;
    first = true;
    firstdtg = !restart;
    if (seaice) fice = remap_mn2i(ficef);
    if (winds) {
      std::vector<T> w2(uwf.size());
      for (size_t q = 0; q < w2.size(); ++q) w2[q] = std::sqrt(uwf[q] * uwf[q] + vwf[q] * vwf[q]);
      wspd = remap_mn2i(w2);
    }
    for (int q = istart; q <= iend; ++q) {
      cd[q] = T(1.2e-3);
      if (wspd[q] > 11) cd[q] = (T(0.49) + T(0.065) * wspd[q]) * T(1e-3);
    }
    for (int q = istart; q <= iend; ++q) ustar[q] = std::sqrt(cd[q]) * wspd[q];
    iip = ii[i2(xpl, ypl)];
  }

  // -------------------------------------------------------------------------
  // dispersion, umwm_init.F90:1422-1658
  // -------------------------------------------------------------------------
  void dispersion(T tol) {
    std::vector<T> f_nd((size_t)om * (im + 1)), kd((size_t)om * (im + 1));
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      for (int o = 1; o <= om; ++o) {
        cp0[oi(o, q)] = twopi * std::sqrt(d[q] / g);
        f_nd[oi(o, q)] = cp0[oi(o, q)] * f[o - 1];
        k[oi(o, q)] = f_nd[oi(o, q)] * f_nd[oi(o, q)];
      }
      T b = sfct / (rhow0 * g * (d[q] * d[q]));
      for (int o = 1; o <= om; ++o) {
        int counter = 1;
        T dk = T(2.) * tol;
        T kk = k[oi(o, q)], fn = f_nd[oi(o, q)];
        while (std::abs(dk) > tol) {
          T t = std::tanh(kk);
          dk = -(fn * fn - kk * t * (T(1.) + b * kk * kk)) /
               (T(3.) * b * kk * kk * t + t + kk * (T(1.) + b * kk * kk) * (T(1.) - t * t));
          kk = kk - dk;
          if (counter == 1000) break;
          counter++;
        }
        k[oi(o, q)] = std::abs(kk) / d[q];
      }
    }
    for (int q = istart; q <= iend; ++q)
      for (int o = 1; o <= om; ++o) {
        kd[oi(o, q)] = k[oi(o, q)] * d[q];
        if (kd[oi(o, q)] > T(20.)) kd[oi(o, q)] = T(20.);
      }
    std::fill(cp0.begin(), cp0.end(), std::numeric_limits<T>::min());
    std::fill(cg0.begin(), cg0.end(), std::numeric_limits<T>::min());
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q)
      for (int o = 1; o <= om; ++o) {
        size_t a = oi(o, q);
        T kk = k[a];
        cp0[a] = twopi * f[o - 1] / kk;
        cg0[a] = cp0[a] * (T(0.5) + kk * d[q] / std::sinh(T(2.) * kd[a]) + sfct * kk * kk / (rhow0 * g + sfct * kk * kk));
        dwn[a] = dom[o - 1] / std::abs(cg0[a]);
        l2[a] = T(0.5) * std::abs(cp0[a]) / f[o - 1];
        k4[a] = std::pow(kk, T(4.));
        oneoverk4[a] = T(1.) / k4[a];
        kdk[a] = kk * dwn[a];
        k3dk[a] = std::pow(kk, T(3.)) * dwn[a];
        fkovg[a] = f[o - 1] * kk / g;
        cothkd[a] = std::cosh(T(0.2) * kd[a]) / std::sinh(T(0.2) * kd[a]);
        invcp0[a] = T(1.) / cp0[a];
        sbf[a] = sbf_fac * kk / (std::sinh(T(2.) * kd[a])) + sbp_fac * kk / (std::cosh(kd[a]) * std::cosh(kd[a]));
        sdv[a] = T(4.) * nu_water * std::pow(kk, T(2.));
      }
    for (int q = istart; q <= iend; ++q)
      for (int o = 1; o <= om - 2; ++o) {
        bf1_renorm[oi(o, q)] = snl_fac * bf1 * kdk[oi(o + 1, q)] / kdk[oi(o, q)];
        bf2_renorm[oi(o, q)] = snl_fac * bf2 * kdk[oi(o + 2, q)] / kdk[oi(o, q)];
        snl_arg[oi(o, q)] = T(1.) - (bf1_renorm[oi(o, q)] + bf2_renorm[oi(o, q)]);
      }
    for (int q = istart; q <= iend; ++q)
      for (int o = 1; o <= om; ++o) {
        size_t a = oi(o, q);
        logl2overz[a] = std::log(l2[a] / z);
        if (l2[a] > T(20.)) logl2overz[a] = std::log(T(20.) / z);
      }
    for (int o = 1; o <= om; ++o) {
      T mc = std::numeric_limits<T>::max(), mg = std::numeric_limits<T>::max();
      for (int q = istart; q <= iend; ++q) { mc = std::min(mc, cp0[oi(o, q)]); mg = std::min(mg, cg0[oi(o, q)]); }
      cp0[oi(o, iistart - 1)] = mc;
      cg0[oi(o, iistart - 1)] = mg;
    }
  }

  // -------------------------------------------------------------------------
  // stokes_drift, umwm_stokes.F90:13-132
  // -------------------------------------------------------------------------
  void stokes_init() {
    lm = 0;
    for (auto v : depths_nml) lm += (v >= 0);
    depth.assign(lm, 0);
    for (int l = 0; l < lm; ++l) depth[l] = -depths_nml[l];
    us.assign((size_t)(im + 1) * lm, 0); vs.assign((size_t)(im + 1) * lm, 0);
    usmag.assign((size_t)(im + 1) * lm, 0); ds.assign(im + 1, 0);
    util.assign((size_t)om * (im + 1) * lm, 0);
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q)
      for (int l = 1; l <= lm; ++l) {
        for (int o = 1; o <= om; ++o) {
          T kk = k[oi(o, q)];
          T kd = kk * d[q];
          T arg = T(2) * kk * (depth[l - 1] + d[q]);
          T u;
          if (std::abs(arg) > 50 || kd > 50)
            u = twopi * f[o - 1] * T(2) * (kk * kk) * std::exp(T(2) * kk * depth[l - 1]) * dwn[oi(o, q)] * dth;
          else {
            T sh = std::sinh(kd);
            u = twopi * f[o - 1] * (kk * kk) * std::cosh(T(2) * kk * (depth[l - 1] + d[q])) / (sh * sh) *
                dwn[oi(o, q)] * dth;
          }
          util[utl(o, q, l)] = u;
        }
        if (std::abs(depth[l - 1]) > d[q])
          for (int o = 1; o <= om; ++o) util[utl(o, q, l)] = 0;
      }
  }
  inline size_t utl(int o, int q, int l) const { return ((size_t)(l - 1) * (im + 1) + q) * om + (o - 1); }
  inline size_t il(int q, int l) const { return (size_t)(l - 1) * (im + 1) + q; }

  void stokes_drift() {
    // euler = exp(1d0) stored as real(rk), eulerinv = 1/euler: umwm_constants.F90:17-18
    T eulerinv = T(1) / (T)(std::exp(1.0));
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      for (int l = 1; l <= lm; ++l) {
        T su = 0, sv = 0;
        for (int p = 1; p <= pm; ++p)
          for (int o = 1; o <= om; ++o) {
            su = su + util[utl(o, q, l)] * e[opi(o, p, q)] * cth[p - 1];
            sv = sv + util[utl(o, q, l)] * e[opi(o, p, q)] * sth[p - 1];
          }
        us[il(q, l)] = su; vs[il(q, l)] = sv;
        usmag[il(q, l)] = std::sqrt(su * su + sv * sv);
      }
      ds[q] = 0;
      if (lm >= 1 && usmag[il(q, 1)] != 0) {
        T ust_ef = usmag[il(q, 1)] * eulerinv;
        for (int l = 2; l <= lm; ++l)
          if (usmag[il(q, l)] < ust_ef) {
            ds[q] = (std::abs(usmag[il(q, l - 1)] - ust_ef) * depth[l - 1] +
                     std::abs(usmag[il(q, l)] - ust_ef) * depth[l - 2]) /
                    (usmag[il(q, l - 1)] - usmag[il(q, l)]);
            break;
          }
      }
      ds[q] = -ds[q];
    }
  }

  // -------------------------------------------------------------------------
  // forcing, umwm_forcing.F90:11-99
  // -------------------------------------------------------------------------
  bool forcinginput(const std::string& timestr) {
    if (winds) { uwb = uwf; vwb = vwf; }
    if (currents) { ucb = ucf; vcb = vcf; }
    if (air_density) rhoab = rhoaf;
    if (water_density) rhowb = rhowf;
    if (seaice) ficeb = ficef;
    if (readfile()) return input_nc(timestr);
    return true;
  }

  // Wind gust draws in place of Fortran random_number (umwm_forcing.F90:49-56):
  // uniform [0, 1) from the top 24 bits of a twice-applied SplitMix64
  // finaliser (Steele, Lea and Flood, 2014) keyed by (seed, substep) and
  // (cell, component); the same draws as the GPU library makes.
  static uint64_t splitmix64_mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  static float gust_uniform(unsigned seed, unsigned step, unsigned cell, unsigned comp) {
    const uint64_t key = splitmix64_mix(((uint64_t)seed << 32) | step);
    const uint64_t z = splitmix64_mix(key ^ (((uint64_t)cell << 1) | comp));
    return (float)(z >> 40) * (1.f / 16777216.f);
  }
  unsigned gust_seed = 1;

  // forcinginterpolate, umwm_forcing.F90:40-99
  void forcinginterpolate() {
    T s = sumt / dtg;
    if (winds) {
      for (size_t q = 0; q < uw.size(); ++q) {
        uw[q] = uwb[q] * (T(1) - sumt / dtg) + uwf[q] * sumt / dtg;
        vw[q] = vwb[q] * (T(1) - sumt / dtg) + vwf[q] * sumt / dtg;
      }
      if (gustiness > 0)  // :49-61, one draw per cell and component each substep
        for (size_t q = 0; q < uw.size(); ++q) {
          const T gu = gustiness * (T(2) * T(gust_uniform(gust_seed, (unsigned)substeps, (unsigned)q, 0)) - T(1));
          const T gv = gustiness * (T(2) * T(gust_uniform(gust_seed, (unsigned)substeps, (unsigned)q, 1)) - T(1));
          uw[q] = uw[q] * (T(1) + gu);
          vw[q] = vw[q] * (T(1) + gv);
        }
      for (size_t q = 0; q < uw.size(); ++q) {
        wspd_2d[q] = std::sqrt(uw[q] * uw[q] + vw[q] * vw[q]);
        wdir_2d[q] = std::atan2(vw[q], uw[q]);
      }
      wspd = remap_mn2i(wspd_2d);
      wdir = remap_mn2i(wdir_2d);
    }
    (void)s;
    if (seaice) {
      for (size_t q = 0; q < fice_2d.size(); ++q) fice_2d[q] = ficeb[q] * (T(1) - sumt / dtg) + ficef[q] * sumt / dtg;
      fice = remap_mn2i(fice_2d);
    }
    if (currents) {
      for (size_t q = 0; q < uc_2d.size(); ++q) {
        uc_2d[q] = ucb[q] * (T(1) - sumt / dtg) + ucf[q] * sumt / dtg;
        vc_2d[q] = vcb[q] * (T(1) - sumt / dtg) + vcf[q] * sumt / dtg;
      }
      uc = remap_mn2i(uc_2d);
      vc = remap_mn2i(vc_2d);
    }
    if (air_density)
      for (int q = 1; q <= imm; ++q) rhoa[q] = rhoab[q] * (T(1) - sumt / dtg) + rhoaf[q] * sumt / dtg;
    if (water_density)
      for (int q = 1; q <= imm; ++q) rhow[q] = rhowb[q] * (T(1) - sumt / dtg) + rhowf[q] * sumt / dtg;
    for (int q = 1; q <= imm; ++q) rhorat[q] = rhoa[q] / rhow[q];
  }

  // -------------------------------------------------------------------------
  // sheltering_coare35, umwm_sheltering.F90:49-79
  // -------------------------------------------------------------------------
  static T sheltering_coare35(T w) {
    const T x1 = 15, x2 = 33, x3 = 60, y1 = T(0.10), y2 = T(0.09), y3 = T(0.06);
    const T intercept = T(0.04), curvature = T(0.65), decay = T(1.6);
    T slope1 = (y1 - intercept) / x1;
    T slope2 = (y3 - y2) / (x3 - x2);
    T c = curvature * (slope2 - slope1) / (x2 - x1);
    T b = slope1 - 2 * c * x1;
    T a = y1 - b * x1 - c * (x1 * x1);
    T s1 = a + b * x2 + c * (x2 * x2);
    if (w <= x1) return intercept + slope1 * w;
    if (w > x1 && w <= x2) return a + b * w + c * (w * w);
    return s1 * std::exp(-(w - x2) / (decay * w));
  }

  // -------------------------------------------------------------------------
  // sin_d12, umwm_source_functions.F90:16-82
  // -------------------------------------------------------------------------
  void sin_d12() {
    for (int q = 1; q <= imm; ++q) wspd[q] = std::max(wspd[q], T(1e-2));
    for (int q = istart; q <= iend; ++q) {
      fcutoff[q] = T(0.53) * g / wspd[q];
      if (fcutoff[q] > fprog) fcutoff[q] = fprog;
    }
    for (int q = istart; q <= iend; ++q)
      for (int o = om - 2; o >= 1; --o) {
        oc[q] = o;
        if (fcutoff[q] > f[o - 1]) break;
      }
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      shelt[q] = sheltering_coare35(wspd[q]);
      for (int p = 1; p <= pm; ++p) {
        T cw = std::cos(wdir[q] - th[p - 1]);
        for (int o = 1; o <= om; ++o) {
          T s = (wspd[q] + T(2.5) * ustar[q] * logl2overz[oi(o, q)]) * cw - cp0[oi(o, q)] - uc[q] * cth[p - 1] -
                vc[q] * sth[p - 1];
          s = sin_fac * std::abs(s) * s;
          if (s > 0) s = s * shelt[q] / sin_fac;
          if (s < 0) s = s * fieldscale1;
          if (s < 0 && cw > 0) s = s * fieldscale2;
          s = (T(1) - fice[q]) * twopi * rhorat[q] * s * fkovg[oi(o, q)];
          if (o > oc[q]) s = std::max(s, T(0));
          ssin[opi(o, p, q)] = s;
        }
      }
    }
  }

  // sds_d12, umwm_source_functions.F90:85-105
  void sds_d12() {
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q)
      for (int p = 1; p <= pm; ++p) {
        dummy[opi(1, p, q)] = 0;
        for (int o = 2; o <= om; ++o) {
          T acc = 0;
          if (mss_fac > 0) {
            for (int pp = 1; pp <= pm; ++pp) acc = acc + e[opi(o - 1, pp, q)] * cth2pp[(size_t)(p - 1) * pm + (pp - 1)];
            dummy[opi(o, p, q)] = dummy[opi(o - 1, p, q)] + acc * k3dk[oi(o - 1, q)];
          } else {
            dummy[opi(o, p, q)] = 0;
          }
        }
        for (int o = 1; o <= om; ++o) {
          T t = T(1) + mss_fac * dummy[opi(o, p, q)];
          dummy[opi(o, p, q)] = t * t;
          sds[opi(o, p, q)] = twopisds_fac * f[o - 1] * dummy[opi(o, p, q)] *
                              std::pow(e[opi(o, p, q)] * k4[oi(o, q)], sds_power);
        }
      }
  }

  // s_ice, umwm_source_functions.F90:108-153
  void s_ice() {
    const T H_th = T(3.0), C1 = T(-5.35e-6), C2 = C1 * H_th;
    std::fill(sice.begin(), sice.end(), T(0));
    for (int q = istart; q <= iend; ++q) {
      if (fice[q] > fice_lth) {
        T ht_ = 0;
        for (int p = 1; p <= pm; ++p)
          for (int o = 1; o <= om; ++o) ht_ = ht_ + e[opi(o, p, q)] * kdk[oi(o, q)];
        ht_ = 4 * std::sqrt(ht_ * dth);
        T sv = ht_ < H_th ? C1 * ht_ : C2;
        for (int o = 1; o <= om; ++o) sice[oi(o, q)] = 2 * cg0[oi(o, q)] * sv;
      }
    }
  }

  // snl_d12, umwm_source_functions.F90:156-183
  void snl_d12() {
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) snl[opi(o, p, q)] = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= oc[q]; ++o)
          snl[opi(o, p, q)] = bf1_renorm[oi(o, q)] * sds[opi(o + 1, p, q)] * e[opi(o + 1, p, q)] +
                              bf2_renorm[oi(o, q)] * sds[opi(o + 2, p, q)] * e[opi(o + 2, p, q)] -
                              snl_fac * sds[opi(o, p, q)] * e[opi(o, p, q)];
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) sds[opi(o, p, q)] = sds[opi(o, p, q)] * cothkd[oi(o, q)];
      for (int o = 1; o <= om; ++o) sdt[oi(o, q)] = sdt_fac * std::sqrt(rhorat[q]) * ustar[q] * k[oi(o, q)];
    }
  }

  // -------------------------------------------------------------------------
  // source, umwm_physics.F90:9-86
  // -------------------------------------------------------------------------
  void source() {
    T mn = std::numeric_limits<T>::infinity();
#pragma omp parallel for schedule(static) reduction(min : mn)
    for (int q = istart; q <= iend; ++q) {
      T mx = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          T a = 0;
          if (o <= oc[q])
            a = ssin[opi(o, p, q)] - sds[opi(o, p, q)] * snl_arg[oi(o, q)] - sbf[oi(o, q)] - sdt[oi(o, q)] -
                sdv[oi(o, q)] + sice[oi(o, q)];
          ef[opi(o, p, q)] = a;
          mx = std::max(mx, std::abs(a));
        }
      physics_time_step[q] = explim / mx;
      mn = std::min(mn, physics_time_step[q]);
    }
    dts = std::min(std::min(mn, dtamin), dtg - sumt);
    if (!restart && first) dts = 0;
    dta = dts;
    sumt = sumt + dts;
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      for (int p = 1; p <= pm; ++p) {
        for (int o = 1; o <= oc[q]; ++o) {
          size_t a = opi(o, p, q), b = oi(o, q);
          ef[a] = e[a] * std::exp(dts * (ssin[a] - sds[a] - sbf[b] - sdt[b] - sdv[b] + sice[b])) + dts * snl[a];
        }
        for (int o = oc[q] + 1; o <= om; ++o) {
          size_t a = opi(o, p, q), b = oi(o, q);
          ef[a] = 0;
          T num = ssin[a] - sdt[b] - sdv[b] + sice[b];
          if (num >= 0)
            ef[a] = oneoverk4[b] * std::pow(num / (twopisds_fac * f[o - 1] * dummy[a] * cothkd[b]), inv_sds_power);
        }
      }
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          size_t a = opi(o, p, q);
          e[a] = T(0.5) * (e[a] + ef[a]);
        }
    }
  }

  // -------------------------------------------------------------------------
  // propagation, umwm_advection.F90:18-99
  // -------------------------------------------------------------------------
  void propagation() {
    bool anyc = false;
    int lo = isglobal ? 1 : iistart, hi = isglobal ? imm : iiend;
    for (int q = lo; q <= hi; ++q) if (uc[q] != 0 || vc[q] != 0) { anyc = true; break; }
    zerocurrents = !anyc;
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      T feup = 0, fedn = 0, fwup = 0, fwdn = 0, fnup = 0, fndn = 0, fsup = 0, fsdn = 0;
      if (!zerocurrents) {
        T ue = uc[q] + uc[iie[q]], uw_ = uc[q] + uc[iiw[q]], vn = vc[q] + vc[iin[q]], vs_ = vc[q] + vc[iis[q]];
        feup = (ue + std::abs(ue)) * dye[q]; fedn = (ue - std::abs(ue)) * dye[q];
        fwup = (uw_ + std::abs(uw_)) * dyw[q]; fwdn = (uw_ - std::abs(uw_)) * dyw[q];
        fnup = (vn + std::abs(vn)) * dxn[q]; fndn = (vn - std::abs(vn)) * dxn[q];
        fsup = (vs_ + std::abs(vs_)) * dxs[q]; fsdn = (vs_ - std::abs(vs_)) * dxs[q];
      }
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= oc[q]; ++o) {
          T cc = cth_curv[pi_(p, q)], sc = sth_curv[pi_(p, q)];
          T cgi = cg0[oi(o, q)];
          T cge = cgi * cc + cg0[oi(o, ie[q])] * cc;
          T cgw = cgi * cc + cg0[oi(o, iw[q])] * cc;
          T cgs = cgi * sc + cg0[oi(o, is[q])] * sc;
          T cgn = cgi * sc + cg0[oi(o, in[q])] * sc;
          T e0 = e[opi(o, p, q)], ee = e[opi(o, p, ie[q])], ew = e[opi(o, p, iw[q])], en = e[opi(o, p, in[q])],
            es = e[opi(o, p, is[q])];
          T flux = (cge + std::abs(cge)) * dye[q] * e0 + (cge - std::abs(cge)) * dye[q] * ee -
                   (cgw + std::abs(cgw)) * dyw[q] * ew - (cgw - std::abs(cgw)) * dyw[q] * e0 +
                   (cgn + std::abs(cgn)) * dxn[q] * e0 + (cgn - std::abs(cgn)) * dxn[q] * en -
                   (cgs + std::abs(cgs)) * dxs[q] * es - (cgs - std::abs(cgs)) * dxs[q] * e0;
          if (!zerocurrents)
            flux = flux + (feup * e0 + fedn * ee - fwup * ew - fwdn * e0 + fnup * e0 + fndn * en - fsup * es -
                           fsdn * e0);
          size_t a = opi(o, p, q);
          ef[a] = ef[a] - T(0.25) * dta * flux * oneovar[q];
          if (fice[q] > fice_uth) ef[a] = T(0.0);
        }
    }
  }

  // -------------------------------------------------------------------------
  // refraction, umwm_advection.F90:102-180
  // -------------------------------------------------------------------------
  void refraction() {
    bool compute_rotation_tendency = currents || first;
    if (compute_rotation_tendency) {
      std::vector<T> flux((size_t)om * pm * (im + 1), T(0));
      T fmax_ = 0;
      bool init = false;
#pragma omp parallel for schedule(static)
      for (int q = istart; q <= iend; ++q)
        for (int p = 1; p <= pm; ++p)
          for (int o = 1; o <= oc[q]; ++o)
            flux[opi(o, p, q)] =
                T(0.5) * (((cp0[oi(o, ie[q])] - cp0[oi(o, iw[q])]) * sth[p - 1] + vc[iie[q]] - vc[iiw[q]]) * oneovdx[q] -
                          ((cp0[oi(o, in[q])] - cp0[oi(o, is[q])]) * cth[p - 1] + uc[iin[q]] - uc[iis[q]]) * oneovdy[q]);
#pragma omp parallel for schedule(static)
      for (int q = istart; q <= iend; ++q) {
        for (int p = 1; p <= pm; ++p)
          for (int o = 1; o <= om; ++o) { rotl[opi(o, p, q)] = 0; rotr[opi(o, p, q)] = 0; }
        for (int p = 1; p <= pm; ++p)
          for (int o = 1; o <= oc[q]; ++o) {
            rotl[opi(o, p, q)] = T(0.5) * (flux[opi(o, p, q)] + flux[opi(o, pl[p - 1], q)]);
            rotr[opi(o, p, q)] = T(0.5) * (flux[opi(o, p, q)] + flux[opi(o, pr[p - 1], q)]);
          }
      }
      // maxval over the whole (om,pm,istart:iend) array, zeros included
      for (int q = istart; q <= iend; ++q)
        for (int p = 1; p <= pm; ++p)
          for (int o = 1; o <= om; ++o) {
            T v = flux[opi(o, p, q)];
            if (!init || v > fmax_) { fmax_ = v; init = true; }
          }
      if (fmax_ <= std::numeric_limits<T>::min()) dtr_temp = dts;
      else dtr_temp = dth / fmax_;
    }
    dtr = std::min(dtr_temp, dts);
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q)
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= oc[q]; ++o) {
          size_t a = opi(o, p, q);
          T rl = rotl[a], rr = rotr[a];
          T flux = T(0.5) *
                   ((rl + std::abs(rl)) * e[a] + (rl - std::abs(rl)) * e[opi(o, pl[p - 1], q)] -
                    (rr + std::abs(rr)) * e[opi(o, pr[p - 1], q)] - (rr - std::abs(rr)) * e[a]) *
                   oneovdth;
          ef[a] = ef[a] - dtr * flux;
          if (fice[q] > fice_uth) ef[a] = T(0.0);
        }
  }

  // -------------------------------------------------------------------------
  // stress('atm'), umwm_stress.F90:17-264 (atm branch) and helpers :268-344
  // -------------------------------------------------------------------------
  static T stress_tail(T w, T kmax) {
    const T kcap = T(1e3), a = T(0.000112), b = T(-0.01451), c = T(-1.0186);
    T tail = a * (w * w) + b * w + c;
    T kpt = std::pow(kmax, tail);
    return (std::pow(kcap, tail + 1) - kmax * kpt) / (kpt * (tail + 1));
  }
  T friction_velocity_skin(T w) const {
    T z0 = T(1e-3), u = 0;
    for (int n = 1; n <= 6; ++n) {
      u = kappa * w / std::log(z / z0);
      z0 = T(0.132) * nu_air / u;
    }
    return u;
  }

  // stress('ocn'), umwm_stress.F90:34-214: momentum and energy fluxes into
  // the ocean from the current spectrum e and the source terms of the last
  // source() call (ssin, sds after the cothkd factor, snl, sdt).
  void stress_ocn() {
    for (auto* v : {&taux_ocntop, &tauy_ocntop, &taux_ocnbot, &tauy_ocnbot, &taux_snl, &tauy_snl, &epsx_ocn,
                    &epsy_ocn, &epsx_atm, &epsy_atm, &tailocnx, &tailocny, &taux1, &tauy1, &taux2, &tauy2,
                    &taux3, &tauy3})
      v->assign(im + 1, T(0));
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      const T tail = stress_tail(wspd[q], k[oi(om, q)]);
      std::vector<T> ux(om + 1), uy(om + 1);
      auto integrate = [&](T& sx, T& sy) {  // sum(util(:,i) * kdk(:,i)) * rhow * dthg, o in order
        T ax = 0, ay = 0;
        for (int o = 1; o <= om; ++o) {
          ax = ax + ux[o] * kdk[oi(o, q)];
          ay = ay + uy[o] * kdk[oi(o, q)];
        }
        sx = ax * rhow[q] * dthg;
        sy = ay * rhow[q] * dthg;
      };
      auto clear = [&] { std::fill(ux.begin(), ux.end(), T(0)); std::fill(uy.begin(), uy.end(), T(0)); };
      // stress into the ocean top (:39-80)
      clear();
      for (int p = 1; p <= pm; ++p) {
        for (int o = 1; o <= om; ++o) {
          const size_t a = opi(o, p, q), b = oi(o, q);
          ux[o] = ux[o] + e[a] * (sds[a] + sdt[b] + sdv[b]) * cth[p - 1] * invcp0[b];
          uy[o] = uy[o] + e[a] * (sds[a] + sdt[b] + sdv[b]) * sth[p - 1] * invcp0[b];
        }
        for (int o = 3; o <= om; ++o) {
          const size_t a = opi(o, p, q), b = oi(o, q);
          const T w = bf1 * cp0[b] * invcp0[oi(o - 1, q)] + bf2 * cp0[b] * invcp0[oi(o - 2, q)];
          ux[o] = ux[o] - snl[a] * w * cth[p - 1] * invcp0[b];
          uy[o] = uy[o] - snl[a] * w * sth[p - 1] * invcp0[b];
        }
      }
      tailocnx[q] = ux[om] * k[oi(om, q)] * tail * rhow[q] * dthg;
      tailocny[q] = uy[om] * k[oi(om, q)] * tail * rhow[q] * dthg;
      integrate(taux_ocntop[q], tauy_ocntop[q]);
      taux_ocntop[q] = taux_ocntop[q] + tailocnx[q] + taux_skin[q];
      tauy_ocntop[q] = tauy_ocntop[q] + tailocny[q] + tauy_skin[q];
      // stress into the ocean bottom (:95-108)
      clear();
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          const size_t a = opi(o, p, q), b = oi(o, q);
          ux[o] = ux[o] + e[a] * sbf[b] * cth[p - 1] * invcp0[b];
          uy[o] = uy[o] + e[a] * sbf[b] * sth[p - 1] * invcp0[b];
        }
      integrate(taux_ocnbot[q], tauy_ocnbot[q]);
      // momentum lost by the downshifting (:110-128)
      clear();
      for (int p = 1; p <= pm; ++p)
        for (int o = 3; o <= oc[q]; ++o) {
          const size_t a = opi(o, p, q), b = oi(o, q);
          const T w = bf1 * (1 - cp0[b] * invcp0[oi(o - 1, q)]) + bf2 * (1 - cp0[b] * invcp0[oi(o - 2, q)]);
          ux[o] = ux[o] + snl[a] * w * cth[p - 1] * invcp0[b];
          uy[o] = uy[o] + snl[a] * w * sth[p - 1] * invcp0[b];
        }
      integrate(taux_snl[q], tauy_snl[q]);
      // energy flux into the ocean (:130-157)
      clear();
      for (int p = 1; p <= pm; ++p) {
        for (int o = 1; o <= om; ++o) {
          const size_t a = opi(o, p, q);
          ux[o] = ux[o] + e[a] * sds[a] * cth[p - 1];
          uy[o] = uy[o] + e[a] * sds[a] * sth[p - 1];
        }
        for (int o = 3; o <= om; ++o) {
          const size_t a = opi(o, p, q), b = oi(o, q);
          const T w = bf1 * cp0[b] * invcp0[oi(o - 1, q)] + bf2 * cp0[b] * invcp0[oi(o - 2, q)];
          ux[o] = ux[o] - snl[a] * w * cth[p - 1];
          uy[o] = uy[o] - snl[a] * w * sth[p - 1];
        }
      }
      integrate(epsx_ocn[q], epsy_ocn[q]);
      // energy flux from the air (:159-172)
      clear();
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          const size_t a = opi(o, p, q);
          ux[o] = ux[o] + e[a] * ssin[a] * cth[p - 1];
          uy[o] = uy[o] + e[a] * ssin[a] * sth[p - 1];
        }
      integrate(epsx_atm[q], epsy_atm[q]);
      // form drag by wind pushing waves (1), waves against wind (2), waves
      // overrunning wind (3) (:174-212)
      T a1x = 0, a1y = 0, a2x = 0, a2y = 0, a3x = 0, a3y = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          const size_t a = opi(o, p, q), b = oi(o, q);
          const T dd = e[a] * ssin[a] * invcp0[b] * kdk[b];
          dummy[a] = dd;
          if (ssin[a] > 0) {
            a1x = a1x + dd * cth[p - 1];
            a1y = a1y + dd * sth[p - 1];
          } else if (std::cos(wdir[q] - th[p - 1]) < 0) {
            a2x = a2x + dd * cth[p - 1];
            a2y = a2y + dd * sth[p - 1];
          } else {
            a3x = a3x + dd * cth[p - 1];
            a3y = a3y + dd * sth[p - 1];
          }
        }
      taux1[q] = a1x * rhow[q] * dthg; tauy1[q] = a1y * rhow[q] * dthg;
      taux2[q] = a2x * rhow[q] * dthg; tauy2[q] = a2y * rhow[q] * dthg;
      taux3[q] = a3x * rhow[q] * dthg; tauy3[q] = a3y * rhow[q] * dthg;
    }
  }

  void stress_atm() {
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      T tail = stress_tail(wspd[q], k[oi(om, q)]);
      std::vector<T> tx(om + 1, T(0)), ty(om + 1, T(0));
      // stress_vector_integral receives cp0(om, 0:im) through an assumed-shape
      // dummy cp(:,:) whose lower bound is 1, so cp(o,i) there is cp0(o,i-1):
      // the form stress at wet point i divides by the phase speed of point i-1
      // (the ghost column for i=1).  umwm_stress.F90:401, :495-513.
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          size_t a = opi(o, p, q);
          tx[o] = tx[o] + e[a] * ssin[a] * cth[p - 1] / cp0[oi(o, q - 1)];
          ty[o] = ty[o] + e[a] * ssin[a] * sth[p - 1] / cp0[oi(o, q - 1)];
        }
      tailatmx[q] = tx[om] * k[oi(om, q)] * tail * rhow[q] * dthg;
      tailatmy[q] = ty[om] * k[oi(om, q)] * tail * rhow[q] * dthg;
      T sx = 0, sy = 0;
      for (int o = 1; o <= om; ++o) { sx = sx + tx[o] * kdk[oi(o, q)]; sy = sy + ty[o] * kdk[oi(o, q)]; }
      taux_form[q] = sx * rhow[q] * dthg + tailatmx[q];
      tauy_form[q] = sy * rhow[q] * dthg + tailatmy[q];
      T dx_ = 0, dy_ = 0;
      for (int o = oc[q]; o <= om; ++o) { dx_ = dx_ + tx[o] * kdk[oi(o, q)]; dy_ = dy_ + ty[o] * kdk[oi(o, q)]; }
      taux_diag[q] = dx_ * rhow[q] * dthg;
      tauy_diag[q] = dy_ * rhow[q] * dthg;
      // wind relative to surface velocity (currents + surface Stokes drift)
      T usv = uc[q] + (lm >= 1 ? us[il(q, 1)] : T(0));
      T vsv = vc[q] + (lm >= 1 ? vs[il(q, 1)] : T(0));
      T urel = wspd[q] * std::cos(wdir[q]) - usv;
      T vrel = wspd[q] * std::sin(wdir[q]) - vsv;
      T wspdrel = std::sqrt(urel * urel + vrel * vrel);
      T wdirrel = std::atan2(vrel, urel);
      T cd_form = std::sqrt(taux_form[q] * taux_form[q] + tauy_form[q] * tauy_form[q]) / (rhoa[q] * (wspd[q] * wspd[q]));
      T us_ = friction_velocity_skin(wspdrel);
      T cds = (us_ * us_) / (wspd[q] * wspd[q]);
      cds = cds * (1 + 2 * cds / (cds + cd_form + std::numeric_limits<T>::min())) / 3;
      if (cds > T(1e-2)) cds = T(1e-2);
      taux_skin[q] = rhoa[q] * cds * (wspdrel * wspdrel) * std::cos(wdirrel);
      tauy_skin[q] = rhoa[q] * cds * (wspdrel * wspdrel) * std::sin(wdirrel);
      taux[q] = taux_form[q] + taux_skin[q];
      tauy[q] = tauy_form[q] + tauy_skin[q];
      cd[q] = std::sqrt(taux[q] * taux[q] + tauy[q] * tauy[q]) / (rhoa[q] * (wspd[q] * wspd[q]));
      ustar[q] = std::sqrt(std::sqrt(taux[q] * taux[q] + tauy[q] * tauy[q]) / rhoa[q]);
    }
  }

  // -------------------------------------------------------------------------
  // diag, umwm_physics.F90:89-205
  // -------------------------------------------------------------------------
  void diag() {
    const T tiny_ = std::numeric_limits<T>::min();
#pragma omp parallel for schedule(static)
    for (int q = istart; q <= iend; ++q) {
      T m0 = 0, m2 = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          m0 = m0 + e[opi(o, p, q)] * kdk[oi(o, q)];
          m2 = m2 + (f[o - 1] * f[o - 1]) * e[opi(o, p, q)] * kdk[oi(o, q)];
        }
      mwp[q] = std::sqrt(m0 / (m2 + tiny_));
      T mx = 0, my = 0, cxx = 0, cxy = 0, cyy = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= oc[q]; ++o) {
          T ek = e[opi(o, p, q)] * kdk[oi(o, q)] * invcp0[oi(o, q)];
          mx = mx + ek * cth[p - 1];
          my = my + ek * sth[p - 1];
          cxx = cxx + cg0[oi(o, q)] * ek * (cth[p - 1] * cth[p - 1]);
          cxy = cxy + cg0[oi(o, q)] * ek * cth[p - 1] * sth[p - 1];
          cyy = cyy + cg0[oi(o, q)] * ek * (sth[p - 1] * sth[p - 1]);
        }
      momx[q] = mx * rhow[q] * dthg; momy[q] = my * rhow[q] * dthg;
      cgmxx[q] = cxx * rhow[q] * dthg; cgmxy[q] = cxy * rhow[q] * dthg; cgmyy[q] = cyy * rhow[q] * dthg;
      T h = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) h = h + e[opi(o, p, q)] * kdk[oi(o, q)];
      ht[q] = 4 * std::sqrt(h * dth);
      T xc = 0, yc = 0;
      for (int p = 1; p <= pm; ++p) {
        T mag = 0;
        for (int o = 1; o <= om; ++o) mag = mag + e[opi(o, p, q)] * kdk[oi(o, q)];
        xc = xc + mag * cth[p - 1];
        yc = yc + mag * sth[p - 1];
      }
      mwd[q] = std::atan2(yc, xc);
      m0 = 0; m2 = 0;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          m0 = m0 + e[opi(o, p, q)] * kdk[oi(o, q)];
          m2 = m2 + e[opi(o, p, q)] * k3dk[oi(o, q)];
        }
      mss[q] = m2 * dth;
      mwl[q] = twopi * std::sqrt(m0 / (m2 + tiny_));
      int opeak = 1, ppeak = 1;
      T best = 0;
      bool have = false;
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o) {
          T v = e[opi(o, p, q)] * kdk[oi(o, q)];
          if (!have || v > best) { best = v; opeak = o; ppeak = p; have = true; }
        }
      dwd[q] = th[ppeak - 1];
      dwl[q] = twopi / k[oi(opeak, q)];
      dwp[q] = T(1.) / f[opeak - 1];
      dcp0[q] = cp0[oi(opeak, q)];
      dcg0[q] = cg0[oi(opeak, q)];
      dcp[q] = dcp0[q] + uc[q] * cth[ppeak - 1] + vc[q] * sth[ppeak - 1];
      dcg[q] = dcg0[q] + uc[q] * cth[ppeak - 1] + vc[q] * sth[ppeak - 1];
    }
  }

  // screen line values, umwm_util.F90:69-124
  T sigwaveheight(int q) const {
    T s = 0;
    for (int p = 1; p <= pm; ++p)
      for (int o = 1; o <= om; ++o) s = s + e[opi(o, p, q)] * kdk[oi(o, q)];
    return T(4.) * std::sqrt(s * dth);
  }
  T meanwaveperiod(int q) const {
    T m0 = 0, m2 = 0;
    for (int p = 1; p <= pm; ++p)
      for (int o = 1; o <= om; ++o) {
        m0 = m0 + e[opi(o, p, q)] * kdk[oi(o, q)];
        m2 = m2 + (f[o - 1] * f[o - 1]) * e[opi(o, p, q)] * kdk[oi(o, q)];
      }
    return std::sqrt(m0 / m2);
  }

  // -------------------------------------------------------------------------
  // umwm_initialize, umwm_top.F90:7-29
  // -------------------------------------------------------------------------
  bool initialize() {
    if (!nmlread()) return false;
    alloc1();
    if (!grid()) return false;
    masks();
    partition();
    alloc2();
    remap();
    if (!input_nc(starttimestr)) return false;
    init();
    stokes_init();
    stokes_drift();
    return true;
  }

  // restart_read, umwm_restart.F90:19-56
  bool restart_read(const std::string& timestr) {
    std::string key = timestr;
    if (key.size() >= 11) key[10] = '_';
    auto it = restarts.find(key);
    if (it == restarts.end()) return fail("restart_read: no restart for " + key);
    const auto& F = it->second.first;
    const auto& U = it->second.second;
    for (int q = 1; q <= im; ++q) {
      for (int p = 1; p <= pm; ++p)
        for (int o = 1; o <= om; ++o)
          e[opi(o, p, q)] = (T)F[((size_t)(q - 1) * pm + (p - 1)) * om + (o - 1)];
      ustar[q] = (T)U[q - 1];
    }
    return true;
  }

  // -------------------------------------------------------------------------
  // umwm_run, umwm_top.F90:32-196
  // -------------------------------------------------------------------------
  bool run(const std::string& start, const std::string& stop) {
    int64_t t0, t1;
    if (!parse_time(start, t0) || !parse_time(stop, t1)) return fail("run: bad time string");
    int64_t now = t0;
    if (first && restart) if (!restart_read(start)) return false;
    while (now < t1) {
      now += nint_d((double)dtg);
      std::string cur = format_time(now, '_');
      if (!forcinginput(cur)) return false;
      sumt = 0;
      while (sumt < dtg) {
        if (max_substeps >= 0 && substeps >= max_substeps) { stopped = true; return true; }
        forcinginterpolate();
        sin_d12(); sds_d12(); snl_d12(); s_ice(); source();
        propagation();
        refraction();
        // e = ef (umwm_top.F90:113), with negatives cut to 0 as the GPU path
        // does: the explicit Snl term can leave a tiny negative ef, after
        // which (e k^4)^sds_power is NaN (seen in fp64 on the hurricane case)
        // cut_count: the bins this cut changed since initialize
        for (int q = istart; q <= iend; ++q)
          for (int p = 1; p <= pm; ++p)
            for (int o = 1; o <= om; ++o) {
              const T v = ef[opi(o, p, q)];
              if (v < T(0)) ++cut_count;
              e[opi(o, p, q)] = v < T(0) ? T(0) : v;
            }
        stress_atm();
        if (first) { diag(); first = false; }
        substeps++;
        if (iip >= 1 && iip <= im) {
          double rec[8] = {(double)(sumt / dtg), (double)dts, (double)wspd[iip], (double)wdir[iip],
                           (double)sigwaveheight(iip), (double)meanwaveperiod(iip), (double)(cd[iip] * T(1e3)),
                           (double)f[oc[iip] - 1]};
          screen.insert(screen.end(), rec, rec + 8);
          if (verbose)
            std::printf("  %4.2f  %8.3f %9.6f %9.6f %9.6f %9.6f %9.6f %9.6f\n", rec[0], rec[1], rec[2], rec[3], rec[4],
                        rec[5], rec[6], rec[7]);
        }
      }
      if (firstdtg) firstdtg = false;
      if (stokes) stokes_drift();
      diag();
      stress_ocn();  // every outer step (the reference calls it before gridded output)
    }
    return true;
  }
};

struct Handle {
  int prec;
  Model<float>* f32 = nullptr;
  Model<double>* f64 = nullptr;
  std::string err;
};

template <typename M>
bool get_field(M& m, const std::string& name, double* out, long n) {
  using T = typename std::remove_reference<decltype(m.dts)>::type;
  auto copy_wet = [&](const std::vector<T>& v) {  // (1..im); zeros before the array is first computed
    if (n < m.im) return false;
    for (int q = 1; q <= m.im; ++q) out[q - 1] = q < (int)v.size() ? (double)v[q] : 0.0;
    return true;
  };
  auto copy_imm = [&](const std::vector<T>& v) {
    if (n < m.imm) return false;
    for (int q = 1; q <= m.imm; ++q) out[q - 1] = (double)v[q];
    return true;
  };
  auto copy_wet_i = [&](const std::vector<int>& v, int lo, int hi) {
    if (n < hi - lo + 1) return false;
    for (int q = lo; q <= hi; ++q) out[q - lo] = (double)v[q];
    return true;
  };
  auto copy_2d_i = [&](const std::vector<int>& v) {
    if (n < (long)v.size()) return false;
    for (size_t q = 0; q < v.size(); ++q) out[q] = (double)v[q];
    return true;
  };
  auto copy_2d = [&](const std::vector<T>& v) {
    if (n < (long)v.size()) return false;
    for (size_t q = 0; q < v.size(); ++q) out[q] = (double)v[q];
    return true;
  };
  auto copy_oi = [&](const std::vector<T>& v, bool ghost) {  // (om, 0..im) or (om, 1..im)
    int lo = ghost ? 0 : 1;
    long need = (long)m.om * (m.im - lo + 1);
    if (n < need) return false;
    for (int q = lo; q <= m.im; ++q)
      for (int o = 1; o <= m.om; ++o) out[(size_t)(q - lo) * m.om + (o - 1)] = (double)v[m.oi(o, q)];
    return true;
  };
  auto copy_opi = [&](const std::vector<T>& v) {
    long need = (long)m.om * m.pm * m.im;
    if (n < need) return false;
    for (int q = 1; q <= m.im; ++q)
      for (int p = 1; p <= m.pm; ++p)
        for (int o = 1; o <= m.om; ++o)
          out[((size_t)(q - 1) * m.pm + (p - 1)) * m.om + (o - 1)] = (double)v[m.opi(o, p, q)];
    return true;
  };
  auto copy_il = [&](const std::vector<T>& v) {  // (im, lm)
    long need = (long)m.im * m.lm;
    if (n < need) return false;
    for (int l = 1; l <= m.lm; ++l)
      for (int q = 1; q <= m.im; ++q) out[(size_t)(l - 1) * m.im + (q - 1)] = (double)v[m.il(q, l)];
    return true;
  };
  // scalars
  std::map<std::string, double> sc = {
      {"dts", (double)m.dts}, {"dta", (double)m.dta}, {"dtr", (double)m.dtr}, {"dtamin", (double)m.dtamin},
      {"sumt", (double)m.sumt}, {"cgmax", (double)m.cgmax}, {"cfllim", (double)m.cfllim},
      {"mindelx", (double)m.mindelx}, {"dth", (double)m.dth}, {"dlnf", (double)m.dlnf}, {"bf1", (double)m.bf1},
      {"bf2", (double)m.bf2}, {"im", (double)m.im}, {"imm", (double)m.imm}, {"lm", (double)m.lm},
      {"iip", (double)m.iip}, {"substeps", (double)m.substeps}, {"dtr_temp", (double)m.dtr_temp},
      {"first", (double)m.first}, {"om", (double)m.om}, {"pm", (double)m.pm}, {"mm", (double)m.mm},
      {"nm", (double)m.nm}, {"zerocurrents", (double)m.zerocurrents}, {"cut_count", (double)m.cut_count}};
  if (sc.count(name)) { if (n < 1) return false; out[0] = sc[name]; return true; }
  if (name == "screen") {
    if (n < (long)m.screen.size()) return false;
    for (size_t q = 0; q < m.screen.size(); ++q) out[q] = m.screen[q];
    return true;
  }
  if (name == "f") { for (int o = 0; o < m.om && o < n; ++o) out[o] = (double)m.f[o]; return n >= m.om; }
  if (name == "th") { for (int p = 0; p < m.pm && p < n; ++p) out[p] = (double)m.th[p]; return n >= m.pm; }
  if (name == "depth") { for (int l = 0; l < m.lm && l < n; ++l) out[l] = (double)m.depth[l]; return n >= m.lm; }
  if (name == "ii") return copy_2d_i(m.ii);
  if (name == "mask") return copy_2d_i(m.mask);
  if (name == "d_2d") return copy_2d(m.d_2d);
  if (name == "dx_2d") return copy_2d(m.dx_2d);
  if (name == "dy_2d") return copy_2d(m.dy_2d);
  if (name == "curv") return copy_2d(m.curv);
  if (name == "mi") return copy_wet_i(m.mi, 1, m.imm);
  if (name == "ni") return copy_wet_i(m.ni, 1, m.imm);
  if (name == "iw") return copy_wet_i(m.iw, 1, m.imm);
  if (name == "ie") return copy_wet_i(m.ie, 1, m.imm);
  if (name == "is") return copy_wet_i(m.is, 1, m.imm);
  if (name == "in") return copy_wet_i(m.in, 1, m.imm);
  if (name == "iiw") return copy_wet_i(m.iiw, 1, m.imm);
  if (name == "iie") return copy_wet_i(m.iie, 1, m.imm);
  if (name == "iis") return copy_wet_i(m.iis, 1, m.imm);
  if (name == "iin") return copy_wet_i(m.iin, 1, m.imm);
  if (name == "oc") return copy_wet_i(m.oc, 1, m.im);
  if (name == "d") return copy_imm(m.d);
  if (name == "dx") return copy_imm(m.dx);
  if (name == "dy") return copy_imm(m.dy);
  if (name == "wspd") return copy_imm(m.wspd);
  if (name == "wdir") return copy_imm(m.wdir);
  if (name == "uc") return copy_imm(m.uc);
  if (name == "vc") return copy_imm(m.vc);
  if (name == "rhoa") return copy_imm(m.rhoa);
  if (name == "rhow") return copy_imm(m.rhow);
  if (name == "rhorat") return copy_imm(m.rhorat);
  if (name == "fice") return copy_imm(m.fice);
  std::map<std::string, const std::vector<T>*> wet = {
      {"ar", &m.ar}, {"cd", &m.cd}, {"dxn", &m.dxn}, {"dxs", &m.dxs}, {"dye", &m.dye}, {"dyw", &m.dyw},
      {"fcutoff", &m.fcutoff}, {"oneovar", &m.oneovar}, {"oneovdx", &m.oneovdx}, {"oneovdy", &m.oneovdy},
      {"shelt", &m.shelt}, {"physics_time_step", &m.physics_time_step}, {"ustar", &m.ustar}, {"taux", &m.taux},
      {"tauy", &m.tauy}, {"taux_form", &m.taux_form}, {"tauy_form", &m.tauy_form}, {"taux_skin", &m.taux_skin}, {"taux_ocntop", &m.taux_ocntop},
      {"tauy_ocntop", &m.tauy_ocntop}, {"taux_ocnbot", &m.taux_ocnbot}, {"tauy_ocnbot", &m.tauy_ocnbot},
      {"taux_snl", &m.taux_snl}, {"tauy_snl", &m.tauy_snl}, {"epsx_ocn", &m.epsx_ocn}, {"epsy_ocn", &m.epsy_ocn},
      {"epsx_atm", &m.epsx_atm}, {"epsy_atm", &m.epsy_atm}, {"tailocnx", &m.tailocnx}, {"tailocny", &m.tailocny},
      {"taux1", &m.taux1}, {"tauy1", &m.tauy1}, {"taux2", &m.taux2}, {"tauy2", &m.tauy2}, {"taux3", &m.taux3},
      {"tauy3", &m.tauy3},
      {"tauy_skin", &m.tauy_skin}, {"taux_diag", &m.taux_diag}, {"tauy_diag", &m.tauy_diag},
      {"tailatmx", &m.tailatmx}, {"tailatmy", &m.tailatmy}, {"ht", &m.ht}, {"mss", &m.mss}, {"mwd", &m.mwd},
      {"mwl", &m.mwl}, {"mwp", &m.mwp}, {"dwd", &m.dwd}, {"dwl", &m.dwl}, {"dwp", &m.dwp}, {"dcp0", &m.dcp0},
      {"dcp", &m.dcp}, {"dcg0", &m.dcg0}, {"dcg", &m.dcg}, {"momx", &m.momx}, {"momy", &m.momy},
      {"cgmxx", &m.cgmxx}, {"cgmxy", &m.cgmxy}, {"cgmyy", &m.cgmyy}, {"ds", &m.ds}};
  if (wet.count(name)) return copy_wet(*wet[name]);
  if (name == "cp0") return copy_oi(m.cp0, true);
  if (name == "cg0") return copy_oi(m.cg0, true);
  std::map<std::string, const std::vector<T>*> oit = {
      {"k", &m.k}, {"bf1_renorm", &m.bf1_renorm}, {"bf2_renorm", &m.bf2_renorm}, {"cothkd", &m.cothkd},
      {"dwn", &m.dwn}, {"fkovg", &m.fkovg}, {"invcp0", &m.invcp0}, {"k4", &m.k4}, {"kdk", &m.kdk},
      {"k3dk", &m.k3dk}, {"oneoverk4", &m.oneoverk4}, {"sbf", &m.sbf}, {"sdt", &m.sdt}, {"sdv", &m.sdv},
      {"snl_arg", &m.snl_arg}, {"l2", &m.l2}, {"logl2overz", &m.logl2overz}, {"sice", &m.sice}};
  if (oit.count(name)) return copy_oi(*oit[name], false);
  std::map<std::string, const std::vector<T>*> opit = {
      {"e", &m.e}, {"ef", &m.ef}, {"dummy", &m.dummy}, {"rotl", &m.rotl}, {"rotr", &m.rotr},
      {"sds", &m.sds}, {"snl", &m.snl}, {"ssin", &m.ssin}};
  if (opit.count(name)) return copy_opi(*opit[name]);
  if (name == "us") return copy_il(m.us);
  if (name == "vs") return copy_il(m.vs);
  return false;
}

}  // namespace

// ---------------------------------------------------------------------------
// Denormal handling.  The reference's production flags (-Ofast, Makefile:5)
// run it with flush-to-zero / denormals-are-zero, and most of a young
// spectrum sits at tiny(e) where denormal arithmetic would otherwise be
// ~30x slower.  The oracle runs with the same FTZ/DAZ mode (set through
// glibc's fenv_t, on x86-64 MXCSR FTZ|DAZ, on aarch64 FPCR.FZ), on every
// OpenMP worker, and restores the caller's environment on return.
// ---------------------------------------------------------------------------
static void set_ftz_this_thread() {
  fenv_t env;
  fegetenv(&env);
#if defined(__x86_64__)
  env.__mxcsr |= 0x8040u;
#elif defined(__aarch64__)
  env.__fpcr |= (1u << 24);
#endif
  fesetenv(&env);
}

struct FtzScope {
  fenv_t saved;
  FtzScope() {
    fegetenv(&saved);
    set_ftz_this_thread();
#ifdef _OPENMP
#pragma omp parallel
    set_ftz_this_thread();
#endif
  }
  ~FtzScope() { fesetenv(&saved); }
};

// ---------------------------------------------------------------------------
// C API used by the tests' ctypes wrapper (oracle/pyoracle.py)
// ---------------------------------------------------------------------------
extern "C" {

void* oracle_new(int prec, const char* nml_text) {
  Handle* h = new Handle();
  h->prec = prec;
  if (prec == 64) { h->f64 = new Model<double>(); h->f64->nml_text = nml_text; }
  else { h->f32 = new Model<float>(); h->f32->nml_text = nml_text; }
  return h;
}

void oracle_free(void* hp) {
  Handle* h = (Handle*)hp;
  delete h->f32;
  delete h->f64;
  delete h;
}

const char* oracle_error(void* hp) {
  Handle* h = (Handle*)hp;
  h->err = h->prec == 64 ? h->f64->error : h->f32->error;
  return h->err.c_str();
}

int oracle_put_gridtopo(void* hp, const char* var, const float* data, long n) {
  Handle* h = (Handle*)hp;
  std::vector<float> v(data, data + n);
  if (h->prec == 64) h->f64->gridtopo[var] = v; else h->f32->gridtopo[var] = v;
  return 0;
}

int oracle_put_exclude(void* hp, const int* mn, int npairs) {
  Handle* h = (Handle*)hp;
  std::vector<std::pair<int, int>> v;
  for (int q = 0; q < npairs; ++q) v.push_back({mn[2 * q], mn[2 * q + 1]});
  if (h->prec == 64) h->f64->exclude = v; else h->f32->exclude = v;
  return 0;
}

int oracle_put_forcing(void* hp, const char* time19, const char* var, const float* data, long n) {
  Handle* h = (Handle*)hp;
  std::string key(time19);
  if (key.size() >= 11) key[10] = '_';
  std::vector<float> v(data, data + n);
  if (h->prec == 64) h->f64->forcing[key][var] = v; else h->f32->forcing[key][var] = v;
  return 0;
}

int oracle_put_restart(void* hp, const char* time19, const float* e, long ne, const float* ust, long nu) {
  Handle* h = (Handle*)hp;
  std::string key(time19);
  if (key.size() >= 11) key[10] = '_';
  auto val = std::make_pair(std::vector<float>(e, e + ne), std::vector<float>(ust, ust + nu));
  if (h->prec == 64) h->f64->restarts[key] = val; else h->f32->restarts[key] = val;
  return 0;
}

int oracle_set_option(void* hp, const char* name, double value) {
  Handle* h = (Handle*)hp;
  std::string n(name);
  auto apply = [&](auto& m) {
    if (n == "max_substeps") { m.max_substeps = (long long)value; m.stopped = false; return 0; }
    if (n == "verbose") { m.verbose = value != 0; return 0; }
    if (n == "gust_seed") { m.gust_seed = (unsigned)value; return 0; }
    return -1;
  };
  return h->prec == 64 ? apply(*h->f64) : apply(*h->f32);
}

int oracle_initialize(void* hp) {
  FtzScope ftz;
  Handle* h = (Handle*)hp;
  bool ok = h->prec == 64 ? h->f64->initialize() : h->f32->initialize();
  return ok ? 0 : 1;
}

int oracle_run(void* hp, const char* start, const char* stop) {
  FtzScope ftz;
  Handle* h = (Handle*)hp;
  bool ok = h->prec == 64 ? h->f64->run(start, stop) : h->f32->run(start, stop);
  return ok ? 0 : 1;
}

int oracle_get(void* hp, const char* name, double* out, long n) {
  Handle* h = (Handle*)hp;
  bool ok = h->prec == 64 ? get_field(*h->f64, name, out, n) : get_field(*h->f32, name, out, n);
  return ok ? 0 : 1;
}

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
