// Host-side model set-up of the GB300 UMWM library: namelist, grid, masks,
// partition, wet-point unrolling and the spectral tables, computed once on
// the host in fp32 and uploaded to the GPU.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace umwm {

// Namelist groups and their raw (string) values, keys lower-cased.
struct NmlGroups {
  std::map<std::string, std::map<std::string, std::vector<std::string>>> g;
};
bool parse_nml(const std::string& text, NmlGroups& out, std::string& err);

// 'YYYY-MM-DD hh:mm:ss' (any separator between date and time) <-> seconds
bool time_from_string(const std::string& s, int64_t& t);
std::string time_to_string(int64_t t, char sep);

struct Inputs {  // stand-ins for the files the reference opens
  std::map<std::string, std::vector<float>> gridtopo;                       // lon, lat, z
  std::vector<std::pair<int, int>> exclude;                                  // lake seeds
  std::map<std::string, std::map<std::string, std::vector<float>>> forcing;  // time -> var -> (mm,nm)
  std::map<std::string, std::pair<std::vector<float>, std::vector<float>>> restarts;
};

std::string time_key(const char* time19);  // 'YYYY-MM-DD_hh:mm:ss'

struct HostModel {
  // namelist values (umwm_init.F90:67-81, umwm_stokes.F90:25)
  bool isglobal = false, restart = false, gridfromfile = false, topofromfile = false, fillestuaries = false,
       filllakes = false, winds = false, currents = false, air_density = false, water_density = false,
       seaice = false, stokes = false;
  int mm = 0, nm = 0, om = 0, pm = 0, outgrid = 0, outspec = 0, outrst = 0, xpl = 0, ypl = 0;
  float fmin = 0, fmax = 0, fprog = 0, dtg = 0, g = 0, nu_air = 0, nu_water = 0, sfct = 0, kappa = 0, z = 0,
        gustiness = 0, dmin = 0, explim = 0, sin_fac = 0, sin_diss1 = 0, sin_diss2 = 0, sds_fac = 0,
        sds_power = 0, mss_fac = 0, snl_fac = 0, sdt_fac = 0, sbf_fac = 0, sbp_fac = 0, delx = 0, dely = 0,
        dpt = 0, wspd0 = 0, wdir0 = 0, uc0 = 0, vc0 = 0, rhoa0 = 0, rhow0 = 0, fice0 = 0, fice_lth = 0,
        fice_uth = 0;
  std::string starttimestr, stoptimestr;
  std::vector<float> depths_nml;  // &STOKES depths (100, default -1)

  // derived scalars (umwm_init.F90:1254-1340)
  float pi = 0, twopi = 0, dlnf = 0, dth = 0, dthg = 0, oneovdth = 0, twopisds_fac = 0, fieldscale1 = 0,
        fieldscale2 = 0, inv_sds_power = 0, cfllim = 0, bf1 = 0, bf2 = 0, mindelx = 0, cgmax = 0, dtamin = 0,
        eulerinv = 0;
  int im = 0, imm = 0, lm = 0, iip = 0;
  bool curvilinear = false;

  // 2-d (mm,nm) Fortran order
  std::vector<int> mask, ii;
  std::vector<float> d_2d, dx_2d, dy_2d, curv, lon, lat;
  // over imm, index 1..imm (entry 0 unused)
  std::vector<int> mi, ni, is, in, iw, ie, iis, iin, iiw, iie;
  std::vector<float> d, dx, dy;
  // over wet points, index 1..im
  std::vector<float> ar, oneovar, oneovdx, oneovdy, dxn, dxs, dye, dyw, curv_i;
  // spectral constants
  std::vector<float> f, th, cth, sth, dom, depth;
  // (om, i): index (i)*om + (o-1); cp0/cg0 carry the ghost point i=0
  std::vector<float> k, cp0, cg0, dwn, kdk, k3dk, k4, fkovg, cothkd, sbf, sdv, bf1r, bf2r, logl2overz;
  // initial state from init (umwm_init.F90:1350-1365) and input_nc
  std::vector<float> wspd_init, ustar_init;

  std::string err;
  inline size_t i2(int m, int n) const { return (size_t)(m - 1) + (size_t)(n - 1) * mm; }
  inline size_t oi(int o, int i) const { return (size_t)i * om + (o - 1); }

  bool read_namelist(const std::string& text);
  bool build(const Inputs& in);  // grid .. dispersion; returns false with err set
};

}  // namespace umwm
