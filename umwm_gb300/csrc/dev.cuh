// Device-side definitions shared by the GB300 UMWM kernels.
//
// HBM layout.  N wet points plus a ghost point at index N (the reference's
// aliased land neighbour iistart-1), grouped in NB = ceil((N+1)/32) blocks
// of 32 consecutive wet points (ldN = 32 NB):
//   spectrum arrays E, ES (= E* after the source half-step), EF:
//       [o][j/32][p][32]: one frequency of one 32-point block is a
//       contiguous P*128-byte region; within it direction p is a 128-byte
//       line of 32 consecutive points, so a warp reading one bin for 16 or
//       32 points is one coalesced access and every direction offset is a
//       compile-time immediate
//   per-(o,i) tables TAB: [o][j/32][table][32], tables T_* below
//   per-point arrays: [ldN]; all-point (land included) arrays: [imm]
#pragma once
#include <cstdint>

namespace umwm {

constexpr int MAX_OM = 64;
constexpr int MAX_PM = 72;
constexpr int MAX_LM = 100;

// per-(o,i) table rows (stored per frequency o, then table, then point)
enum TableRow {
  T_K = 0,      // wavenumber k                       umwm_init.F90:1473
  T_CP0,        // phase speed cp0 (ghost = min)      :1493, :1653-1656
  T_CG0,        // group velocity cg0 (ghost = min)   :1494, :1653-1656
  T_LOGL2Z,     // log(l2/z), capped                  :1530-1533
  T_FKOVG,      // f k / g                            :1507
  T_K4,         // k^4                                :1503
  T_K3DK,       // k^3 dk                             :1506
  T_KDK,        // k dk                               :1505
  T_COTHKD,     // coth(0.2 kd)                       :1508
  T_SBF,        // bottom friction+percolation        :1510-1511
  T_SDV,        // viscous dissipation                :1512
  T_BF1R,       // Snl weight to o+1                  :1523
  T_BF2R,       // Snl weight to o+2                  :1524
  T_COUNT
};

struct Params {
  int N, ldN, NB, O, P, NM, mm, nm, lm;
  int iip;  // 0-based wet index of the screen point, -1 if none
  float g, explim, sin_fac, fieldscale1, fieldscale2, twopisds_fac, sds_power, inv_sds_power, mss_fac, snl_fac,
      sdt_fac, z, nu_air, kappa, fprog, dth, dthg, oneovdth, dtamin, dtg, fice_lth, fice_uth, eulerinv, rhow0;
  int winds, currents, air_density, water_density, seaice, restart, curvilinear, isglobal;
  int ice_possible;  // fice can exceed fice_lth somewhere
  float f[MAX_OM], dom[MAX_OM];
  float th[MAX_PM], cth[MAX_PM], sth[MAX_PM], c2th[MAX_PM], s2th[MAX_PM];
  float depth[MAX_LM];
};

// Device-resident control block of the inner (dynamic-dts) loop.
struct Ctl {
  float sumt, dts, dta, dtr, dtr_temp;
  unsigned minphys_enc;   // ordered encoding of min_i(explim/max|arg|)
  unsigned maxrot_enc;    // ordered encoding of max rotation flux
  int anycurrent;         // set by the forcing kernel when a wet current is non-zero
  int zerocurrents;       // latched for propagation of this substep
  int first;              // reference's 'first' (first substep of the first run)
  int compute_rot;        // rotation recomputed this substep
  int done;               // sumt >= dtg after this substep
  int substep;            // substeps since initialize
  int err;                // error flags (bit 0: timeout)
  int log_count;
};

struct Ptrs {
  float *E, *ES, *EF;  // spectrum arrays [O][P][ldN]
  const float* TAB;     // [O][T_COUNT][ldN]
  // wet-point arrays [ldN]
  const int *ie, *iw, *in, *is;      // aliased neighbours (N = ghost)
  const int *iie, *iiw, *iin, *iis;  // true neighbours, 0-based over imm
  const float *oneovar, *oneovdx, *oneovdy, *dxn, *dxs, *dye, *dyw, *d, *curv;
  int* oc;
  int* oc_rot;      // oc at the last rotation computation
  float* ustar;
  float* cd;
  float *taux, *tauy, *taux_form, *tauy_form, *taux_skin, *tauy_skin, *taux_diag, *tauy_diag, *tailatmx,
      *tailatmy;
  float* shelt;
  float* fcutoff;
  float* phys;      // physics_time_step
  float* sice_v;    // per-point sea-ice attenuation factor (0 when no ice)
  // all-point arrays [NM] (0-based unrolled index, land included)
  float *wspd, *wdir, *uc, *vc, *rhoa, *rhow, *rhorat, *fice;
  const int *mi, *ni;  // 1-based (m, n) of each unrolled index
  // forcing levels (mm*nm, Fortran order): b = n, f = n+1
  const float *uwb, *uwf, *vwb, *vwf, *ucb, *ucf, *vcb, *vcf, *rhoab, *rhoaf, *rhowb, *rhowf, *ficeb, *ficef;
  // Stokes drift [lm][ldN] and e-folding depth
  float *us, *vs, *ds;
  // diagnostics [ldN]
  float *ht, *mwp, *mwd, *mss, *mwl, *dwd, *dwl, *dwp, *dcp0, *dcp, *dcg0, *dcg, *momx, *momy, *cgmxx, *cgmxy,
      *cgmyy;
  Ctl* ctl;
  double* log;  // screen lines, 8 per substep
  int log_cap;
};

// element offsets in the blocked layouts
__host__ __device__ inline size_t sidx(const Params& prm, int o, int p, int j) {
  return ((size_t)(o * prm.NB + (j >> 5)) * prm.P + p) * 32 + (j & 31);
}
__host__ __device__ inline size_t tidx(const Params& prm, int o, int t, int j) {
  return ((size_t)(o * prm.NB + (j >> 5)) * T_COUNT + t) * 32 + (j & 31);
}

}  // namespace umwm
