// Device-side definitions shared by the GB300 UMWM kernels.
//
// One model is an ensemble of members (a single domain is a one-member
// ensemble).  Member m owns the wet indices [off, off + N) of a common index
// space, then its own ghost point at off + N (the reference's aliased land
// neighbour iistart-1), padded to a multiple of 64 points so that every CTA
// tile belongs to one member.  The index space is grouped in NB blocks of 32
// consecutive points (ldN = 32 NB):
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

// per-(o,i) table rows (stored per frequency o, then table, then point);
// the rows the propagation reads come first (T_ADV_ROWS of them), so that
// it prefetches only those
enum TableRow {
  T_K = 0,      // wavenumber k                       umwm_init.F90:1473
  T_CP0,        // phase speed cp0 (ghost = min)      :1493, :1653-1656
  T_CG0,        // group velocity cg0 (ghost = min)   :1494, :1653-1656
  T_LOGL2Z,     // log(l2/z), capped                  :1530-1533
  T_FKOVG,      // f k / g                            :1507
  T_KDK,        // k dk                               :1505
  T_K4,         // k^4                                :1503
  T_K3DK,       // k^3 dk                             :1506
  T_COTHKD,     // coth(0.2 kd)                       :1508
  T_SBF,        // bottom friction+percolation        :1510-1511
  T_SDV,        // viscous dissipation                :1512
  T_BF1R,       // Snl weight to o+1                  :1523
  T_BF2R,       // Snl weight to o+2                  :1524
  T_COUNT
};
constexpr int T_ADV_ROWS = T_KDK + 1;  // rows 0 .. T_KDK: all the propagation and stress read

constexpr int TILE = 64;  // wet points of a tile (a member's points start on a tile boundary)

// default levels ahead the spectral kernels prefetch the spectrum (and table)
// rows into L2 (Params::pf_*, tunable); measured on 1000x1000: the
// integration and the propagation are fastest at one level (two: +3 % and
// +5 %, four: +13 % and +8 %), the dts pre-pass at two
#ifndef UMWM_PF_DIST_PHYS
#define UMWM_PF_DIST_PHYS 2
#endif
#ifndef UMWM_PF_DIST_INTEG
#define UMWM_PF_DIST_INTEG 1
#endif
#ifndef UMWM_PF_DIST_ADV
#define UMWM_PF_DIST_ADV 1
#endif

// Direction groups per point of the spectral kernels: 4 quarter-turn groups
// when pm % 4 == 0 and pm/4 is a supported group size, else 2 half-turn groups.
__host__ __device__ constexpr bool quarter_groups(int pm) {
  return pm % 4 == 0 && (pm / 4 == 4 || pm / 4 == 6 || pm / 4 == 8 || pm / 4 == 9 || pm / 4 == 12);
}

struct Ctl;
struct Member;

struct Params {
  int Ntot, ldN, NB, O, P, NMtot, lm;
  int nmem;              // members
  int ntiles;            // CTA tiles of TILE points over the whole index space
  const Member* mem;     // [nmem]
  const int* tile_mem;   // member of each tile [ntiles]
  float g, explim, sin_fac, fieldscale1, fieldscale2, twopisds_fac, sds_power, inv_sds_power, mss_fac, snl_fac,
      sdt_fac, z, nu_air, kappa, fprog, dth, dthg, oneovdth, dtg, fice_lth, fice_uth, eulerinv, rhow0;
  float bf1, bf2;  // downshifting weights (umwm_init.F90:1290-1294)
  // Sin factors of negative x (sin_fold): sin_fac fieldscale1, and with
  // fieldscale2 where cos(wdir - th) > 0 (umwm_source_functions.F90:60-67)
  float sin_neg1, sin_neg2;
  float gustiness;      // wind gust amplitude (umwm_forcing.F90:49-61)
  unsigned gust_seed;   // seed of the gust draws (option "gust_seed")
  int winds, currents, air_density, water_density, seaice, restart, curvilinear, isglobal;
  int ice_possible;  // fice can exceed fice_lth somewhere
  int groups4;       // the integration uses 4 quarter-turn direction groups (option "direction_groups")
  int groups4_phys;  // the dts pre-pass does (options "direction_groups", "phys_groups")
  int adv_groups4;   // the propagation kernel does (options "direction_groups", "advect_groups")
  // Launch configuration of the three spectral kernels, chosen by the
  // autotuner or the options: the resident CTAs per SM their register budget
  // is sized for (__launch_bounds__ instances) and how many frequency levels
  // ahead they prefetch the spectrum and table rows into L2.  Results do not
  // depend on these.
  int minb_phys, minb_integ, minb_adv;
  int pf_phys, pf_integ, pf_adv;
  int count_cut;     // the propagation counts the bins its non-negativity cut changes (Global::cut_count)
  int swsign;        // the first pm/2 directions have sin th < 0, and cos th < 0 exactly for the first pm/4
                     // (pm % 4 == 0): the two-group flux takes one upwind term per slot pair
  int adv_tma;       // the propagation stages its own rows with bulk copies (k_advect_tma; option "advect_tma")
  int phys_tma;      // the dts pre-pass does (k_source_tma; option "phys_tma")
  float f[MAX_OM], dom[MAX_OM];
  float th[MAX_PM], cth[MAX_PM], sth[MAX_PM], c2th[MAX_PM], s2th[MAX_PM];
  float shs[MAX_PM], chs[MAX_PM];  // (sin th(p) + sin th(p+1)) / 2, the same for cos: the edge between p and p+1
  // max(cos th, 0), min(cos th, 0), max(sin th, 0), min(sin th, 0): the
  // upwind weights of propagation (umwm_advection.F90:34-47)
  float cthp[MAX_PM], cthm[MAX_PM], sthp[MAX_PM], sthm[MAX_PM];
  float depth[MAX_LM];
};

// Device-resident control block of the inner (dynamic-dts) loop, one per member.
struct Ctl {
  float sumt, dts, dta, dtr, dtr_temp;
  unsigned minphys_enc;   // ordered encoding of min_i(explim/max|arg|)
  unsigned maxrot_enc;    // ordered encoding of max rotation flux
  int anycurrent;         // set by the forcing kernel when a wet current is non-zero
  int zerocurrents;       // latched for propagation of this substep
  int first;              // reference's 'first' (first substep of the first run)
  int compute_rot;        // rotation recomputed this substep
  int done;               // sumt >= dtg: the member has finished the current dtg
  int running;            // the member takes part in the current substep
  int substep;            // substeps since initialize
  int err;                // error flags (bit 0: timeout)
  int log_count;
};

// Per-member ranges, scalars and pointers.
struct Member {
  int off, N, ghost;       // wet indices [off, off+N), ghost point off+N
  int nmoff, NM, mm, nm;   // all-point range [nmoff, nmoff+NM) and 2-d grid
  int iip;                 // index of the screen point, -1 if none
  float dtamin;
  Ctl* ctl;
  double* log;             // screen lines, 8 per substep
  int log_cap;
  const int *mi, *ni;      // 1-based (m, n) of each all-point index (member-local, [NM])
  // forcing levels (mm*nm, Fortran order): b = n, f = n+1
  const float *uwb, *uwf, *vwb, *vwf, *ucb, *ucf, *vcb, *vcf, *rhoab, *rhoaf, *rhowb, *rhowf, *ficeb, *ficef;
};

// control shared by all members (one per model)
struct Global {
  int not_done;            // members still inside the current dtg after this substep
  int budget;              // substeps the graph-driven inner loop may still run (-1: no limit)
  int iters;               // substeps the graph-driven inner loop ran since it was armed
  int nonfinite;           // non-finite values found by the last finite check
  int save_src;            // the last substep of this dtg keeps its source terms (for stress('ocn'))
  unsigned long long cut_count;  // bins whose negative ef the propagation cut to 0 (option "count_cut")
  // grid barrier of the persistent substep kernel: arrivals, generation,
  // and the error flag a timed-out wait sets (reset before each launch)
  unsigned bar_count, bar_gen;
  int bar_err;
  // time block 0 of the persistent kernel spent in each stage, up to and
  // including the barrier that ends it (globaltimer ns, accumulated over
  // launches until read): forcing, sea ice, dts pre-pass, dts, integration,
  // propagation, screen
  unsigned long long stage_ns[8];
};

struct Ptrs {
  float *E, *ES, *EF;  // spectrum arrays (EF aliases E: each bin is read and then overwritten by one thread)
  const float* TAB;     // [O][T_COUNT][ldN]
  // wet-point arrays [ldN]
  const int *ie, *iw, *in, *is;      // aliased neighbours (global index; the member's ghost for land)
  const int *iie, *iiw, *iin, *iis;  // true neighbours (global all-point index)
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
  // all-point arrays, member m at [nmoff, nmoff+NM) (land included; wet
  // points first, in the member's unrolled order)
  float *wspd, *wdir, *uc, *vc, *rhoa, *rhow, *rhorat, *fice;
  // Stokes drift [lm][ldN] and e-folding depth
  float *us, *vs, *ds;
  // diagnostics [ldN]
  float *ht, *mwp, *mwd, *mss, *mwl, *dwd, *dwl, *dwp, *dcp0, *dcp, *dcg0, *dcg, *momx, *momy, *cgmxx, *cgmxy,
      *cgmyy;
  Global* glob;
  // surrogate fallback (null otherwise): the source integration runs only
  // tiles with fb_tile[t] != 0 and writes only points with fb_pt[j] != 0
  const int* fb_tile;
  const unsigned char* fb_pt;
  // source terms of the last substep of a dtg, kept for stress('ocn') when
  // Global::save_src is set (null when not allocated): Sin, Sds after the
  // cothkd factor, Snl (spectrum layout) and the ustar they used [ldN]
  float *src_sin, *src_sds, *src_snl, *src_ust;
  float* ocn;  // stress('ocn') outputs, OCN_COUNT arrays of [ldN]
};

// stress('ocn') outputs (umwm_stress.F90:34-214), in this order in Ptrs::ocn
enum OcnField {
  OCN_TAUX_TOP = 0, OCN_TAUY_TOP, OCN_TAUX_BOT, OCN_TAUY_BOT, OCN_TAUX_SNL, OCN_TAUY_SNL, OCN_EPSX_OCN,
  OCN_EPSY_OCN, OCN_EPSX_ATM, OCN_EPSY_ATM, OCN_TAILX, OCN_TAILY, OCN_TAUX1, OCN_TAUY1, OCN_TAUX2, OCN_TAUY2,
  OCN_TAUX3, OCN_TAUY3, OCN_COUNT
};

// Wind gust draws, umwm_forcing.F90:49-56.  The reference fills gustu and
// gustv with Fortran random_number once per substep; here draw number
// (substep, cell, component) is a function of those three and a seed, so a
// run is reproducible and the oracle makes the same draws: the SplitMix64
// finaliser (Steele, Lea and Flood, 2014) of the seed and substep keys a
// second finalising of the cell index (column-major over the 2-d grid, as
// random_number fills an array) and the component (0: u, 1: v); its top
// 24 bits are the uniform draw in [0, 1).
__host__ __device__ inline uint64_t splitmix64_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ inline float gust_uniform(unsigned seed, unsigned substep, unsigned cell, unsigned comp) {
  const uint64_t key = splitmix64_mix(((uint64_t)seed << 32) | substep);
  const uint64_t z = splitmix64_mix(key ^ (((uint64_t)cell << 1) | comp));
  return (float)(z >> 40) * (1.f / 16777216.f);
}

// element offsets in the blocked layouts
__host__ __device__ inline size_t sidx(const Params& prm, int o, int p, int j) {
  return ((size_t)(o * prm.NB + (j >> 5)) * prm.P + p) * 32 + (j & 31);
}
__host__ __device__ inline size_t tidx(const Params& prm, int o, int t, int j) {
  return ((size_t)(o * prm.NB + (j >> 5)) * T_COUNT + t) * 32 + (j & 31);
}

}  // namespace umwm
