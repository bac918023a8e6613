// Device body of the propagation/refraction/stress kernel (see k_advect.cu),
// shared by the per-stage kernel and the persistent substep kernel.
#pragma once
#include "dev_common.cuh"

namespace umwm {

// bulk prefetch of a contiguous, 16-byte aligned range into L2
__device__ __forceinline__ void bulk_prefetch(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Sin at one direction (same expression as the source kernels)
__device__ __forceinline__ float sin_dir(const Params& prm, const WindIn& w, float U, float cw, float ucs, float vss,
                                         float cp0, float fkovg, bool tail) {
  return sin_fold(prm, w.shelt, U * cw - cp0 - ucs - vss, cw, w.c1 * fkovg, tail);
}

#ifndef UMWM_ADVECT_MINB
#define UMWM_ADVECT_MINB 4  // resident CTAs per SM the register budget is sized for (two groups):
                            // with the rows in halves, 128 registers and no spills measured fastest
                            // (3.06 ms against 3.25 at 5 CTAs, 3.71 at 6, 3.23 at 3)
#endif

#ifndef UMWM_ADVECT_HALVES
#define UMWM_ADVECT_HALVES 2  // each level's directions in this many parts (2: halves; 1: whole rows)
#endif

#ifndef UMWM_ADVECT_STAGE
#define UMWM_ADVECT_STAGE 1  // east/west neighbour rows staged in shared memory one level ahead
                             // (two buffers, or the own row staged too, measured slower)
#endif

#ifndef UMWM_ADVECT_PACKED
#define UMWM_ADVECT_PACKED 1  // the plain-grid propagation flux and the stress sums on direction pairs
                              // with packed f32x2 arithmetic: fastest propagation 3.05 ms (the staged
                              // form) against 3.13 scalar at 1000x1000; with the rows in thirds (whole
                              // pairs per part) 3.18
#endif

#ifndef UMWM_ADVECT_MINB4
#define UMWM_ADVECT_MINB4 4  // the same with four quarter-turn groups
#endif

// Shared memory of one CTA: cos(wdir - th) per lane and direction, the
// curvature-turned directions (curvilinear grids) and the staged east/west
// rows of the next level (ST).
template <int G, int H, bool CURV>
struct AdvSmem {
  // ST: the east/west neighbours' E* rows of the next level are copied into
  // shared memory (cp.async, per lane) once this level's propagation has
  // read them, and land while its refraction and stress run
  static constexpr bool ST = G == 2 && !CURV && H <= 18 && UMWM_ADVECT_STAGE;
  float cws[H][128];
  float ccs[CURV ? H : 1][128], scs[CURV ? H : 1][128];
  float stg[2][ST ? H : 1][128];
};

// The body of k_advect for CTA tile `cta` (the kernel's block index, or a
// persistent CTA's current tile).  CNT: also count the bins whose negative ef
// is cut to 0 (option "count_cut"; a separate instance so that the plain one
// carries no counter).  COH: E* is read with coherent loads instead of the
// read-only path, for a persistent kernel in which the same launch wrote it.
// TMA: the own rows come from shared memory staged by bulk copies (OwnStage;
// 1: the E* and e rows, 2: the E* rows only, e read as before;
// the two-group, plain-grid mapping with rows in halves only).
template <int G, int H, bool CURV, bool CNT, bool COH, int TMA = 0>
__device__ __forceinline__ void advect_body(const Params& prm, const Ptrs& P, int cta, AdvSmem<G, H, CURV>& sm,
                                            OwnStage own = OwnStage{nullptr, 0u}) {
  constexpr int PW = 32 / G;   // points per warp
  constexpr int PPC = 4 * PW;  // points per CTA (4 warps)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int jl = lane % PW, q = lane / PW;
  const int O = prm.O;
  const Member& Mb = prm.mem[prm.tile_mem[(cta * PPC) / TILE]];
  const Ctl* ctl = Mb.ctl;
  if (!ctl->running) return;  // the member has finished the current dtg
  const int N = Mb.ghost;
  const int j = cta * PPC + w * PW + jl;
  const bool valid = j < N;
  const int jj = valid ? j : N;
  const int ja = apt(Mb, jj);
  // rotation of this lane's group relative to the base group
  const float ra = G == 2 ? (q ? -1.f : 1.f) : (q == 0 ? 1.f : (q == 2 ? -1.f : 0.f));
  const float rb = G == 2 ? 0.f : (q == 1 ? 1.f : (q == 3 ? -1.f : 0.f));
  auto& cws = sm.cws;
  auto& ccs = sm.ccs;
  auto& scs = sm.scs;
  auto& stg = sm.stg;
  constexpr bool ST = AdvSmem<G, H, CURV>::ST;
  // loads of E*: the read-only path, or in a persistent kernel (which wrote
  // E* in the same launch) loads cached in L2 only (ld.global.cg), which
  // see the other CTAs' writes after the grid barrier (ordinary L1-cached
  // loads measured the same there: 6.90 ms against 6.91 per propagation
  // stage at 1000x1000).  E* is never written by this body, so its loads
  // may be ordered freely against the e stores
  auto lde = [](const float* __restrict__ p) { return COH ? __ldcg(p) : __ldg(p); };

  const float dta = ctl->dta, dtr = ctl->dtr;
  const bool zerocur = ctl->zerocurrents != 0;

  const int ie = P.ie[jj], iw = P.iw[jj], in = P.in[jj], is = P.is[jj];
  const int oc = P.oc[jj], ocr = P.oc_rot[jj];
  const bool ice = P.fice[ja] > prm.fice_uth;
  const float oneovar = P.oneovar[jj], dxn = P.dxn[jj], dxs = P.dxs[jj], dye = P.dye[jj], dyw = P.dyw[jj];
  const float odx = P.oneovdx[jj], ody = P.oneovdy[jj];
  const float ustar = P.ustar[jj];
  const WindIn wi = load_wind(prm, P, jj, ja, ustar);
  const float wdir = P.wdir[ja];
  const float ucg = G == 2 ? ra * wi.uc : ra * wi.uc + rb * wi.vc;
  const float vcg = G == 2 ? ra * wi.vc : ra * wi.vc - rb * wi.uc;

  // current advection, umwm_advection.F90:62-82, folded per point
  float F0 = 0.f, fedn = 0.f, fwup = 0.f, fndn = 0.f, fsup = 0.f;
  const float uci = P.uc[ja], vci = P.vc[ja];
  const float ucn = P.uc[P.iin[jj]], ucs = P.uc[P.iis[jj]];
  const float vce = P.vc[P.iie[jj]], vcw = P.vc[P.iiw[jj]];
  if (!zerocur) {
    const float uce = P.uc[P.iie[jj]], ucw = P.uc[P.iiw[jj]], vcn = P.vc[P.iin[jj]], vcs = P.vc[P.iis[jj]];
    const float ue = uci + uce, uw = uci + ucw, vn = vci + vcn, vs = vci + vcs;
    const float feup = (ue + fabsf(ue)) * dye, fwdn = (uw - fabsf(uw)) * dyw;
    const float fnup = (vn + fabsf(vn)) * dxn, fsdn = (vs - fabsf(vs)) * dxs;
    fedn = (ue - fabsf(ue)) * dye; fwup = (uw + fabsf(uw)) * dyw;
    fndn = (vn - fabsf(vn)) * dxn; fsup = (vs + fabsf(vs)) * dxs;
    F0 = feup - fwdn + fnup - fsdn;
  }
  const float bx = (vce - vcw), by = (ucn - ucs);
  // SW: each group reads its four neighbours in slots chosen so that every
  // group uses the base group's upwind weights max/min(cos th0, 0) and
  // max/min(sin th0, 0).  The flux is, per slot pair (A, B) with weights (wp, wm),
  //   D_A (wp e0 + wm e_A) - D_B (wp e_B + wm e0),
  // the cos pair (C) and the sin pair (S) summed.  Turned by a half turn
  // (cos th = -cos th0) the east-west terms of umwm_advection.F90:40-47 are
  // this with A = west, B = east; turned by a quarter turn (cos th = -sin th0,
  // sin th = cos th0) the north-south terms are the cos pair (N, S) and the
  // east-west terms the sin pair (W, E).  Slots: 0 east, 1 west, 2 north,
  // 3 south; the current terms follow their neighbours.
  constexpr bool SW = !CURV;
  const int turn = G == 2 ? 2 * q : q;  // quarter turns of this group
  const int sCA = turn == 0 ? 0 : turn == 1 ? 2 : turn == 2 ? 1 : 3;
  const int sCB = turn == 0 ? 1 : turn == 1 ? 3 : turn == 2 ? 0 : 2;
  const int sSA = turn == 0 ? 2 : turn == 1 ? 1 : turn == 2 ? 3 : 0;
  const int sSB = turn == 0 ? 3 : turn == 1 ? 0 : turn == 2 ? 2 : 1;
  auto slot = [](int n, auto e, auto w, auto nn, auto ss) { return n == 0 ? e : n == 1 ? w : n == 2 ? nn : ss; };
  const float kCA = slot(sCA, fedn, -fwup, fndn, -fsup), kCB = slot(sCB, fedn, -fwup, fndn, -fsup);
  const float kSA = slot(sSA, fedn, -fwup, fndn, -fsup), kSB = slot(sSB, fedn, -fwup, fndn, -fsup);

#pragma unroll
  for (int k = 0; k < H; ++k) {
    const float th = prm.th[q * H + k];
    cws[k][threadIdx.x] = cosf(wdir - th);
    if (CURV) {
      const float cv = P.curv[jj];
      ccs[k][threadIdx.x] = cosf(th + cv);
      scs[k][threadIdx.x] = sinf(th + cv);
    }
  }

  // blocked-layout offsets of the point and its neighbours
  const size_t lstride = (size_t)prm.NB * prm.P * 32;
  const size_t tstride = (size_t)prm.NB * T_COUNT * 32;
  const size_t hoff = (size_t)(q * H) * 32;
  const size_t oS = sidx(prm, 0, 0, jj) + hoff, oE = sidx(prm, 0, 0, ie) + hoff, oW = sidx(prm, 0, 0, iw) + hoff,
               oN = sidx(prm, 0, 0, in) + hoff, oSs = sidx(prm, 0, 0, is) + hoff;
  const size_t oCA = slot(sCA, oE, oW, oN, oSs), oCB = slot(sCB, oE, oW, oN, oSs);
  const size_t oSA = slot(sSA, oE, oW, oN, oSs), oSB = slot(sSB, oE, oW, oN, oSs);
  // stress_vector_integral divides by cp0 of the previous unrolled point
  // (assumed-shape dummy with lower bound 1 over cp0(:,0:im)),
  // umwm_stress.F90:401, :495-513; the member's first point uses its ghost
  const int jprev = (jj == Mb.off || jj >= N) ? N : jj - 1;
  const size_t tS = tidx(prm, 0, 0, jj), tE = tidx(prm, 0, 0, ie), tW = tidx(prm, 0, 0, iw),
               tN = tidx(prm, 0, 0, in), tSs = tidx(prm, 0, 0, is), tP = tidx(prm, 0, 0, jprev);
  const float dtaq = 0.25f * dta * oneovar;
  const float dtrq = dtr * prm.oneovdth;
  const size_t tCA = slot(sCA, tE, tW, tN, tSs), tCB = slot(sCB, tE, tW, tN, tSs);
  const size_t tSA = slot(sSA, tE, tW, tN, tSs), tSB = slot(sSB, tE, tW, tN, tSs);
  const float lCA = slot(sCA, dye, dyw, dxn, dxs), lCB = slot(sCB, dye, dyw, dxn, dxs);
  const float lSA = slot(sSA, dye, dyw, dxn, dxs), lSB = slot(sSB, dye, dyw, dxn, dxs);

  float sx = 0.f, sy = 0.f, dsx = 0.f, dsy = 0.f, txom = 0.f, tyom = 0.f;
  unsigned ncut = 0;  // bins of this lane whose negative ef was cut (CNT)
  // E* and e of this block prm.pf_adv frequencies ahead go to L2 in the background
  const size_t blk = sidx(prm, 0, 0, jj & ~31);
  // E* is read only at propagated levels o < oc (the warp's largest oc bounds them)
  const int ocw = (int)__reduce_max_sync(0xffffffffu, (unsigned)max(oc, 0));
  // (and the block's table rows, which every level reads)
  const size_t tblk = tidx(prm, 0, 0, jj & ~31);
  auto pf = [&](int o) {
    if (o < O && lane == 0) {
      if (o < ocw) bulk_prefetch(P.ES + blk + (size_t)o * lstride, (unsigned)(prm.P * 128));
      bulk_prefetch(P.EF + blk + (size_t)o * lstride, (unsigned)(prm.P * 128));
      if (UMWM_PREFETCH_TAB) bulk_prefetch(P.TAB + tblk + (size_t)o * tstride, (unsigned)(T_ADV_ROWS * 128));
    }
  };
  const int PFD = prm.pf_adv;  // levels prefetched ahead (a tunable)
  for (int o = 0; o < PFD; ++o) pf(o);

  // copies of level o's east/west rows (the cos slots A, B)
  auto stage = [&](int o) {
    if (ST && o < O && o < oc) {
      const float* __restrict__ ESo = P.ES + (size_t)o * lstride;
#pragma unroll
      for (int k = 0; k < (ST ? H : 0); ++k) {
        cp_async4(&stg[0][ST ? k : 0][threadIdx.x], ESo + oCA + k * 32);
        cp_async4(&stg[1][ST ? k : 0][threadIdx.x], ESo + oCB + k * 32);
      }
    }
    if (ST) cp_async_commit();
  };
  stage(0);

  // HV: the level's directions in two halves of H/2, so that a lane holds
  // half a row of e and E* at a time (fewer live registers); the rows at the
  // halves' edges and the neighbouring groups' edge rows are loaded again
  constexpr int NPART = UMWM_ADVECT_HALVES;  // parts of a row (2: halves)
  // (two groups: plain grids, whose neighbour slots are swapped per group,
  // and curvilinear grids, with the turned directions from shared memory;
  // with four groups a lane's row already holds H = 9 directions)
  constexpr bool HV = NPART > 1 && G == 2 && (H % (NPART > 1 ? NPART : 1) == 0);
  const size_t oPt = sidx(prm, 0, 0, jj);  // the point's row 0 (all groups)
  const int pprev = ((q + G - 1) % G) * H + H - 1, pnext = ((q + 1) % G) * H;
  // TMA: the own rows in shared memory.  jj (the ghost for padding lanes)
  // lies in this CTA's 64 points: a member's ghost is in its last tile
  static_assert(!TMA || (HV && SW && ST), "the TMA form is the two-group, plain-grid form with rows in halves");
  const int row = 2 * prm.P * 32;  // floats of one array (two blocks) in a buffer
  const int jl64 = jj - cta * PPC;
  const int sS = ((jl64 >> 5) * prm.P + q * H) * 32 + (jl64 & 31);  // the lane's row in a staged array
  const int sPt = ((jl64 >> 5) * prm.P) * 32 + (jl64 & 31);          // the point's row 0
  int occ = O;  // levels of which E* is staged: the CTA's largest cut-off
  const size_t src0 = sidx(prm, 0, 0, cta * PPC);
  constexpr bool TEF = TMA == 1;     // e staged as well
  constexpr int NA = TEF ? 2 : 1;    // arrays per buffer: E* (and e)
  auto issue = [&](int o) {  // one thread: level o's rows into buffer o & 1
    if (o >= O) return;
    const int b = o & 1;
    const uint32_t bar = own.mbar + 8u * b;
    const uint32_t bytes = (uint32_t)row * 4u;
    // (a level above every cut-off of a CTA that stages E* only copies
    // nothing: the arrival alone completes the phase)
    adv_mbar_expect(bar, ((o < occ ? 1u : 0u) + (TEF ? 1u : 0u)) * bytes);
    if (TEF)
      adv_bulk_copy(adv_smem_u32(own.buf + (size_t)(NA * b + 1) * row), P.EF + src0 + (size_t)o * lstride, bytes, bar);
    if (o < occ) adv_bulk_copy(adv_smem_u32(own.buf + (size_t)(NA * b) * row), P.ES + src0 + (size_t)o * lstride, bytes, bar);
  };
  if (TMA) {
    __shared__ int s_occ;
    if (threadIdx.x == 0) {
      s_occ = 0;
      adv_mbar_init(own.mbar);
      adv_mbar_init(own.mbar + 8u);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (lane == 0) atomicMax(&s_occ, ocw);
    __syncthreads();
    occ = s_occ;
    if (threadIdx.x == 0) issue(0);
  }
  for (int o = 0; o < (HV ? O : 0); ++o) {
    pf(o + PFD);
    if (ST) cp_async_wait<0>();  // this level's copies have landed
    if (TMA) {
      // this level's own rows have landed (bounded wait: an error flag and
      // a bounded drain of the other buffer's copy instead of a hang)
      const bool ok = adv_mbar_wait(own.mbar + 8u * (o & 1), (o >> 1) & 1, 4000000000LL);
      if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) {
          atomicOr(&const_cast<Ctl*>(ctl)->err, 2);
          if (o + 1 < O) adv_mbar_wait(own.mbar + 8u * ((o + 1) & 1), ((o + 1) >> 1) & 1, 400000000LL);
        }
        return;
      }
      // every thread is done with the other buffer (level o - 1): refill it
      if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(o + 1);
      }
    }
    const float* ownES = TMA ? own.buf + (size_t)(NA * (o & 1)) * row : nullptr;
    const float* ownE = TEF ? own.buf + (size_t)(NA * (o & 1) + 1) * row : nullptr;
    constexpr int HH = HV ? H / NPART : 1;
    const float* T = P.TAB + (size_t)o * tstride;
    const float* __restrict__ ESo = P.ES + (size_t)o * lstride;
    const float* EFo = P.EF + (size_t)o * lstride;
    float* Eo = P.E + (size_t)o * lstride;
    const bool prog = o < oc;
    const bool refr = prog && o < ocr;
    float DCA = 0.f, DCB = 0.f, DSA = 0.f, DSB = 0.f;
    float alc = 0.f, bec = 0.f, alp = 0.f, bep = 0.f, aln = 0.f, ben = 0.f, c0 = 0.f;
    if (prog) {
      // the four face weights: per slot (SW), or east, west, north, south
      const float cgi = __ldg(T + tS + T_CG0 * 32);
      DCA = 2.f * (cgi + __ldg(T + (SW ? tCA : tE) + T_CG0 * 32)) * (SW ? lCA : dye);
      DCB = 2.f * (cgi + __ldg(T + (SW ? tCB : tW) + T_CG0 * 32)) * (SW ? lCB : dyw);
      DSA = 2.f * (cgi + __ldg(T + (SW ? tSA : tN) + T_CG0 * 32)) * (SW ? lSA : dxn);
      DSB = 2.f * (cgi + __ldg(T + (SW ? tSB : tSs) + T_CG0 * 32)) * (SW ? lSB : dxs);
    }
    if (refr) {
      const float gx = 0.5f * (__ldg(T + tE + T_CP0 * 32) - __ldg(T + tW + T_CP0 * 32));
      const float gy = 0.5f * (__ldg(T + tN + T_CP0 * 32) - __ldg(T + tSs + T_CP0 * 32));
      c0 = (0.5f * bx) * odx - (0.5f * by) * ody;
      alc = gx * ra * odx; bec = -(gy * ra * ody);  // this group (G = 2: cb = 0)
      alp = gx * -ra * odx; bep = -(gy * -ra * ody);  // the other group, both neighbours
      aln = alp; ben = bep;
    }
    auto rot = [&](int k, float al, float be) { return al * prm.sth[k] + (be * prm.cth[k] + c0); };
    float rr = 0.f, fprev = 0.f;  // the rate and the flux of the edge before direction 0
    if (refr) rr = 0.5f * (rot(0, alc, bec) + rot(H - 1, alp, bep));
    const float U = wi.wspd + wi.ustar25 * __ldg(T + tS + T_LOGL2Z * 32);
    const float cp0 = __ldg(T + tS + T_CP0 * 32), fkovg = __ldg(T + tS + T_FKOVG * 32);
    const float kdk = __ldg(T + tS + T_KDK * 32);
    const float icp = 1.f / __ldg(T + tP + T_CP0 * 32);
    // PKD: packed f32x2 arithmetic (in every form, so that the forms stay
    // bit-identical to one another)
    constexpr bool PKD = UMWM_ADVECT_PACKED;
    float tx = 0.f, ty = 0.f;
    float2 tx2 = make_float2(0.f, 0.f), ty2 = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < (HV ? NPART : 1); ++h) {
      const int k0 = h * HH;
      float ef[HH];
#pragma unroll
      for (int i = 0; i < HH; ++i) ef[i] = TEF ? ownE[sS + (k0 + i) * 32] : EFo[oS + (k0 + i) * 32];  // e below the cut-off, ef above
      if (prog) {
        float es[HH];
#pragma unroll
        for (int i = 0; i < HH; ++i) es[i] = TMA ? ownES[sS + (k0 + i) * 32] : lde(ESo + oS + (k0 + i) * 32);
#pragma unroll
        for (int i = 0; i < HH; ++i) ef[i] = 2.f * es[i] - ef[i];  // ef = 2 E* - e
        // ---- propagation, umwm_advection.F90:30-97
        // PK: the swapped-slot flux of two directions (k, k+1) at a time in
        // packed f32x2 arithmetic; an odd last direction takes the scalar form
        constexpr bool PK = PKD && SW;
        constexpr int NPK = PK ? HH / 2 : 0;
        if constexpr (PK) {
          const float2 dca = make_float2(DCA, DCA), ndcb = make_float2(-DCB, -DCB);
          const float2 dsa = make_float2(DSA, DSA), ndsb = make_float2(-DSB, -DSB);
          const float2 ndt = make_float2(-dtaq, -dtaq);
#pragma unroll
          for (int n = 0; n < NPK; ++n) {
            const int i = 2 * n, k = k0 + i;
            const float2 e0 = make_float2(es[i], es[i + 1]);
            const float2 eca = ST ? make_float2(stg[0][ST ? k : 0][threadIdx.x], stg[0][ST ? k + 1 : 0][threadIdx.x])
                                  : make_float2(lde(ESo + oCA + k * 32), lde(ESo + oCA + (k + 1) * 32));
            const float2 ecb = ST ? make_float2(stg[1][ST ? k : 0][threadIdx.x], stg[1][ST ? k + 1 : 0][threadIdx.x])
                                  : make_float2(lde(ESo + oCB + k * 32), lde(ESo + oCB + (k + 1) * 32));
            const float2 esa = make_float2(lde(ESo + oSA + k * 32), lde(ESo + oSA + (k + 1) * 32));
            const float2 esb = make_float2(lde(ESo + oSB + k * 32), lde(ESo + oSB + (k + 1) * 32));
            float2 f;
            if constexpr (H % 2 == 0) {  // pm % 4 == 0 (checked at set-up: Params::swsign)
              // the base directions' signs: sin th < 0, and cos th < 0 for
              // k < H/2, > 0 above, so one upwind weight of each slot pair
              // is zero: cos th (D_A e_A - D_B e0) below H/2, cos th (D_A e0
              // - D_B e_B) above, sin th (D_A e_A - D_B e0) throughout
              constexpr int HF = H / 2;
              const bool nx = k < HF, ny = k + 1 < HF;
              const float2 ea = make_float2(nx ? eca.x : e0.x, ny ? eca.y : e0.y);
              const float2 eb = make_float2(nx ? e0.x : ecb.x, ny ? e0.y : ecb.y);
              const float2 u = __ffma2_rn(ndcb, eb, __fmul2_rn(dca, ea));
              const float2 v = __ffma2_rn(ndsb, e0, __fmul2_rn(dsa, esa));
              f = __ffma2_rn(make_float2(prm.sth[k], prm.sth[k + 1]), v,
                             __fmul2_rn(make_float2(prm.cth[k], prm.cth[k + 1]), u));
            } else {
              const float2 cp = make_float2(prm.cthp[k], prm.cthp[k + 1]), cm = make_float2(prm.cthm[k], prm.cthm[k + 1]);
              const float2 sp = make_float2(prm.sthp[k], prm.sthp[k + 1]), sm = make_float2(prm.sthm[k], prm.sthm[k + 1]);
              f = __fmul2_rn(dca, __ffma2_rn(cm, eca, __fmul2_rn(cp, e0)));
              f = __ffma2_rn(ndcb, __ffma2_rn(cm, e0, __fmul2_rn(cp, ecb)), f);
              f = __ffma2_rn(dsa, __ffma2_rn(sm, esa, __fmul2_rn(sp, e0)), f);
              f = __ffma2_rn(ndsb, __ffma2_rn(sm, e0, __fmul2_rn(sp, esb)), f);
            }
            if (!zerocur) {
              f = __ffma2_rn(make_float2(F0, F0), e0, f);
              f = __ffma2_rn(make_float2(kCA, kCA), eca, f);
              f = __ffma2_rn(make_float2(kCB, kCB), ecb, f);
              f = __ffma2_rn(make_float2(kSA, kSA), esa, f);
              f = __ffma2_rn(make_float2(kSB, kSB), esb, f);
            }
            const float2 r = __ffma2_rn(ndt, f, make_float2(ef[i], ef[i + 1]));
            ef[i] = r.x;
            ef[i + 1] = r.y;
          }
        }
#pragma unroll
        for (int i = 2 * NPK; i < HH; ++i) {
          const int k = k0 + i;
          const float e0 = es[i];
          float flux;
          if (SW) {
            const float eca = ST ? stg[0][ST ? k : 0][threadIdx.x] : lde(ESo + oCA + k * 32);
            const float ecb = ST ? stg[1][ST ? k : 0][threadIdx.x] : lde(ESo + oCB + k * 32);
            const float esa = lde(ESo + oSA + k * 32), esb = lde(ESo + oSB + k * 32);
            const float cp = prm.cthp[k], cm = prm.cthm[k], sp = prm.sthp[k], sm = prm.sthm[k];
            flux = DCA * (cp * e0 + cm * eca) - DCB * (cp * ecb + cm * e0) + DSA * (sp * e0 + sm * esa) -
                   DSB * (sp * esb + sm * e0);
            if (!zerocur) flux += F0 * e0 + kCA * eca + kCB * ecb + kSA * esa + kSB * esb;
          } else {  // curvilinear: the directions turned by the grid's curvature
            const float ee = lde(ESo + oE + k * 32), ew = lde(ESo + oW + k * 32);
            const float en = lde(ESo + oN + k * 32), esn = lde(ESo + oSs + k * 32);
            const float cc = ccs[CURV ? k : 0][threadIdx.x], sc = scs[CURV ? k : 0][threadIdx.x];
            const float cp = fmaxf(cc, 0.f), cm = fminf(cc, 0.f), sp = fmaxf(sc, 0.f), sm = fminf(sc, 0.f);
            flux = DCA * (cp * e0 + cm * ee) - DCB * (cp * ew + cm * e0) + DSA * (sp * e0 + sm * en) -
                   DSB * (sp * esn + sm * e0);
            if (!zerocur) flux += F0 * e0 + fedn * ee - fwup * ew + fndn * en - fsup * esn;
          }
          ef[i] = ef[i] - dtaq * flux;
        }
        if (h == NPART - 1) stage(o + 1);  // the staged rows have been read
        // ---- refraction, umwm_advection.F90:122-178
        if (refr) {
          // E* beyond this part's edges: the neighbouring parts, or the other
          // group's edge rows
          const float esL = TMA ? (h == 0 ? ownES[sPt + pprev * 32] : ownES[sS + (k0 - 1) * 32])
                                : (h == 0 ? lde(ESo + oPt + pprev * 32) : lde(ESo + oS + (k0 - 1) * 32));
          const float esR = TMA ? (h == NPART - 1 ? ownES[sPt + pnext * 32] : ownES[sS + (k0 + HH) * 32])
                                : (h == NPART - 1 ? lde(ESo + oPt + pnext * 32) : lde(ESo + oS + (k0 + HH) * 32));
          // the flux through the edge between k and k+1, F(k) = max(rl, 0)
          // e(k) + min(rl, 0) e(k+1) = rl e(upwind side), with rl the edge's
          // rotation rate (the mean of the two directions' rates, from the
          // edge's mean sin and cos); each direction takes F(k) - F(k-1),
          // and F(k) carries on
          if (h == 0) fprev = rr * (rr > 0.f ? esL : es[0]);
#pragma unroll
          for (int i = 0; i < HH; ++i) {
            const int k = k0 + i;
            const float rl = (k + 1 < H) ? fmaf(alc, prm.shs[k], fmaf(bec, prm.chs[k], c0))
                                         : 0.5f * (rot(H - 1, alc, bec) + rot(0, aln, ben));
            const float el = (i + 1 < HH) ? es[i + 1] : esR;
            const float fk = rl * (rl > 0.f ? es[i] : el);  // the upwind side's E*
            ef[i] = ef[i] - dtrq * (fk - fprev);
            fprev = fk;
          }
        }
        if (ice) {
#pragma unroll
          for (int i = 0; i < HH; ++i) ef[i] = 0.f;
        }
      }
      // ---- e = ef, and the form-stress integrand with the new spectrum
      float sdir[HH];
#pragma unroll
      for (int i = 0; i < HH; ++i) {
        const int k = k0 + i;
        if (CNT) ncut += (valid && ef[i] < 0.f) ? 1 : 0;
        ef[i] = max_nan0(ef[i]);  // NaN stays NaN
        if (valid && prog) Eo[oS + k * 32] = ef[i];
        // Sin without the level's factor gl = c1 fkovg (>= 0), which
        // multiplies the level's stress sums instead
        const float cw = cws[k][threadIdx.x];
        const float x = U * cw - cp0 - ucg * prm.cth[k] - vcg * prm.sth[k];
        const float sf = (x * fabsf(x)) * (x > 0.f ? wi.shelt : (cw > 0.f ? prm.sin_neg2 : prm.sin_neg1));
        sdir[i] = prog ? sf : fmaxf(sf, 0.f);
      }
      if constexpr (PKD) {  // even and odd directions summed apart
#pragma unroll
        for (int i = 0; i + 1 < HH; i += 2) {
          const int k = k0 + i;
          const float2 es2 = __fmul2_rn(make_float2(ef[i], ef[i + 1]), make_float2(sdir[i], sdir[i + 1]));
          tx2 = __ffma2_rn(es2, make_float2(prm.cth[k], prm.cth[k + 1]), tx2);
          ty2 = __ffma2_rn(es2, make_float2(prm.sth[k], prm.sth[k + 1]), ty2);
        }
      }
#pragma unroll
      for (int i = PKD ? HH & ~1 : 0; i < HH; ++i) {
        const int k = k0 + i;
        const float es_ = ef[i] * sdir[i];
        tx += es_ * prm.cth[k];
        ty += es_ * prm.sth[k];
      }
    }
    if (PKD) {
      tx += tx2.x + tx2.y;
      ty += ty2.x + ty2.y;
    }
    tx *= ra * icp * (wi.c1 * fkovg);
    ty *= ra * icp * (wi.c1 * fkovg);
    sx += tx * kdk; sy += ty * kdk;
    if (o >= oc - 1) { dsx += tx * kdk; dsy += ty * kdk; }
    if (o == O - 1) { txom = tx; tyom = ty; }
  }

  for (int o = 0; o < (HV ? 0 : O); ++o) {
    pf(o + PFD);
    if (ST) cp_async_wait<0>();  // this level's copies have landed
    const float* T = P.TAB + (size_t)o * tstride;
    const float* __restrict__ ESo = P.ES + (size_t)o * lstride;
    const float* EFo = P.EF + (size_t)o * lstride;
    float* Eo = P.E + (size_t)o * lstride;
    float ef[H];
#pragma unroll
    for (int k = 0; k < H; ++k) ef[k] = EFo[oS + k * 32];  // EF aliases E: e below the cut-off, ef above
    const bool prog = o < oc;
    const unsigned pm = __ballot_sync(0xffffffffu, prog);
    if (prog) {
      float es[H];
#pragma unroll
      for (int k = 0; k < H; ++k) es[k] = lde(ESo + oS + k * 32);
      // the integration left e here and wrote E* = (e + ef)/2: ef = 2 E* - e.
      // The explicit step keeps ef/e within about [exp(-explim), exp(explim)],
      // so the difference loses at most a few ulp of ef
#pragma unroll
      for (int k = 0; k < H; ++k) ef[k] = 2.f * es[k] - ef[k];
      const float esm = __shfl_sync(pm, es[H - 1], (lane - PW) & 31);  // E* at p-1 for k = 0 (group q-1)
      const float esp = __shfl_sync(pm, es[0], (lane + PW) & 31);      // E* at p+1 for k = H-1 (group q+1)
      // ---- propagation, umwm_advection.F90:30-97
      const float cgi = __ldg(T + tS + T_CG0 * 32);
      if (SW) {
        const float DCA = 2.f * (cgi + __ldg(T + tCA + T_CG0 * 32)) * lCA;
        const float DCB = 2.f * (cgi + __ldg(T + tCB + T_CG0 * 32)) * lCB;
        const float DSA = 2.f * (cgi + __ldg(T + tSA + T_CG0 * 32)) * lSA;
        const float DSB = 2.f * (cgi + __ldg(T + tSB + T_CG0 * 32)) * lSB;
#pragma unroll
        for (int k = 0; k < H; ++k) {
          const float e0 = es[k];
          const float eca = ST ? stg[0][ST ? k : 0][threadIdx.x] : lde(ESo + oCA + k * 32);
          const float ecb = ST ? stg[1][ST ? k : 0][threadIdx.x] : lde(ESo + oCB + k * 32);
          const float esa = lde(ESo + oSA + k * 32), esb = lde(ESo + oSB + k * 32);
          const float cp = prm.cthp[k], cm = prm.cthm[k], sp = prm.sthp[k], sm = prm.sthm[k];
          float flux = DCA * (cp * e0 + cm * eca) - DCB * (cp * ecb + cm * e0) + DSA * (sp * e0 + sm * esa) -
                       DSB * (sp * esb + sm * e0);
          if (!zerocur) flux += F0 * e0 + kCA * eca + kCB * ecb + kSA * esa + kSB * esb;
          ef[k] = ef[k] - dtaq * flux;
        }
      }
      if (ST) stage(o + 1);  // the buffer has been read
      const float DE = SW ? 0.f : 2.f * (cgi + __ldg(T + tE + T_CG0 * 32)) * dye;
      const float DW = SW ? 0.f : 2.f * (cgi + __ldg(T + tW + T_CG0 * 32)) * dyw;
      const float DN = SW ? 0.f : 2.f * (cgi + __ldg(T + tN + T_CG0 * 32)) * dxn;
      const float DS = SW ? 0.f : 2.f * (cgi + __ldg(T + tSs + T_CG0 * 32)) * dxs;
#pragma unroll
      for (int k = 0; k < (SW ? 0 : H); ++k) {
        const float e0 = es[k];
        const float ee = lde(ESo + oE + k * 32), ew = lde(ESo + oW + k * 32);
        const float en = lde(ESo + oN + k * 32), esn = lde(ESo + oSs + k * 32);
        const float cc = CURV ? ccs[k][threadIdx.x]
                              : (G == 2 ? ra * prm.cth[k] : ra * prm.cth[k] - rb * prm.sth[k]);
        const float sc = CURV ? scs[k][threadIdx.x]
                              : (G == 2 ? ra * prm.sth[k] : rb * prm.cth[k] + ra * prm.sth[k]);
        const float cp = fmaxf(cc, 0.f), cm = fminf(cc, 0.f), sp = fmaxf(sc, 0.f), sm = fminf(sc, 0.f);
        float flux = DE * (cp * e0 + cm * ee) - DW * (cp * ew + cm * e0) + DN * (sp * e0 + sm * en) -
                     DS * (sp * esn + sm * e0);
        if (!zerocur) flux += F0 * e0 + fedn * ee - fwup * ew + fndn * en - fsup * esn;
        ef[k] = ef[k] - dtaq * flux;
      }
      // ---- refraction, umwm_advection.F90:122-178
      if (o < ocr) {
        const float gx = 0.5f * (__ldg(T + tE + T_CP0 * 32) - __ldg(T + tW + T_CP0 * 32));
        const float gy = 0.5f * (__ldg(T + tN + T_CP0 * 32) - __ldg(T + tSs + T_CP0 * 32));
        const float hbx = 0.5f * bx, hby = 0.5f * by;
        // rotation rate at base direction k of a group turned by (ca, cb)
        // (sin th = cb cos th0 + ca sin th0, cos th = ca cos th0 - cb sin th0):
        //   (gx sin th + hbx) odx - (gy cos th + hby) ody
        //   = al sin th0 + be cos th0 + c0, the coefficients per group
        const float c0 = hbx * odx - hby * ody;
        auto coef = [&](float ca, float cb, float& al, float& be) {
          al = gx * ca * odx + gy * cb * ody;
          be = gx * cb * odx - gy * ca * ody;
        };
        float alc, bec, alp, bep, aln, ben;
        coef(ra, rb, alc, bec);
        // the previous group is this one turned back by 2pi/G, the next one turned on
        coef(G == 2 ? -ra : rb, G == 2 ? 0.f : -ra, alp, bep);
        coef(G == 2 ? -ra : -rb, G == 2 ? 0.f : ra, aln, ben);
        auto rot = [&](int k, float al, float be) { return al * prm.sth[k] + (be * prm.cth[k] + c0); };
        // rr(p) = rl(p-1): the edge rate between p-1 and p, carried over k
        float rr = 0.5f * (rot(0, alc, bec) + rot(H - 1, alp, bep));
        float rcur = rot(0, alc, bec);
#pragma unroll
        for (int k = 0; k < H; ++k) {
          const float rnext = (k + 1 < H) ? rot(k + 1, alc, bec) : rot(0, aln, ben);
          const float rl = 0.5f * (rcur + rnext);  // pl(p) = p+1
          const float el = (k + 1 < H) ? es[k + 1] : esp;
          const float er = (k > 0) ? es[k - 1] : esm;
          const float fl = fmaxf(rl, 0.f) * es[k] + fminf(rl, 0.f) * el - fmaxf(rr, 0.f) * er - fminf(rr, 0.f) * es[k];
          ef[k] = ef[k] - dtrq * fl;
          rr = rl;
          rcur = rnext;
        }
      }
      // sea ice above fice_uth: propagation and refraction leave ef = 0
      // (umwm_advection.F90:89-97, :170-178)
      if (ice) {
#pragma unroll
        for (int k = 0; k < H; ++k) ef[k] = 0.f;
      }
    }
    // ---- e = ef, and the form-stress integrand with the new spectrum
    const float U = wi.wspd + wi.ustar25 * __ldg(T + tS + T_LOGL2Z * 32);
    const float cp0 = __ldg(T + tS + T_CP0 * 32), fkovg = __ldg(T + tS + T_FKOVG * 32);
    const float kdk = __ldg(T + tS + T_KDK * 32);
    const float icp = 1.f / __ldg(T + tP + T_CP0 * 32);
    const bool tail = !prog;
    float tx = 0.f, ty = 0.f;
#pragma unroll
    for (int k = 0; k < H; ++k) {
      // negatives are cut to 0: the explicit Snl term (snl_d12) can leave a
      // tiny negative ef, and a negative e makes the next step's
      // (e k^4)^sds_power NaN (the oracle cuts them at the same point)
      if (CNT) ncut += (valid && ef[k] < 0.f) ? 1 : 0;
      ef[k] = ef[k] < 0.f ? 0.f : ef[k];  // NaN stays NaN (the finite check must see it)
      // above the cut-off e = ef is already in place (EF aliases E)
      if (valid && prog) Eo[oS + k * 32] = ef[k];
      const float s = sin_dir(prm, wi, U, cws[k][threadIdx.x], ucg * prm.cth[k], vcg * prm.sth[k], cp0, fkovg, tail);
      const float es_ = ef[k] * s;
      tx += es_ * prm.cth[k];
      ty += es_ * prm.sth[k];
    }
    if (G == 2) {
      tx *= ra * icp;
      ty *= ra * icp;
    } else {  // sums over cos/sin th0 turned into the group's frame
      const float bx_ = tx, by_ = ty;
      tx = (ra * bx_ - rb * by_) * icp;
      ty = (rb * bx_ + ra * by_) * icp;
    }
    sx += tx * kdk; sy += ty * kdk;
    if (o >= oc - 1) { dsx += tx * kdk; dsy += ty * kdk; }
    if (o == O - 1) { txom = tx; tyom = ty; }
  }
#pragma unroll
  for (int m = PW; m < 32; m <<= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, m);
    sy += __shfl_xor_sync(0xffffffffu, sy, m);
    dsx += __shfl_xor_sync(0xffffffffu, dsx, m);
    dsy += __shfl_xor_sync(0xffffffffu, dsy, m);
    txom += __shfl_xor_sync(0xffffffffu, txom, m);
    tyom += __shfl_xor_sync(0xffffffffu, tyom, m);
  }
  if (CNT) {
    const unsigned c = __reduce_add_sync(0xffffffffu, ncut);
    if (lane == 0 && c) atomicAdd(&P.glob->cut_count, (unsigned long long)c);
  }
  if (q != 0 || !valid) return;
  // ---- stress('atm') per point, umwm_stress.F90:216-262
  const float rhow = P.rhow[ja], rhoa = P.rhoa[ja], wspd = wi.wspd;
  const float kom = __ldg(P.TAB + (size_t)(O - 1) * tstride + tS + T_K * 32);
  const float tl = stress_tail(wspd, kom);
  const float tax = txom * kom * tl * rhow * prm.dthg;
  const float tay = tyom * kom * tl * rhow * prm.dthg;
  const float tfx = sx * rhow * prm.dthg + tax;
  const float tfy = sy * rhow * prm.dthg + tay;
  P.tailatmx[j] = tax; P.tailatmy[j] = tay;
  P.taux_form[j] = tfx; P.tauy_form[j] = tfy;
  P.taux_diag[j] = dsx * rhow * prm.dthg;
  P.tauy_diag[j] = dsy * rhow * prm.dthg;
  const float us1 = prm.lm > 0 ? P.us[j] : 0.f, vs1 = prm.lm > 0 ? P.vs[j] : 0.f;
  const float urel = wspd * cosf(wdir) - (uci + us1);
  const float vrel = wspd * sinf(wdir) - (vci + vs1);
  const float wrel = sqrtf(urel * urel + vrel * vrel);
  const float drel = atan2f(vrel, urel);
  const float cdf = sqrtf(tfx * tfx + tfy * tfy) / (rhoa * (wspd * wspd));
  float z0 = 1e-3f, usk = 0.f;
  for (int n = 0; n < 6; ++n) {  // friction_velocity_skin, :275-298
    usk = prm.kappa * wrel / logf(prm.z / z0);
    z0 = 0.132f * prm.nu_air / usk;
  }
  float cds = (usk * usk) / (wspd * wspd);
  cds = cds * (1.f + 2.f * cds / (cds + cdf + 1.17549435e-38f)) / 3.f;
  if (cds > 1e-2f) cds = 1e-2f;
  const float tsx = rhoa * cds * (wrel * wrel) * cosf(drel);
  const float tsy = rhoa * cds * (wrel * wrel) * sinf(drel);
  P.taux_skin[j] = tsx; P.tauy_skin[j] = tsy;
  const float tx = tfx + tsx, ty = tfy + tsy;
  P.taux[j] = tx; P.tauy[j] = ty;
  const float tm = sqrtf(tx * tx + ty * ty);
  P.cd[j] = tm / (rhoa * (wspd * wspd));
  P.ustar[j] = sqrtf(tm / rhoa);
}

}  // namespace umwm
