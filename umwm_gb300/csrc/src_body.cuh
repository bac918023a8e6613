// Device bodies of the source-term kernels (see k_source.cu for the thread
// mapping and the two modes), shared by the per-stage kernels and the
// persistent substep kernel.
#pragma once
#include "dev_common.cuh"

namespace umwm {

// bulk prefetch of a contiguous, 16-byte aligned range into L2 (sizes are multiples of 16 bytes)
__device__ __forceinline__ void bulk_prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ float ex2a(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2a(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// x^y for x >= 0 (0 for x == 0)
__device__ __forceinline__ float powp(float x, float y) { return ex2a(y * lg2a(x)); }

template <int H>
struct Level {  // per-(o, point) inputs of one frequency level
  float k4, logl2z, cp0, fkovg, cothkd, sbf, sdv, kk, bf1r, bf2r, cg0, k3dk;
};
struct Coef {  // dummy coefficients A + B cos2th + C sin2th of one level
  float a, b, c;
};

// T points at table row 0 of this point's block and frequency
template <int H>
__device__ __forceinline__ Level<H> load_level(const Params& prm, const float* T, bool full) {
  Level<H> L;
  L.k4 = __ldg(T + T_K4 * 32);
  L.k3dk = __ldg(T + T_K3DK * 32);
  if (full) {
    L.logl2z = __ldg(T + T_LOGL2Z * 32);
    L.cp0 = __ldg(T + T_CP0 * 32);
    L.fkovg = __ldg(T + T_FKOVG * 32);
    L.cothkd = __ldg(T + T_COTHKD * 32);
    L.sbf = __ldg(T + T_SBF * 32);
    L.sdv = __ldg(T + T_SDV * 32);
    L.kk = __ldg(T + T_K * 32);
    L.bf1r = __ldg(T + T_BF1R * 32);
    L.bf2r = __ldg(T + T_BF2R * 32);
    L.cg0 = prm.ice_possible ? __ldg(T + T_CG0 * 32) : 0.f;
  }
  return L;
}

// Sin at direction k of this half; cw = cos(wdir - th(p)) from shared memory.
__device__ __forceinline__ float sin_k(const Params& prm, const WindIn& w, float U, float cw, float ucs, float vss,
                                       float cp0, float fkovg, bool tail) {
  return sin_fold(prm, w.shelt, U * cw - cp0 - ucs - vss, cw, w.c1 * fkovg, tail);
}

#ifndef UMWM_INTEG_MINB
#define UMWM_INTEG_MINB 4  // resident CTAs per SM the register budget is sized for (two groups);
                           // with the lagged levels in shared memory: 122 registers, no spills
#endif
#ifndef UMWM_INTEG_PACKED
#define UMWM_INTEG_PACKED 1  // the mss sums, the Sds factors and the integration step on direction
                             // pairs in packed f32x2 arithmetic
#endif
#ifndef UMWM_INTEG_SMEM_LAGS
#define UMWM_INTEG_SMEM_LAGS 1  // the integration keeps its two lagged levels in shared memory
                                // (37 KB per CTA): 3.56 ms instead of 4.28 ms with them in registers
#endif
#ifndef UMWM_PHYS_MINB
#define UMWM_PHYS_MINB 6  // 80 registers, no spills; measured faster than 5 (96) and 4 (128)
#endif

// Shared memory of one CTA: cos(wdir - th) per lane and direction, and (with
// SL) the integration's two lagged levels of e and raw Sds.
template <int G, int H, bool INTEG>
struct SrcSmem {
  static constexpr bool SL = INTEG && UMWM_INTEG_SMEM_LAGS && H <= 18;  // within 48 KB of static shared memory
  float cws[H][128];
  float lag[SL ? 2 : 1][2][SL ? H : 1][128];
};

// The body of k_source for the CTA tile bx (the kernel's blockIdx.x, or a
// persistent CTA's current tile).  SAVE (integration only): this substep also stores
// its source terms for stress('ocn'); a separate instantiation, so that the
// substeps that store nothing carry no predicated stores.
// TMA (dts pre-pass, two groups): the own e rows come from shared memory,
// staged one level ahead by bulk copies (OwnStage, one array per buffer).
template <int G, int H, bool INTEG, bool SAVE, bool TMA = false>
__device__ __forceinline__ void source_body(const Params& prm, const Ptrs& P, int compute_rot, int bx,
                                            SrcSmem<G, H, INTEG>& sm, OwnStage own = OwnStage{nullptr, 0u}) {
  static_assert(!TMA || (!INTEG && G == 2), "the TMA form is the two-group dts pre-pass");
  constexpr int PW = 32 / G;   // points per warp
  constexpr int PPC = 4 * PW;  // points per CTA (4 warps)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int jl = lane % PW, q = lane / PW;
  const int O = prm.O;
  const int tile = (bx * PPC) / TILE;
  const Member& Mb = prm.mem[prm.tile_mem[tile]];
  Ctl* ctl = Mb.ctl;
  // members that have finished the current dtg sit the substep out
  if (INTEG ? !ctl->running : ctl->done) return;
  if (INTEG && P.fb_tile && !P.fb_tile[tile]) return;  // surrogate fallback: flagged tiles only
  const int N = Mb.ghost;  // this member's ghost point (its wet points end here)
  const int j = bx * PPC + w * PW + jl;
  const bool valid = j < N && (!INTEG || !P.fb_pt || P.fb_pt[j]);
  const int jj = valid ? j : N;  // the ghost keeps loads in bounds
  const int ja = apt(Mb, jj);
  // rotation of this lane's group relative to the base group
  const float ra = G == 2 ? (q ? -1.f : 1.f) : (q == 0 ? 1.f : (q == 2 ? -1.f : 0.f));
  const float rb = G == 2 ? 0.f : (q == 1 ? 1.f : (q == 3 ? -1.f : 0.f));
  const float c2s = (G == 4 && (q & 1)) ? -1.f : 1.f;  // cos/sin(2 th) sign of the group
  auto& cws = sm.cws;  // cos(wdir - th) per lane and direction

  const float dts = INTEG ? ctl->dts : 0.f;
  const float dtsl2 = dts * 1.44269504f;  // dts log2(e)
  // the last substep of the dtg keeps its source terms when stress('ocn') is due
  constexpr bool save = INTEG && SAVE;
  const float ustar = P.ustar[jj];
  if (save && valid && q == 0) P.src_ust[j] = ustar;  // the ustar of this substep's sdt
  const WindIn wi = load_wind(prm, P, jj, ja, ustar);
  const float wdir = P.wdir[ja];
  const float sdtc = (prm.sdt_fac * sqrtf(P.rhorat[ja])) * ustar;
  const float sv = prm.ice_possible ? P.sice_v[jj] : 0.f;
  const float hdth = 0.5f * prm.dth;
  // currents in the group's frame: uc cos th + vc sin th = ucg cos th0 + vcg sin th0
  const float ucg = G == 2 ? ra * wi.uc : ra * wi.uc + rb * wi.vc;
  const float vcg = G == 2 ? ra * wi.vc : ra * wi.vc - rb * wi.uc;
#pragma unroll
  for (int k = 0; k < H; ++k) cws[k][threadIdx.x] = cosf(wdir - prm.th[q * H + k]);
#define CW(k) (cws[k][threadIdx.x])
  // own bins only: no barrier needed (each thread reads its own column)

  int nie = N, niw = N, nin = N, nis = N;
  float vce = 0.f, vcw = 0.f, ucn = 0.f, ucs = 0.f, odx = 0.f, ody = 0.f;
  if (!INTEG && compute_rot) {
    nie = P.ie[jj]; niw = P.iw[jj]; nin = P.in[jj]; nis = P.is[jj];  // global indices
    vce = P.vc[P.iie[jj]]; vcw = P.vc[P.iiw[jj]]; ucn = P.uc[P.iin[jj]]; ucs = P.uc[P.iis[jj]];
    odx = P.oneovdx[jj]; ody = P.oneovdy[jj];
  }

  // level strides of the blocked layouts
  const size_t lstride = (size_t)prm.NB * prm.P * 32;
  const size_t tstride = (size_t)prm.NB * T_COUNT * 32;
  const float* Eb = P.E + sidx(prm, 0, q * H, jj);
  const float* Tb = P.TAB + tidx(prm, 0, 0, jj);
  const float* Eblk = P.E + sidx(prm, 0, 0, jj & ~31);  // start of this block's region
  // the dts pre-pass needs only the prognostic levels o < oc (the mss prefix
  // of a level uses the levels below it): the warp stops at its largest oc
  const int OP = INTEG ? O : min(O, (int)__reduce_max_sync(0xffffffffu, (unsigned)max(wi.oc, 0)));
  const float* Tblk = P.TAB + tidx(prm, 0, 0, jj & ~31);  // this block's table rows
  auto pf = [&](int o) {
    if (o < OP && lane == 0 && (G == 2 || (w * PW) % 32 == 0)) {
      bulk_prefetch_l2(Eblk + (size_t)o * lstride, (unsigned)(prm.P * 128));
      if (UMWM_PREFETCH_TAB) bulk_prefetch_l2(Tblk + (size_t)o * tstride, (unsigned)(T_COUNT * 128));
    }
  };
  const int PFD = INTEG ? prm.pf_integ : prm.pf_phys;  // levels prefetched ahead (a tunable)
  for (int o = 0; o < PFD; ++o) pf(o);

  float A = 0.f, B = 0.f, C = 0.f;  // dummy coefficients of the current level
  float mx = 0.f, rmx = 0.f;
  // the current level and the two previous ones (e and raw Sds per direction);
  // with SL the previous two live in shared memory, slot = level & 1
  constexpr bool SL = SrcSmem<G, H, INTEG>::SL;
  auto& lag = sm.lag;
  float ec[H], sc[H], e1[SL ? 1 : H], s1[SL ? 1 : H], e2[SL ? 1 : H], s2[SL ? 1 : H];
#pragma unroll
  for (int k = 0; k < H; ++k) ec[k] = sc[k] = 0.f;
  if (!SL) {
#pragma unroll
    for (int k = 0; k < (SL ? 1 : H); ++k) e1[k] = s1[k] = e2[k] = s2[k] = 0.f;
  }
#define LAG_E1(k) (SL ? lag[(o - 1) & 1][0][SL ? (k) : 0][threadIdx.x] : e1[SL ? 0 : (k)])
#define LAG_S1(k) (SL ? lag[(o - 1) & 1][1][SL ? (k) : 0][threadIdx.x] : s1[SL ? 0 : (k)])
#define LAG_E2(k) (SL ? lag[o & 1][0][SL ? (k) : 0][threadIdx.x] : e2[SL ? 0 : (k)])
#define LAG_S2(k) (SL ? lag[o & 1][1][SL ? (k) : 0][threadIdx.x] : s2[SL ? 0 : (k)])
  Coef Cc{}, C1{}, C2{};

  int OL = INTEG ? O + 2 : OP;
  // TMA: the CTA's two blocks of e at level o in buffer o & 1; every warp
  // walks to the CTA's largest cut-off (levels above a lane's own add
  // nothing to its max).  jj (the ghost for padding lanes) lies in this
  // CTA's 64 points: a member's ghost is in its last tile
  const int row = 2 * prm.P * 32;
  const int jl64 = jj - bx * PPC;
  const int sS = ((jl64 >> 5) * prm.P + q * H) * 32 + (jl64 & 31);
  const size_t src0 = sidx(prm, 0, 0, bx * PPC);
  auto issue = [&](int o) {  // one thread
    if (o >= OL) return;
    const uint32_t bar = own.mbar + 8u * (o & 1);
    adv_mbar_expect(bar, (uint32_t)row * 4u);
    adv_bulk_copy(adv_smem_u32(own.buf + (size_t)(o & 1) * row), P.E + src0 + (size_t)o * lstride, (uint32_t)row * 4u,
                  bar);
  };
  if (TMA) {
    __shared__ int s_ol;
    if (threadIdx.x == 0) {
      s_ol = 0;
      adv_mbar_init(own.mbar);
      adv_mbar_init(own.mbar + 8u);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (lane == 0) atomicMax(&s_ol, OL);
    __syncthreads();
    OL = s_ol;
    if (threadIdx.x == 0) issue(0);
  }
  for (int o = 0; o < OL; ++o) {
    pf(o + PFD);
    if (TMA) {
      // this level's rows have landed (bounded: an error flag and a bounded
      // drain of the other buffer's copy instead of a hang)
      const bool ok = adv_mbar_wait(own.mbar + 8u * (o & 1), (o >> 1) & 1, 4000000000LL);
      if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) {
          atomicOr(&ctl->err, 2);
          if (o + 1 < OL) adv_mbar_wait(own.mbar + 8u * ((o + 1) & 1), ((o + 1) >> 1) & 1, 400000000LL);
        }
        return;
      }
      if (threadIdx.x == 0) {  // every thread is done with the other buffer
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(o + 1);
      }
    }
    if (o < O) {
      const float* r = Eb + (size_t)o * lstride;
      const float* rs = TMA ? own.buf + (size_t)(o & 1) * row + sS : r;
#pragma unroll
      for (int k = 0; k < H; ++k) ec[k] = rs[k * 32];  // E is also written (as ef) by the integration
      const bool prog = o < wi.oc;
      const Level<H> Lc = load_level<H>(prm, Tb + (size_t)o * tstride, !INTEG && prog);
      // the group's cos/sin 2th sign folded into the coefficients
      const float Bq = G == 4 ? c2s * B : B, Cq = G == 4 ? c2s * C : C;
      Cc.a = A; Cc.b = Bq; Cc.c = Cq;
      // PKI: pairs of directions (k, k+1) in packed f32x2 arithmetic; an
      // odd last direction takes the scalar form
      constexpr bool PKI = UMWM_INTEG_PACKED;
      constexpr int NPI = PKI ? H / 2 : 0;
      float s0 = 0.f, sc2 = 0.f, ss2 = 0.f;
      if constexpr (PKI) {  // even and odd directions summed apart
        float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0;
#pragma unroll
        for (int n = 0; n < NPI; ++n) {
          const float2 e = make_float2(ec[2 * n], ec[2 * n + 1]);
          a0 = __fadd2_rn(a0, e);
          a1 = __ffma2_rn(e, make_float2(prm.c2th[2 * n], prm.c2th[2 * n + 1]), a1);
          a2 = __ffma2_rn(e, make_float2(prm.s2th[2 * n], prm.s2th[2 * n + 1]), a2);
        }
        s0 = a0.x + a0.y;
        sc2 = a1.x + a1.y;
        ss2 = a2.x + a2.y;
      }
#pragma unroll
      for (int k = 2 * NPI; k < H; ++k) {
        s0 += ec[k];
        sc2 += ec[k] * prm.c2th[k];
        ss2 += ec[k] * prm.s2th[k];
      }
      if (G == 4) {
        sc2 *= c2s;
        ss2 *= c2s;
      }
#pragma unroll
      for (int m = PW; m < 32; m <<= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, m);
        sc2 += __shfl_xor_sync(0xffffffffu, sc2, m);
        ss2 += __shfl_xor_sync(0xffffffffu, ss2, m);
      }
      const float sA = prm.twopisds_fac * prm.f[o];
      // Sds = sA (1 + mss_fac chi)^2 (e k4)^sds_power, umwm_source_functions.F90:99-103,
      // with the level's factors in the exponent: 2^(p log2 e + p log2 k4 + log2 sA)
      const float lsk = fmaf(prm.sds_power, lg2a(Lc.k4), lg2a(sA));
      if (INTEG || prog) {
        if constexpr (PKI) {
          const float2 a2 = make_float2(A, A), b2 = make_float2(Bq, Bq), c2 = make_float2(Cq, Cq);
          const float2 mf = make_float2(prm.mss_fac, prm.mss_fac), one = make_float2(1.f, 1.f);
          const float2 pw = make_float2(prm.sds_power, prm.sds_power), lk = make_float2(lsk, lsk);
#pragma unroll
          for (int n = 0; n < NPI; ++n) {
            const int k = 2 * n;
            const float2 chi = __ffma2_rn(c2, make_float2(prm.s2th[k], prm.s2th[k + 1]),
                                          __ffma2_rn(b2, make_float2(prm.c2th[k], prm.c2th[k + 1]), a2));
            const float2 t = __ffma2_rn(mf, chi, one);
            const float2 x = __ffma2_rn(pw, make_float2(lg2a(ec[k]), lg2a(ec[k + 1])), lk);
            const float2 r = __fmul2_rn(__fmul2_rn(t, t), make_float2(ex2a(x.x), ex2a(x.y)));
            sc[k] = r.x;
            sc[k + 1] = r.y;
          }
        }
#pragma unroll
        for (int k = 2 * NPI; k < H; ++k) {
          const float chi = A + Bq * prm.c2th[k] + Cq * prm.s2th[k];
          const float t = 1.f + prm.mss_fac * chi;
          sc[k] = (t * t) * ex2a(fmaf(prm.sds_power, lg2a(ec[k]), lsk));
        }
      }
      if (!INTEG && prog) {
        const float U = wi.wspd + wi.ustar25 * Lc.logl2z;
        const float snl_arg = 1.f - (Lc.bf1r + Lc.bf2r);
        const float cs = Lc.cothkd * snl_arg;
        const float sink = Lc.sbf + sdtc * Lc.kk + Lc.sdv - (sv != 0.f ? 2.f * Lc.cg0 * sv : 0.f);
#pragma unroll
        for (int k = 0; k < H; ++k) {
          const float s = sin_k(prm, wi, U, CW(k), ucg * prm.cth[k], vcg * prm.sth[k], Lc.cp0,
                                Lc.fkovg, false);
          mx = fmaxf(mx, fabsf(s - sc[k] * cs - sink));
        }
        if (compute_rot) {
          const float* CP = P.TAB + (size_t)o * tstride + T_CP0 * 32;
          const float dcx = __ldg(CP + tidx(prm, 0, 0, nie)) - __ldg(CP + tidx(prm, 0, 0, niw));
          const float dcy = __ldg(CP + tidx(prm, 0, 0, nin)) - __ldg(CP + tidx(prm, 0, 0, nis));
          // the rotation rate 0.5 ((dcx sin th + vce - vcw) odx - (dcy cos th
          // + ucn - ucs) ody) in the group's frame, as ps sin th0 + pc cos th0
          // + p0 per direction (two multiply-adds)
          const float ps = 0.5f * (ra * dcx * odx + rb * dcy * ody), pc = 0.5f * (rb * dcx * odx - ra * dcy * ody);
          const float p0 = 0.5f * ((vce - vcw) * odx - (ucn - ucs) * ody);
#pragma unroll
          for (int k = 0; k < H; ++k) rmx = fmaxf(rmx, fmaf(ps, prm.sth[k], fmaf(pc, prm.cth[k], p0)));
        }
      }
      const float hk = Lc.k3dk * hdth;
      A += hk * s0; B += hk * sc2; C += hk * ss2;
    } else {
#pragma unroll
      for (int k = 0; k < H; ++k) { ec[k] = 0.f; sc[k] = 0.f; }
    }
    if (INTEG && o >= 2 && o < O + 2) {
      const int Lv = o - 2;
      const bool prog = Lv < wi.oc;
      const Level<H> L2 = load_level<H>(prm, Tb + (size_t)Lv * tstride, true);
      const float U = wi.wspd + wi.ustar25 * L2.logl2z;
      const float sdt = sdtc * L2.kk;
      const float sice = sv != 0.f ? 2.f * L2.cg0 * sv : 0.f;
      const float sinkL = ((L2.sbf + sdt) + L2.sdv) - sice;
      float* ES = P.ES + sidx(prm, 0, q * H, jj) + (size_t)Lv * lstride;
      float* EF = P.EF + sidx(prm, 0, q * H, jj) + (size_t)Lv * lstride;
      const size_t so = sidx(prm, 0, q * H, jj) + (size_t)Lv * lstride;  // saved source terms
      if (prog) {
        constexpr bool PKI = UMWM_INTEG_PACKED && !SAVE;
        constexpr int NPI = PKI ? H / 2 : 0;
        if constexpr (PKI) {
          // snl, the summed sinks and the exponential step of two directions
          const float2 b1 = make_float2(L2.bf1r, L2.bf1r), b2 = make_float2(L2.bf2r, L2.bf2r);
          const float2 nsf = make_float2(-prm.snl_fac, -prm.snl_fac), nct = make_float2(-L2.cothkd, -L2.cothkd);
          const float2 nsk = make_float2(-sinkL, -sinkL), dl = make_float2(dtsl2, dtsl2), dd = make_float2(dts, dts);
          const float2 half = make_float2(0.5f, 0.5f);
#pragma unroll
          for (int n = 0; n < NPI; ++n) {
            const int k = 2 * n;
            const float2 sn = sin_fold2(prm, wi.shelt, U, make_float2(CW(k), CW(k + 1)), ucg, vcg,
                                        make_float2(prm.cth[k], prm.cth[k + 1]), make_float2(prm.sth[k], prm.sth[k + 1]),
                                        L2.cp0, wi.c1 * L2.fkovg, false);
            const float2 pe2 = make_float2(LAG_E2(k), LAG_E2(k + 1)), ps2 = make_float2(LAG_S2(k), LAG_S2(k + 1));
            const float2 pe1 = make_float2(LAG_E1(k), LAG_E1(k + 1)), ps1 = make_float2(LAG_S1(k), LAG_S1(k + 1));
            float2 snl = __fmul2_rn(__fmul2_rn(b1, ps1), pe1);
            snl = __ffma2_rn(__fmul2_rn(b2, make_float2(sc[k], sc[k + 1])), make_float2(ec[k], ec[k + 1]), snl);
            snl = __ffma2_rn(__fmul2_rn(nsf, ps2), pe2, snl);
            const float2 S = __fadd2_rn(__ffma2_rn(ps2, nct, sn), nsk);
            const float2 x = __fmul2_rn(dl, S);
            const float2 ef = __ffma2_rn(pe2, make_float2(ex2a(x.x), ex2a(x.y)), __fmul2_rn(dd, snl));
            const float2 es = __fmul2_rn(half, __fadd2_rn(pe2, ef));
            if (valid) {
              ES[k * 32] = es.x;
              ES[(k + 1) * 32] = es.y;
            }
          }
        }
#pragma unroll
        for (int k = 2 * NPI; k < H; ++k) {
          const float s = sin_k(prm, wi, U, CW(k), ucg * prm.cth[k], vcg * prm.sth[k], L2.cp0,
                                L2.fkovg, false);
          const float e2k = LAG_E2(k), s2k = LAG_S2(k);
          const float snl = (L2.bf1r * LAG_S1(k)) * LAG_E1(k) + (L2.bf2r * sc[k]) * ec[k] - (prm.snl_fac * s2k) * e2k;
          // the level's sinks summed once: S = Sin - Sds coth - (sbf + sdt + sdv - sice)
          const float S = fmaf(-s2k, L2.cothkd, s) - sinkL;
          const float ef = e2k * ex2a(dtsl2 * S) + dts * snl;
          if (valid) {
            // only E*: e stays in place and the propagation forms ef = 2 E* - e
            ES[k * 32] = 0.5f * (e2k + ef);
            if (save) {
              P.src_sin[so + k * 32] = s;
              P.src_sds[so + k * 32] = s2k * L2.cothkd;
              P.src_snl[so + k * 32] = snl;
            }
          }
        }
      } else {
        // ef = (num / (sAc t^2 cothkd))^(1/p) / k^4, umwm_physics.F90:73-82, as
        // 2^((log2 num - 2 log2 t) / p + lt0) with the level's part lt0
        const float sAc = prm.twopisds_fac * prm.f[Lv];
        const float lt0 = -fmaf(prm.inv_sds_power, lg2a(sAc * L2.cothkd), lg2a(L2.k4));
        constexpr bool PKT = UMWM_INTEG_PACKED && !SAVE;
        constexpr int NPT = PKT ? H / 2 : 0;
        if constexpr (PKT) {  // two directions at a time, packed f32x2
          const float2 nk = make_float2(sice - sdt - L2.sdv, sice - sdt - L2.sdv);
          const float2 ca = make_float2(C2.a, C2.a), cb = make_float2(C2.b, C2.b), cc = make_float2(C2.c, C2.c);
          const float2 mf = make_float2(prm.mss_fac, prm.mss_fac), one = make_float2(1.f, 1.f);
          const float2 ip = make_float2(prm.inv_sds_power, prm.inv_sds_power), l0 = make_float2(lt0, lt0);
          const float2 m2 = make_float2(-2.f, -2.f), half = make_float2(0.5f, 0.5f);
#pragma unroll
          for (int n = 0; n < NPT; ++n) {
            const int k = 2 * n;
            const float2 sn = sin_fold2(prm, wi.shelt, U, make_float2(CW(k), CW(k + 1)), ucg, vcg,
                                        make_float2(prm.cth[k], prm.cth[k + 1]), make_float2(prm.sth[k], prm.sth[k + 1]),
                                        L2.cp0, wi.c1 * L2.fkovg, true);
            const float2 num = __fadd2_rn(sn, nk);
            const float2 chi = __ffma2_rn(cc, make_float2(prm.s2th[k], prm.s2th[k + 1]),
                                          __ffma2_rn(cb, make_float2(prm.c2th[k], prm.c2th[k + 1]), ca));
            const float2 t = __ffma2_rn(mf, chi, one);
            const float2 x = __ffma2_rn(ip, __ffma2_rn(m2, make_float2(lg2a(t.x), lg2a(t.y)),
                                                       make_float2(lg2a(num.x), lg2a(num.y))), l0);
            const float2 ef = make_float2(num.x >= 0.f ? ex2a(x.x) : 0.f, num.y >= 0.f ? ex2a(x.y) : 0.f);
            const float2 es = __fmul2_rn(half, __fadd2_rn(make_float2(LAG_E2(k), LAG_E2(k + 1)), ef));
            if (valid) {
              ES[k * 32] = es.x;
              ES[(k + 1) * 32] = es.y;
              EF[k * 32] = ef.x;
              EF[(k + 1) * 32] = ef.y;
            }
          }
        }
#pragma unroll
        for (int k = 2 * NPT; k < H; ++k) {
          const float s = sin_k(prm, wi, U, CW(k), ucg * prm.cth[k], vcg * prm.sth[k], L2.cp0,
                                L2.fkovg, true);
          const float num = s - sdt - L2.sdv + sice;
          float ef = 0.f;
          if (num >= 0.f) {
            const float chi = C2.a + C2.b * prm.c2th[k] + C2.c * prm.s2th[k];
            const float t = 1.f + prm.mss_fac * chi;
            ef = ex2a(fmaf(prm.inv_sds_power, fmaf(-2.f, lg2a(t), lg2a(num)), lt0));
          }
          if (valid) {
            ES[k * 32] = 0.5f * (LAG_E2(k) + ef);
            EF[k * 32] = ef;
            if (save) {
              P.src_sin[so + k * 32] = s;
              P.src_sds[so + k * 32] = LAG_S2(k) * L2.cothkd;
              P.src_snl[so + k * 32] = 0.f;  // snl is zero above the cut-off
            }
          }
        }
      }
    }

    if (INTEG) {
#pragma unroll
      for (int k = 0; k < H; ++k) {
        if (SL) {  // level o replaces level o-2, finished above
          lag[o & 1][0][SL ? k : 0][threadIdx.x] = ec[k];
          lag[o & 1][1][SL ? k : 0][threadIdx.x] = sc[k];
        } else {
          e2[SL ? 0 : k] = e1[SL ? 0 : k]; s2[SL ? 0 : k] = s1[SL ? 0 : k];
          e1[SL ? 0 : k] = ec[k]; s1[SL ? 0 : k] = sc[k];
        }
      }
      C2 = C1;
      C1 = Cc;
    }
  }

  if (!INTEG) {
#pragma unroll
    for (int m = PW; m < 32; m <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, m));
    float ph = prm.explim / mx;
    if (valid && q == 0) P.phys[j] = ph;
    float bm = valid ? ph : __int_as_float(0x7f800000);
#pragma unroll
    for (int s = PW / 2; s > 0; s >>= 1) bm = fminf(bm, __shfl_xor_sync(0xffffffffu, bm, s));
    if (lane == 0) atomicMin(&ctl->minphys_enc, enc_ord_d(bm));
    if (compute_rot) {
      float m = valid ? rmx : 0.f;
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
      if (lane == 0) atomicMax(&ctl->maxrot_enc, enc_ord_d(m));
    }
  }
}

}  // namespace umwm
