// Device bodies of the per-substep control kernels (forcing interpolation,
// dts/dtr, sea-ice Hs, screen line), shared by their per-stage kernels in
// k_misc.cu and the persistent substep kernel.
#pragma once
#include <cfloat>

#include "dev_common.cuh"

namespace umwm {

// The cut-off index oc: the largest o <= O - 2 with f(o) < fc (1-based f),
// else 1 (umwm_source_functions.F90:25-36), by bisection over the
// increasing frequencies (the same index as the reference's downward scan)
__device__ __forceinline__ int cutoff_level(const Params& prm, float fc) {
  int a = -1, b = prm.O - 3;  // 0-based: the largest i in [0, O - 3] with f[i] < fc, or -1
  while (a < b) {
    const int m = (a + b + 1) >> 1;
    if (prm.f[m] < fc) a = m;
    else b = m - 1;
  }
  return a >= 0 ? a + 1 : 1;
}

// ctl->anycurrent = 1 where cur holds, one store per warp (every lane of
// the warp's active set calls this)
__device__ __forceinline__ void set_anycurrent(Ctl* ctl, bool cur) {
  const unsigned act = __activemask();
  if (__any_sync(act, cur) && (threadIdx.x & 31) == __ffs(act) - 1) ctl->anycurrent = 1;
}

// One all-point index i of member M (its forcing interpolation at sumt; for
// wet points also oc, oc_rot and the sheltering coefficient): the per-stage
// kernel's form, one point per thread (0.13 ms at 1000x1000, against 0.27
// measured for prep_points<1>, which takes 40 registers instead of 30).
// prep_points below computes the same values by the same expressions.
__device__ __forceinline__ void prep_point(const Params& prm, const Ptrs& P, const Member& M, Ctl* ctl, int i,
                                           int compute_rot) {
  const float sumt = ctl->sumt, dtg = prm.dtg;
  const float a = 1.f - sumt / dtg;
  const int q = (M.mi[i] - 1) + (M.ni[i] - 1) * M.mm;
  const int ia = M.nmoff + i;
  if (prm.winds) {
    float uw = M.uwb[q] * a + M.uwf[q] * sumt / dtg;
    float vw = M.vwb[q] * a + M.vwf[q] * sumt / dtg;
    if (prm.gustiness > 0.f) {  // umwm_forcing.F90:49-61
      const float gu = prm.gustiness * (2.f * gust_uniform(prm.gust_seed, ctl->substep, q, 0) - 1.f);
      const float gv = prm.gustiness * (2.f * gust_uniform(prm.gust_seed, ctl->substep, q, 1) - 1.f);
      uw = uw * (1.f + gu);
      vw = vw * (1.f + gv);
    }
    P.wspd[ia] = sqrtf(uw * uw + vw * vw);
    P.wdir[ia] = atan2f(vw, uw);
  }
  if (prm.seaice) P.fice[ia] = M.ficeb[q] * a + M.ficef[q] * sumt / dtg;
  if (prm.currents) {
    P.uc[ia] = M.ucb[q] * a + M.ucf[q] * sumt / dtg;
    P.vc[ia] = M.vcb[q] * a + M.vcf[q] * sumt / dtg;
  }
  if (prm.air_density) P.rhoa[ia] = M.rhoab[q] * a + M.rhoaf[q] * sumt / dtg;
  if (prm.water_density) P.rhow[ia] = M.rhowb[q] * a + M.rhowf[q] * sumt / dtg;
  P.rhorat[ia] = P.rhoa[ia] / P.rhow[ia];
  const float ws = fmaxf(P.wspd[ia], 1e-2f);
  P.wspd[ia] = ws;
  set_anycurrent(ctl, (prm.isglobal || i < M.N) && (P.uc[ia] != 0.f || P.vc[ia] != 0.f));
  if (i < M.N) {
    const int j = M.off + i;
    float fc = 0.53f * prm.g / ws;
    if (fc > prm.fprog) fc = prm.fprog;
    P.fcutoff[j] = fc;
    const int oc = cutoff_level(prm, fc);
    P.oc[j] = oc;
    if (compute_rot) P.oc_rot[j] = oc;
    P.shelt[j] = shelter_coare35(ws);
  }
}

// The same in two halves, for a thread that takes several points (the
// persistent kernel): prep_load issues every load of a point, prep_finish
// computes and stores, and prep_points loads all its points before it
// stores any, so their memory latencies overlap.
struct PrepIn {
  int q;
  float w[4];   // uwb, uwf, vwb, vwf; or w[0] = wspd when the winds are fixed
  float fi[2];  // ficeb, ficef
  float c[4];   // ucb, ucf, vcb, vcf; or c[0], c[1] = uc, vc when fixed
  float ra[2];  // rhoab, rhoaf; or ra[0] = rhoa when fixed
  float rw[2];  // rhowb, rhowf; or rw[0] = rhow when fixed
};

__device__ __forceinline__ PrepIn prep_load(const Params& prm, const Ptrs& P, const Member& M, int i) {
  PrepIn in;
  in.q = (M.mi[i] - 1) + (M.ni[i] - 1) * M.mm;
  const int q = in.q, ia = M.nmoff + i;
  if (prm.winds) {
    in.w[0] = M.uwb[q], in.w[1] = M.uwf[q], in.w[2] = M.vwb[q], in.w[3] = M.vwf[q];
  } else {
    in.w[0] = P.wspd[ia];
  }
  if (prm.seaice) in.fi[0] = M.ficeb[q], in.fi[1] = M.ficef[q];
  if (prm.currents) {
    in.c[0] = M.ucb[q], in.c[1] = M.ucf[q], in.c[2] = M.vcb[q], in.c[3] = M.vcf[q];
  } else {
    in.c[0] = P.uc[ia], in.c[1] = P.vc[ia];
  }
  if (prm.air_density) in.ra[0] = M.rhoab[q], in.ra[1] = M.rhoaf[q];
  else in.ra[0] = P.rhoa[ia];
  if (prm.water_density) in.rw[0] = M.rhowb[q], in.rw[1] = M.rhowf[q];
  else in.rw[0] = P.rhow[ia];
  return in;
}

__device__ __forceinline__ void prep_finish(const Params& prm, const Ptrs& P, const Member& M, Ctl* ctl, int i,
                                            const PrepIn& in, int compute_rot) {
  const float sumt = ctl->sumt, dtg = prm.dtg;
  const float a = 1.f - sumt / dtg;
  const int q = in.q;
  const int ia = M.nmoff + i;
  float wspd = in.w[0];
  if (prm.winds) {
    float uw = in.w[0] * a + in.w[1] * sumt / dtg;
    float vw = in.w[2] * a + in.w[3] * sumt / dtg;
    if (prm.gustiness > 0.f) {  // umwm_forcing.F90:49-61
      const float gu = prm.gustiness * (2.f * gust_uniform(prm.gust_seed, ctl->substep, q, 0) - 1.f);
      const float gv = prm.gustiness * (2.f * gust_uniform(prm.gust_seed, ctl->substep, q, 1) - 1.f);
      uw = uw * (1.f + gu);
      vw = vw * (1.f + gv);
    }
    wspd = sqrtf(uw * uw + vw * vw);
    P.wdir[ia] = atan2f(vw, uw);
  }
  if (prm.seaice) P.fice[ia] = in.fi[0] * a + in.fi[1] * sumt / dtg;
  float uc = in.c[0], vc = in.c[1];
  if (prm.currents) {
    uc = in.c[0] * a + in.c[1] * sumt / dtg;
    vc = in.c[2] * a + in.c[3] * sumt / dtg;
    P.uc[ia] = uc;
    P.vc[ia] = vc;
  }
  float rhoa = in.ra[0], rhow = in.rw[0];
  if (prm.air_density) P.rhoa[ia] = rhoa = in.ra[0] * a + in.ra[1] * sumt / dtg;
  if (prm.water_density) P.rhow[ia] = rhow = in.rw[0] * a + in.rw[1] * sumt / dtg;
  P.rhorat[ia] = rhoa / rhow;
  const float ws = fmaxf(wspd, 1e-2f);
  P.wspd[ia] = ws;
  set_anycurrent(ctl, (prm.isglobal || i < M.N) && (uc != 0.f || vc != 0.f));
  if (i < M.N) {
    const int j = M.off + i;
    float fc = 0.53f * prm.g / ws;
    if (fc > prm.fprog) fc = prm.fprog;
    P.fcutoff[j] = fc;
    const int oc = cutoff_level(prm, fc);
    P.oc[j] = oc;
    if (compute_rot) P.oc_rot[j] = oc;
    P.shelt[j] = shelter_coare35(ws);
  }
}

// Points i0, i0 + stride, ... (U of them, those below M.NM) of one thread.
template <int U>
__device__ __forceinline__ void prep_points(const Params& prm, const Ptrs& P, const Member& M, Ctl* ctl, int i0,
                                            int stride, int compute_rot) {
  PrepIn in[U];
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (i0 + u * stride < M.NM) in[u] = prep_load(prm, P, M, i0 + u * stride);
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (i0 + u * stride < M.NM) prep_finish(prm, P, M, ctl, i0 + u * stride, in[u], compute_rot);
}

// source(): dts = min(min_i physics_time_step, dtamin, dtg - sumt), the
// first-step rule and sumt update (umwm_physics.F90:41-58); refraction's
// dtr (umwm_advection.F90:145-158).  One block, members over its threads.
__device__ __forceinline__ void dts_body(const Params& prm, const Ptrs& P, int compute_rot, int first) {
  int left = 0;
  for (int m = threadIdx.x; m < prm.nmem; m += blockDim.x) {
    const Member& M = prm.mem[m];
    Ctl& c = *M.ctl;
    if (c.done) {  // finished this dtg in an earlier substep
      c.running = 0;
      continue;
    }
    float mn = dec_ord_d(c.minphys_enc);
    float dts = fminf(fminf(mn, M.dtamin), prm.dtg - c.sumt);
    if (!prm.restart && first) dts = 0.f;
    c.dts = dts;
    c.dta = dts;
    c.sumt = c.sumt + dts;
    if (compute_rot) {
      float mx = dec_ord_d(c.maxrot_enc);
      c.dtr_temp = (mx <= FLT_MIN) ? dts : prm.dth / mx;
    }
    c.dtr = fminf(c.dtr_temp, dts);
    c.zerocurrents = c.anycurrent ? 0 : 1;
    c.anycurrent = 0;
    c.minphys_enc = enc_ord_d(__int_as_float(0x7f800000));
    c.maxrot_enc = enc_ord_d(0.f);
    c.done = (c.sumt < prm.dtg) ? 0 : 1;
    c.running = 1;
    c.first = first;
    left += !c.done;
  }
  left = __syncthreads_count(left > 0) ? 1 : 0;  // any member left in this block
  if (threadIdx.x == 0) P.glob->not_done = left;
}

// s_ice for wet point j: significant wave height where fice > fice_lth and
// the attenuation factor (umwm_source_functions.F90:108-153).
__device__ __forceinline__ void sice_point(const Params& prm, const Ptrs& P, int j) {
  const Member& M = prm.mem[prm.tile_mem[j / TILE]];
  if (j >= M.ghost || M.ctl->done) return;
  float sv = 0.f;
  if (P.fice[apt(M, j)] > prm.fice_lth) {
    float h = 0.f;
    for (int p = 0; p < prm.P; ++p)
      for (int o = 0; o < prm.O; ++o)
        h += P.E[sidx(prm, o, p, j)] * P.TAB[tidx(prm, o, T_KDK, j)];
    h = 4.f * sqrtf(h * prm.dth);
    const float C1 = -5.35e-6f;
    sv = (h < 3.f) ? C1 * h : C1 * 3.f;
  }
  P.sice_v[j] = sv;
}

// Screen line of member m at its print point (umwm_top.F90:143-148,
// umwm_util.F90:69-124); also clears 'first' and counts the substep.  The
// sums run over V virtual threads (bins strided by V, then a tree
// reduction), carried by the NT <= V threads of the block, so that any NT
// gives the same result bit for bit.
template <int V, int NT>
__device__ __forceinline__ void screen_member(const Params& prm, const Ptrs& P, int m, float (&s0)[V],
                                              float (&s2)[V]) {
  static_assert(V % NT == 0, "virtual threads must be a multiple of the block");
  const Member& M = prm.mem[m];
  Ctl& c = *M.ctl;
  if (!c.running) return;
  const int j = M.iip;
  for (int v = threadIdx.x; v < V; v += NT) {
    float a = 0.f, b = 0.f;
    if (j >= 0) {
      for (int b_ = v; b_ < prm.O * prm.P; b_ += V) {
        const int o = b_ / prm.P, p = b_ % prm.P;
        const float ek = P.E[sidx(prm, o, p, j)] * P.TAB[tidx(prm, o, T_KDK, j)];
        a += ek;
        b += (prm.f[o] * prm.f[o]) * ek;
      }
    }
    s0[v] = a;
    s2[v] = b;
  }
  __syncthreads();
  for (int s = V / 2; s > 0; s >>= 1) {
    for (int v = threadIdx.x; v < s; v += NT) { s0[v] += s0[v + s]; s2[v] += s2[v + s]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int r = c.log_count;
    if (r < M.log_cap && j >= 0) {
      double* L = M.log + (size_t)r * 8;
      const int ja = apt(M, j);
      L[0] = c.sumt / prm.dtg;
      L[1] = c.dts;
      L[2] = P.wspd[ja];
      L[3] = P.wdir[ja];
      L[4] = 4.f * sqrtf(s0[0] * prm.dth);
      L[5] = sqrtf(s0[0] / s2[0]);
      L[6] = P.cd[j] * 1e3f;
      L[7] = prm.f[P.oc[j] - 1];
      c.log_count = r + 1;
    }
    c.substep += 1;
    c.first = 0;
  }
}

}  // namespace umwm
