// Source-term kernels: sin_d12, sds_d12, snl_d12, s_ice and source()
// (umwm_source_functions.F90:16-183, umwm_physics.F90:9-86).
//
// Thread mapping.  The pm directions of a point are split into G groups of
// H = pm/G consecutive directions (G = 4 when pm/4 is a supported group size,
// else G = 2); a warp owns 32/G consecutive wet points and lane = point +
// (32/G) * q, where group q takes directions p = qH .. qH+H-1.  Group q is the
// base group 0 turned by q*2pi/G (a quarter turn for G = 4, a half turn for
// G = 2), so every group runs the same code with the direction index
// k = 0..H-1 known at compile time (every direction constant of the base
// group is a constant-bank operand) and a per-lane rotation (ra, rb):
// cos th = ra cos th0 - rb sin th0, sin th = rb cos th0 + ra sin th0, and
// cos/sin 2th pick up the sign cos(2 q 2pi/G).  The groups of a point combine
// their partial sums with log2(G) shuffles.
//
// The frequency loop walks o = 1..om in order because the mean-square-slope
// adjustment of Sds is a prefix over o:
//   dummy(o,p) = dummy(o-1,p) + k3dk(o-1) * sum_pp e(o-1,pp) cth2pp(pp,p),
//   cth2pp(pp,p) = cos^2(th(pp)-th(p)) dth
//                = dth/2 (1 + cos2th(pp)cos2th(p) + sin2th(pp)sin2th(p)),
// so dummy(o,.) = A + B cos2th(p) + C sin2th(p) with three running sums per
// point (exact algebra; two multiply-adds per bin instead of pm).
// Snl at level o needs Sds*e at o+1 and o+2, so the integration finishes
// level o two levels after it was loaded (registers hold two levels of e and
// Sds per direction).  Upcoming levels are prefetched into L2.
//
// MODE_PHYS : per-point max |exponent argument| -> physics_time_step and the
//             global min for dts (umwm_physics.F90:18-41); with compute_rot
//             also the global max of the rotation rate for refraction's dtr
//             (umwm_advection.F90:125-154).
// MODE_INTEG: exponential integration (o <= oc), equilibrium tail (o > oc),
//             E* = (e + ef)/2 -> ES (umwm_physics.F90:61-84); ef -> EF (= E)
//             above the cut-off only: below it e stays and the propagation
//             forms ef = 2 E* - e, which saves a spectrum write per substep.
#include "kernels.hpp"
#include "src_body.cuh"

namespace umwm {

// Resident CTAs per SM the register budget of each instance is sized for
// when no tuned value applies.
template <int G, int H, bool INTEG>
constexpr int default_minb() {
  return G == 4 ? (INTEG ? 4 : 5) : (INTEG ? (UMWM_INTEG_SMEM_LAGS && H <= 18 ? UMWM_INTEG_MINB : 3) : UMWM_PHYS_MINB);
}

template <int G, int H, bool INTEG, int MINB>
__global__ void __launch_bounds__(128, MINB) k_source(const Params prm, const Ptrs P, int compute_rot) {
  __shared__ SrcSmem<G, H, INTEG> sm;
  if (INTEG && P.src_sin) {
    // the last substep of a step that computes stress('ocn') or writes output
    // keeps its source terms, and so does the model's first substep (its
    // spectrum output)
    const Ctl* ctl = prm.mem[prm.tile_mem[(blockIdx.x * (4 * 32 / G)) / TILE]].ctl;
    if ((ctl->done || ctl->first) && P.glob->save_src) {
      source_body<G, H, INTEG, true>(prm, P, compute_rot, blockIdx.x, sm);
      return;
    }
  }
  source_body<G, H, INTEG, false>(prm, P, compute_rot, blockIdx.x, sm);
}

// k_source_tma: the dts pre-pass with its own e rows staged in shared memory
// by bulk copies (OwnStage), for the two-group mapping; 5 CTAs per SM.
template <int G, int H>
__global__ void __launch_bounds__(128, 5) k_source_tma(const Params prm, const Ptrs P, int compute_rot) {
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ __align__(8) unsigned long long mbar[2];
  auto& sm = *reinterpret_cast<SrcSmem<G, H, false>*>(dsm);
  constexpr size_t off = (sizeof(SrcSmem<G, H, false>) + 127) & ~size_t(127);
  const OwnStage own{reinterpret_cast<float*>(dsm + off), adv_smem_u32(mbar)};
  source_body<G, H, false, false, true>(prm, P, compute_rot, blockIdx.x, sm, own);
}

// Launch with the register budget of `minb` resident CTAs per SM.  The
// 36-direction mappings (the configured workloads) have instances for the
// budgets the autotuner tries (the integration's shared memory allows at
// most 4 CTAs of the two-group mapping); other budgets and direction counts
// use the default instance.
template <int G, int H, bool INTEG>
static void launch_src(int minb, dim3 grid, const Params& prm, const Ptrs& P, int compute_rot, cudaStream_t st) {
  const dim3 block(128);
#define INST(B)                                                              \
  case B:                                                                    \
    k_source<G, H, INTEG, B><<<grid, block, 0, st>>>(prm, P, compute_rot);   \
    return;
  if constexpr (G == 2 && H == 18 && INTEG) {
    switch (minb) { INST(3) INST(4) default: break; }
  } else if constexpr (G == 2 && H == 18) {
    if (prm.phys_tma) {
      const size_t smem = ((sizeof(SrcSmem<2, 18, false>) + 127) & ~size_t(127)) + (size_t)2 * 2 * prm.P * 32 * 4;
      static const cudaError_t attr =
          cudaFuncSetAttribute(k_source_tma<2, 18>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (attr == cudaSuccess) {
        k_source_tma<2, 18><<<grid, block, smem, st>>>(prm, P, compute_rot);
        return;
      }
    }
    switch (minb) { INST(5) INST(6) INST(7) default: break; }
  } else if constexpr (G == 4 && H == 9) {
    switch (minb) { INST(3) INST(4) INST(5) INST(6) default: break; }
  }
#undef INST
  k_source<G, H, INTEG, default_minb<G, H, INTEG>()><<<grid, block, 0, st>>>(prm, P, compute_rot);
}

template <bool INTEG>
static cudaError_t launch_source_t(const Params& prm, const Ptrs& P, int compute_rot, cudaStream_t st) {
  const int minb = INTEG ? prm.minb_integ : prm.minb_phys;
  if ((INTEG ? prm.groups4 : prm.groups4_phys) && quarter_groups(prm.P)) {
    const dim3 grid(prm.ntiles * (TILE / 32));  // 32 points per CTA
    switch (prm.P / 4) {
#define CASE(X) \
  case X: launch_src<4, X, INTEG>(minb, grid, prm, P, compute_rot, st); break;
      CASE(4) CASE(6) CASE(8) CASE(9) CASE(12)
#undef CASE
      default: return cudaErrorInvalidConfiguration;
    }
    return cudaGetLastError();
  }
  const dim3 grid(prm.ntiles);  // 64 points per CTA
  switch (prm.P / 2) {
#define CASE(X) \
  case X: launch_src<2, X, INTEG>(minb, grid, prm, P, compute_rot, st); break;
    CASE(4) CASE(6) CASE(8) CASE(12) CASE(16) CASE(18) CASE(24)
#undef CASE
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

cudaError_t launch_source_phys(const Params& prm, const Ptrs& P, int compute_rot, cudaStream_t st) {
  return launch_source_t<false>(prm, P, compute_rot, st);
}
cudaError_t launch_source_integ(const Params& prm, const Ptrs& P, cudaStream_t st) {
  return launch_source_t<true>(prm, P, 0, st);
}
bool supported_pm(int pm) {
  const int h = pm / 2;
  return pm % 4 == 0 && (h == 4 || h == 6 || h == 8 || h == 12 || h == 16 || h == 18 || h == 24);
}

}  // namespace umwm
