// Propagation, refraction, e = ef and stress('atm') in one pass
// (umwm_advection.F90:18-180, umwm_top.F90:113-115, umwm_stress.F90:17-264).
//
// Same thread mapping as the source kernels: G direction groups of H = pm/G
// directions per point, lane = point + (32/G) * q, group q is the base group
// turned by q*2pi/G (per-lane rotation ra, rb), so direction constants are
// those of the base group and known at compile time.
//
// Propagation.  cg0 > 0, so for an edge velocity cge = (cg0_i + cg0_ie) c,
// (cge + |cge|) = 2 (cg0_i + cg0_ie) max(c, 0) and (cge - |cge|) uses min(c, 0):
// the eight upwind terms of umwm_advection.F90:40-47 (and the current terms
// of :76-82) collapse to five coefficients times E* at the point and its four
// unrolled neighbours.  The half-turned group reads its neighbours in swapped
// slots (east for west, north for south), so the upwind weights of every
// group are the base group's compile-time max/min(cos th0, 0) and
// max/min(sin th0, 0).  The east/west neighbours sit about one wet column
// (~nm points) away and are served from L2, which holds the window of blocks
// the CTAs in flight work on; each lane copies the next level's east/west
// rows into shared memory (cp.async) once this level's propagation has read
// its own, so they arrive while the refraction and the stress run.
// Refraction needs E* at p-1 and p+1: inside a group they are registers, at
// the group's edges they come from the neighbouring groups' lanes (shuffle).  The rotation
// rate is recomputed from cp0 and the currents (it depends on no spectral
// value); when the reference would reuse the rotation of an earlier substep
// (currents = .F.) the mask o <= oc of that substep is kept in oc_rot.
// The wind stress sums e*Sin*cos/sin(th)/cp over the new spectrum while it is
// in registers; group 0 then finishes the drag, skin stress and ustar.
#include "kernels.hpp"
#include "adv_body.cuh"

namespace umwm {

// k_advect: one CTA per tile (blockIdx.x), register budget for MINB
// resident CTAs per SM; CNT counts the non-negativity cut.
template <int G, int H, bool CURV, int MINB, bool CNT = false>
__global__ void __launch_bounds__(128, MINB) k_advect(const Params prm, const Ptrs P) {
  __shared__ AdvSmem<G, H, CURV> sm;
  advect_body<G, H, CURV, CNT, false>(prm, P, blockIdx.x, sm);
}

// k_advect_tma: the same body with each level's own rows staged in shared
// memory by bulk copies (OwnStage), for the two-group plain-grid mapping.
// TM 1: the E* and e rows, 64.9 KB of shared memory per CTA, 3 CTAs per SM;
// TM 2: the E* rows only, 47.1 KB, 4 CTAs per SM (128 registers).
template <int G, int H, int TM>
__global__ void __launch_bounds__(128, TM == 1 ? 3 : 4) k_advect_tma(const Params prm, const Ptrs P) {
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ __align__(8) unsigned long long mbar[2];
  auto& sm = *reinterpret_cast<AdvSmem<G, H, false>*>(dsm);
  constexpr size_t off = (sizeof(AdvSmem<G, H, false>) + 127) & ~size_t(127);
  const OwnStage own{reinterpret_cast<float*>(dsm + off), adv_smem_u32(mbar)};
  advect_body<G, H, false, false, false, TM>(prm, P, blockIdx.x, sm, own);
}

// shared memory of k_advect_tma<2, H, TM>: the AdvSmem and two buffers of
// one or two arrays (TM 2 or 1) of the CTA's two blocks
template <int H>
constexpr size_t tma_smem_bytes(int pm, int tm) {
  return ((sizeof(AdvSmem<2, H, false>) + 127) & ~size_t(127)) + (size_t)2 * (tm == 1 ? 2 : 1) * 2 * pm * 32 * 4;
}

// Launch with the register budget of `minb` resident CTAs per SM (tuned
// instances for the 36-direction mappings on plain grids; the default
// instance otherwise).
template <int G, int H, bool CURV>
static void launch_adv(int minb, dim3 grid, const Params& prm, const Ptrs& P, cudaStream_t st) {
  const dim3 block(128);
#define INST(B)                                                  \
  case B:                                                        \
    k_advect<G, H, CURV, B><<<grid, block, 0, st>>>(prm, P);     \
    return;
  if constexpr (G * H == 36) {
    if (prm.count_cut) {
      k_advect<G, H, CURV, G == 4 ? UMWM_ADVECT_MINB4 : UMWM_ADVECT_MINB, true><<<grid, block, 0, st>>>(prm, P);
      return;
    }
  }
  if constexpr (!CURV && G == 2 && H == 18 && UMWM_ADVECT_HALVES > 1) {  // the staged form takes rows in halves
    if (prm.adv_tma == 1) {
      const size_t smem = tma_smem_bytes<18>(prm.P, 1);
      static const cudaError_t attr =
          cudaFuncSetAttribute(k_advect_tma<2, 18, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (attr == cudaSuccess) {
        k_advect_tma<2, 18, 1><<<grid, block, smem, st>>>(prm, P);
        return;
      }
    } else if (prm.adv_tma == 2) {
      const size_t smem = tma_smem_bytes<18>(prm.P, 2);
      static const cudaError_t attr =
          cudaFuncSetAttribute(k_advect_tma<2, 18, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (attr == cudaSuccess) {
        k_advect_tma<2, 18, 2><<<grid, block, smem, st>>>(prm, P);
        return;
      }
    }
  }
  if constexpr (!CURV && G * H == 36) {
    switch (minb) { INST(3) INST(4) INST(5) default: break; }
  }
#undef INST
  k_advect<G, H, CURV, G == 4 ? UMWM_ADVECT_MINB4 : UMWM_ADVECT_MINB><<<grid, block, 0, st>>>(prm, P);
}

cudaError_t launch_advect(const Params& prm, const Ptrs& P, cudaStream_t st) {
  const bool curv = prm.curvilinear != 0;
  const int minb = prm.minb_adv;
  if (prm.adv_groups4 && quarter_groups(prm.P)) {
    const dim3 grid(prm.ntiles * (TILE / 32));  // 32 points per CTA
    switch (prm.P / 4) {
#define CASE(X)                                                          \
  case X:                                                                \
    if (curv) launch_adv<4, X, true>(minb, grid, prm, P, st);            \
    else launch_adv<4, X, false>(minb, grid, prm, P, st);                \
    break;
      CASE(4) CASE(6) CASE(8) CASE(9) CASE(12)
#undef CASE
      default: return cudaErrorInvalidConfiguration;
    }
    return cudaGetLastError();
  }
  const dim3 grid(prm.ntiles);  // 64 points per CTA
  switch (prm.P / 2) {
#define CASE(X)                                                          \
  case X:                                                                \
    if (curv) launch_adv<2, X, true>(minb, grid, prm, P, st);            \
    else launch_adv<2, X, false>(minb, grid, prm, P, st);                \
    break;
    CASE(4) CASE(6) CASE(8) CASE(12) CASE(16) CASE(18) CASE(24)
#undef CASE
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

}  // namespace umwm
