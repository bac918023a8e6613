// Persistent substep kernel: the inner dynamic-dts loop of umwm_run
// (umwm_top.F90:97-150) for every member of a model in one cooperative
// launch.  Each CTA loops over substeps; within a substep it takes the
// stages in order (forcing interpolation, [sea-ice Hs], the dts pre-pass,
// dts, the integration, propagation + refraction + stress, the screen line),
// working through the stage's tiles grid-stride, with a grid-wide barrier
// between stages.  The stage bodies are those of the per-stage kernels
// (src_body.cuh, adv_body.cuh, misc_body.cuh); the propagation reads E*
// with coherent loads, since the same launch wrote it.  The loop ends when no
// member is left inside the dtg or the armed substep budget is spent.
//
// Every barrier wait is bounded (a globaltimer limit); a wait that runs out
// sets Global::bar_err and its CTA returns, and so does every CTA at its next
// barrier, so the launch always ends and the host reports UMWM_ERR_TIMEOUT.
// All CTAs are co-resident (cooperative launch, grid sized from the occupancy
// of this kernel), which is what the barrier needs.
#include <algorithm>

#include "adv_body.cuh"
#include "kernels.hpp"
#include "misc_body.cuh"
#include "src_body.cuh"

namespace umwm {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier over `expected` CTAs with a bounded wait.  Returns false
// (in every thread of the CTA) when this or an earlier wait gave up.
__device__ __forceinline__ bool grid_barrier(Global* g, unsigned expected, unsigned long long limit_ns, int* ok_s) {
  __syncthreads();  // this CTA's stage work is done
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* genp = &g->bar_gen;
    const unsigned gen = *genp;
    __threadfence();  // release this CTA's writes before arriving
    if (atomicAdd(&g->bar_count, 1u) == expected - 1) {
      atomicExch(&g->bar_count, 0u);
      __threadfence();
      atomicAdd(&g->bar_gen, 1u);
    } else {
      const unsigned long long t0 = globaltimer_ns();
      while (*genp == gen) {
        if (globaltimer_ns() - t0 > limit_ns) {
          atomicExch(&g->bar_err, 1);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();  // acquire the other CTAs' writes
    *ok_s = ok && *(volatile int*)&g->bar_err == 0;
  }
  __syncthreads();
  return *ok_s != 0;
}

// The forcing interpolation of every member still inside the dtg, PREP_U
// points per thread with their loads first (prep_points).  Measured on the
// 1000x1000 random field (ms per substep, forcing / propagation / whole
// substep): one point per thread 0.53 / 6.90 / 11.71; four points 0.20 /
// 7.45 / 12.05 inlined and 0.20 / 7.51 / 12.40 as a separate function (the
// larger register demand of the forcing stage costs the propagation more
// than it saves).
#ifndef UMWM_PERSIST_PREP_U
#define UMWM_PERSIST_PREP_U 1
#endif
__device__ __forceinline__ void forcing_stage(const Params& prm, const Ptrs& P, int nb, int compute_rot) {
  constexpr int U = UMWM_PERSIST_PREP_U;
  for (int m = 0; m < prm.nmem; ++m) {
    const Member& M = prm.mem[m];
    Ctl* ctl = M.ctl;
    if (ctl->done) continue;
    for (int i = blockIdx.x * 128 + threadIdx.x; i < M.NM; i += U * nb * 128)
      prep_points<U>(prm, P, M, ctl, i, nb * 128, compute_rot);
  }
}

template <int G, int H, bool CURV>
union PersistSmem {
  SrcSmem<G, H, false> phys;
  SrcSmem<G, H, true> integ;
  AdvSmem<G, H, CURV> adv;
  float scr[2][256];
};

template <int G, int H, bool CURV>
#ifndef UMWM_PERSIST_MINB
#define UMWM_PERSIST_MINB 4  // resident CTAs per SM (3, at 168 registers: 12.42 ms per substep against 11.71)
#endif
__global__ void __launch_bounds__(128, UMWM_PERSIST_MINB)
    k_persist(const Params prm, const Ptrs P, unsigned expected, unsigned long long limit_ns) {
  __shared__ PersistSmem<G, H, CURV> sm;
  __shared__ int ok_s;
  constexpr int PPC = 4 * (32 / G);  // points of a spectral CTA tile
  const int nvb = prm.Ntot / PPC;
  const int nb = gridDim.x;
  const int compute_rot = prm.currents;
  Global* gl = P.glob;
  // each barrier ends a stage; block 0 books the stage's time
  unsigned long long t_last = globaltimer_ns();
  auto bar_s = [&](int stage) {
    const bool ok = grid_barrier(gl, expected, limit_ns, &ok_s);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      const unsigned long long t = globaltimer_ns();
      gl->stage_ns[stage] += t - t_last;
      t_last = t;
    }
    return ok;
  };
  const int budget = gl->budget;  // armed before the launch (k_loop_arm)
  for (int it = 0; it < budget; ++it) {
    forcing_stage(prm, P, nb, compute_rot);
    if (!bar_s(0)) return;
    if (prm.ice_possible) {
      for (int j = blockIdx.x * 128 + threadIdx.x; j < prm.Ntot; j += nb * 128) sice_point(prm, P, j);
      if (!bar_s(1)) return;
    }
    for (int v = blockIdx.x; v < nvb; v += nb) source_body<G, H, false, false>(prm, P, compute_rot, v, sm.phys);
    if (!bar_s(2)) return;
    if (blockIdx.x == 0) dts_body(prm, P, compute_rot, 0);
    if (!bar_s(3)) return;
    for (int v = blockIdx.x; v < nvb; v += nb) {
      const Ctl* ctl = prm.mem[prm.tile_mem[(v * PPC) / TILE]].ctl;
      if (P.src_sin && (ctl->done || ctl->first) && gl->save_src)
        source_body<G, H, true, true>(prm, P, 0, v, sm.integ);
      else
        source_body<G, H, true, false>(prm, P, 0, v, sm.integ);
    }
    if (!bar_s(4)) return;
    for (int v = blockIdx.x; v < nvb; v += nb) advect_body<G, H, CURV, false, true>(prm, P, v, sm.adv);
    if (!bar_s(5)) return;
    for (int m = blockIdx.x; m < prm.nmem; m += nb) screen_member<256, 128>(prm, P, m, sm.scr[0], sm.scr[1]);
    if (blockIdx.x == 0 && threadIdx.x == 0) gl->iters += 1;
    if (!bar_s(6)) return;
    // not_done was set by this substep's dts, two barriers ago
    if (*(volatile int*)&gl->not_done == 0) break;
  }
}

// reset of the barrier before a launch
__global__ void k_persist_arm(Global* g) {
  g->bar_count = 0;
  g->bar_gen = 0;
  g->bar_err = 0;
}

template <int G, int H, bool CURV>
static cudaError_t launch_persist_t(const Params& prm, const Ptrs& P, int stall_test, cudaStream_t st) {
  int dev = 0, nsm = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persist<G, H, CURV>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorLaunchOutOfResources;
  constexpr int PPC = 4 * (32 / G);
  const unsigned grid = (unsigned)std::max(1, std::min(nsm * per_sm, prm.Ntot / PPC));
  // the barrier expects one CTA more than launched when the stall test is
  // armed: every wait then runs out after 20 ms
  const unsigned expected = grid + (stall_test ? 1u : 0u);
  const unsigned long long limit_ns = stall_test ? 20000000ull : 2000000000ull;
  k_persist_arm<<<1, 1, 0, st>>>(P.glob);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  void* args[] = {(void*)&prm, (void*)&P, (void*)&expected, (void*)&limit_ns};
  return cudaLaunchCooperativeKernel((const void*)k_persist<G, H, CURV>, dim3(grid), dim3(128), args, 0, st);
}

bool persist_supported(const Params& prm) {
  return prm.P == 36 && prm.groups4 == prm.groups4_phys && prm.groups4 == prm.adv_groups4;
}

cudaError_t launch_persist(const Params& prm, const Ptrs& P, int stall_test, cudaStream_t st) {
  if (!persist_supported(prm)) return cudaErrorInvalidConfiguration;
  const bool curv = prm.curvilinear != 0;
  if (prm.groups4)
    return curv ? launch_persist_t<4, 9, true>(prm, P, stall_test, st)
                : launch_persist_t<4, 9, false>(prm, P, stall_test, st);
  return curv ? launch_persist_t<2, 18, true>(prm, P, stall_test, st)
              : launch_persist_t<2, 18, false>(prm, P, stall_test, st);
}

}  // namespace umwm
