// Per-substep forcing and cut-off kernel, the dts/dtr control kernel, and the
// once-per-output kernels: diag, Stokes drift, sea-ice Hs, the screen line
// and the spectrum layout transposes.
#include <algorithm>
#include <cfloat>

#include "kernels.hpp"
#include "misc_body.cuh"

namespace umwm {

// forcinginterpolate + the global side effects at the top of sin_d12
// (umwm_forcing.F90:40-99, umwm_source_functions.F90:21-36): per unrolled
// point (land included) interpolate the 2-d forcing levels in sumt/dtg,
// clamp wspd, rhorat; per wet point the cut-off index oc and the
// sheltering coefficient (umwm_source_functions.F90:52).
__global__ void k_prep(const Params prm, const Ptrs P, int compute_rot) {
  const Member& M = prm.mem[blockIdx.y];
  Ctl* ctl = M.ctl;
  if (ctl->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.NM; i += gridDim.x * blockDim.x)
    prep_point(prm, P, M, ctl, i, compute_rot);
}

// source(): dts = min(min_i physics_time_step, dtamin, dtg - sumt), the
// first-step rule and sumt update (umwm_physics.F90:41-58); refraction's
// dtr (umwm_advection.F90:145-158).  One thread.
__global__ void k_dts(const Params prm, const Ptrs P, int compute_rot, int first) {
  dts_body(prm, P, compute_rot, first);
}

// s_ice: significant wave height where fice > fice_lth and the attenuation
// factor C1*Hs (Hs < 3 m) or C1*3 (umwm_source_functions.F90:108-153).
__global__ void k_sice(const Params prm, const Ptrs P) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < prm.Ntot) sice_point(prm, P, j);
}

// diag, umwm_physics.F90:89-205, one thread per wet point.  The bins are
// visited frequency by frequency (the level's table rows read once), so the
// sums run in another order than the reference's direction-outer loops; the
// peak keeps the reference's choice among equal values, the first in its
// (o fastest, p slowest) order.
__global__ void k_diag(const Params prm, const Ptrs P) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= prm.Ntot) return;
  const Member& Mb = prm.mem[prm.tile_mem[j / TILE]];
  if (j >= Mb.ghost) return;
  const int ja = apt(Mb, j);
  const int O = prm.O, NP = prm.P, oc = P.oc[j];
  const float* E = P.E;
  auto tab = [&](int t, int o) { return P.TAB[tidx(prm, o, t, j)]; };
  float m0 = 0.f, m2 = 0.f, m2k = 0.f, mx = 0.f, my = 0.f, cxx = 0.f, cxy = 0.f, cyy = 0.f, xc = 0.f, yc = 0.f;
  float best = -1.f;
  int op = 0, pp = 0;
  for (int o = 0; o < O; ++o) {
    const float kdk = tab(T_KDK, o), k3dk = tab(T_K3DK, o), f2 = prm.f[o] * prm.f[o];
    const bool pr = o < oc;
    const float icp = pr ? 1.f / tab(T_CP0, o) : 0.f, cg = pr ? tab(T_CG0, o) : 0.f;
    const float* Eo = E + sidx(prm, o, 0, j);
#pragma unroll 4
    for (int p = 0; p < NP; ++p) {
      const float cth = prm.cth[p], sth = prm.sth[p];
      const float e = Eo[p * 32];
      const float ek = e * kdk;
      m0 += ek;
      m2 += (f2 * e) * kdk;
      m2k += e * k3dk;
      xc += ek * cth; yc += ek * sth;
      if (ek > best || (ek == best && p < pp)) { best = ek; op = o; pp = p; }
      if (pr) {
        const float ekc = ek * icp;
        mx += ekc * cth; my += ekc * sth;
        cxx += cg * ekc * (cth * cth); cxy += cg * ekc * cth * sth; cyy += cg * ekc * (sth * sth);
      }
    }
  }
  const float rw = P.rhow[ja] * prm.dthg;
  P.mwp[j] = sqrtf(m0 / (m2 + FLT_MIN));
  P.momx[j] = mx * rw; P.momy[j] = my * rw;
  P.cgmxx[j] = cxx * rw; P.cgmxy[j] = cxy * rw; P.cgmyy[j] = cyy * rw;
  P.ht[j] = 4.f * sqrtf(m0 * prm.dth);
  P.mwd[j] = atan2f(yc, xc);
  P.mss[j] = m2k * prm.dth;
  P.mwl[j] = 2.f * 3.14159274f * sqrtf(m0 / (m2k + FLT_MIN));
  P.dwd[j] = prm.th[pp];
  P.dwl[j] = 2.f * 3.14159274f / tab(T_K, op);
  P.dwp[j] = 1.f / prm.f[op];
  const float c0 = tab(T_CP0, op), g0 = tab(T_CG0, op);
  P.dcp0[j] = c0; P.dcg0[j] = g0;
  const float uc = P.uc[ja], vc = P.vc[ja];
  P.dcp[j] = c0 + uc * prm.cth[pp] + vc * prm.sth[pp];
  P.dcg[j] = g0 + uc * prm.cth[pp] + vc * prm.sth[pp];
}

// stokes_drift, umwm_stokes.F90:55-128: util recomputed from k, d and cg0
// instead of stored (it would be om*im*lm floats).  Per point the
// direction sums X(o), Y(o) are formed once; the depths are then taken in
// chunks of SLC with the per-frequency factors computed once per chunk, and
// the depth-dependent exponentials through ex2 (cosh(x) = (2^(x log2 e) +
// 2^(-x log2 e)) / 2, which has no cancellation; sinh(kd), which has, stays
// sinhf).
__global__ void k_stokes(const Params prm, const Ptrs P) {
  constexpr int SLC = 8;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= prm.Ntot) return;
  const Member& Mb = prm.mem[prm.tile_mem[j / TILE]];
  if (j >= Mb.ghost) return;
  const int O = prm.O, NP = prm.P, ldN = prm.ldN, lm = prm.lm;
  float X[MAX_OM], Y[MAX_OM];
  for (int o = 0; o < O; ++o) {
    float x = 0.f, y = 0.f;
    const float* Eo = P.E + sidx(prm, o, 0, j);
#pragma unroll 4
    for (int p = 0; p < NP; ++p) {
      const float e = Eo[p * 32];
      x += e * prm.cth[p];
      y += e * prm.sth[p];
    }
    X[o] = x; Y[o] = y;
  }
  const float d = P.d[j];
  const float twopi = 2.f * 3.14159274f, log2e = 1.44269504f;
  float um1 = 0.f, usm_prev = 0.f, ds = 0.f, ust_ef = 0.f;
  bool found = false;
  for (int l0 = 0; l0 < lm; l0 += SLC) {
    float su[SLC], sv[SLC];
#pragma unroll
    for (int i = 0; i < SLC; ++i) su[i] = sv[i] = 0.f;
    for (int o = 0; o < O; ++o) {
      const float kk = P.TAB[tidx(prm, o, T_K, j)];
      const float dwn = prm.dom[o] / fabsf(P.TAB[tidx(prm, o, T_CG0, j)]);
      const float kd = kk * d;
      const float a = ((twopi * prm.f[o]) * (kk * kk)) * dwn * prm.dth;  // util without its depth factor
      const float sh = sinhf(kd);
      const float ish2 = kd > 50.f ? 0.f : 1.f / (sh * sh);
      const float k2l = 2.f * kk * log2e;
#pragma unroll
      for (int i = 0; i < SLC; ++i) {
        const int l = l0 + i;
        if (l < lm) {
          const float dep = prm.depth[l];
          if (!(fabsf(dep) > d)) {
            const float arg = 2.f * kk * (dep + d);
            float u;
            if (fabsf(arg) > 50.f || kd > 50.f) {
              u = (2.f * a) * ex2_approx(k2l * dep);
            } else {
              const float t = k2l * (dep + d);
              u = a * (0.5f * (ex2_approx(t) + ex2_approx(-t))) * ish2;
            }
            su[i] += u * X[o];
            sv[i] += u * Y[o];
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < SLC; ++i) {
      const int l = l0 + i;
      if (l < lm) {
        const float dep = prm.depth[l];
        P.us[(size_t)l * ldN + j] = su[i];
        P.vs[(size_t)l * ldN + j] = sv[i];
        const float um = sqrtf(su[i] * su[i] + sv[i] * sv[i]);
        if (l == 0) {
          um1 = um;
          ust_ef = um1 * prm.eulerinv;
        } else if (um1 != 0.f && !found && um < ust_ef) {
          ds = (fabsf(usm_prev - ust_ef) * dep + fabsf(um - ust_ef) * prm.depth[l - 1]) / (usm_prev - um);
          found = true;
        }
        usm_prev = um;
      }
    }
  }
  P.ds[j] = -ds;
}

// Screen line at the print point (umwm_top.F90:143-148, umwm_util.F90:69-124);
// also clears 'first' after the first substep.
__global__ void k_screen(const Params prm, const Ptrs P) {
  __shared__ float s0[256], s2[256];
  screen_member<256, 256>(prm, P, blockIdx.x, s0, s2);
}

// Reference order F(om,pm,im) (o fastest) <-> the blocked device layout.
__global__ void k_to_ref(const Params prm, const float* __restrict__ E, float* __restrict__ F, int off, int n) {
  __shared__ float tile[32][33];
  const int R = prm.O * prm.P;
  const int c0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < 32; k += blockDim.y) {
    const int c = c0 + k;  // column of F: c = p*O + o
    if (c < R && j0 + tx < n) {
      const int o = c % prm.O, p = c / prm.O;
      tile[k][tx] = E[sidx(prm, o, p, off + j0 + tx)];
    }
  }
  __syncthreads();
  for (int k = ty; k < 32; k += blockDim.y) {
    const int jrow = j0 + k, c = c0 + tx;
    if (jrow < n && c < R) F[(size_t)jrow * R + c] = tile[tx][k];
  }
}

__global__ void k_from_ref(const Params prm, const float* __restrict__ F, float* __restrict__ E, int off, int n) {
  __shared__ float tile[32][33];
  const int R = prm.O * prm.P;
  const int c0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < 32; k += blockDim.y) {
    const int jrow = j0 + k, c = c0 + tx;
    if (jrow < n && c < R) tile[k][tx] = F[(size_t)jrow * R + c];
  }
  __syncthreads();
  for (int k = ty; k < 32; k += blockDim.y) {
    const int c = c0 + k;
    if (c < R && j0 + tx < n) {
      const int o = c % prm.O, p = c / prm.O;
      E[sidx(prm, o, p, off + j0 + tx)] = tile[tx][k];
    }
  }
}

// start of a dtg: sumt = 0 and no member done (umwm_top.F90:88)
__global__ void k_begin_dtg(const Params prm) {
  for (int m = threadIdx.x; m < prm.nmem; m += blockDim.x) {
    Ctl& c = *prm.mem[m].ctl;
    c.sumt = 0.f;
    c.done = 0;
  }
}

// stress('ocn'), umwm_stress.F90:34-214: per wet point, from the current
// spectrum and the source terms the last substep of the dtg kept (Sin, Sds
// after cothkd, Snl, and the ustar of its sdt).  One thread per point; the
// sums over directions run inside the frequency sums in the reference's
// order (p outer, o inner per accumulator, then the sum over o with kdk).
__global__ void k_stress_ocn(const Params prm, const Ptrs P) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= prm.Ntot) return;
  const Member& M = prm.mem[prm.tile_mem[j / TILE]];
  if (j >= M.ghost) return;
  const int ja = apt(M, j);
  const int O = prm.O, NP = prm.P, oc = P.oc[j];
  const float rhow = P.rhow[ja], wdir = P.wdir[ja];
  const float sdtc = (prm.sdt_fac * sqrtf(P.rhorat[ja])) * P.src_ust[j];
  auto tab = [&](int t, int o) { return P.TAB[tidx(prm, o, t, j)]; };
  float top_x = 0, top_y = 0, bot_x = 0, bot_y = 0, snl_x = 0, snl_y = 0, eo_x = 0, eo_y = 0, ea_x = 0, ea_y = 0;
  float tailx = 0, taily = 0;
  float f1x = 0, f1y = 0, f2x = 0, f2y = 0, f3x = 0, f3y = 0;
  for (int o = 0; o < O; ++o) {
    const float cp0 = tab(T_CP0, o), icp = 1.f / cp0, kdk = tab(T_KDK, o), kk = tab(T_K, o);
    const float sdt = sdtc * kk, sdv = tab(T_SDV, o), sbf = tab(T_SBF, o);
    // downshifting weights at levels o >= 3 (1-based)
    float wm = 0.f, wl = 0.f;
    if (o >= 2) {
      const float i1 = 1.f / tab(T_CP0, o - 1), i2 = 1.f / tab(T_CP0, o - 2);
      wm = prm.bf1 * cp0 * i1 + prm.bf2 * cp0 * i2;
      wl = prm.bf1 * (1.f - cp0 * i1) + prm.bf2 * (1.f - cp0 * i2);
    }
    float ux = 0, uy = 0, bx = 0, by = 0, nx = 0, ny = 0, ex = 0, ey = 0, ax = 0, ay = 0;
    for (int p = 0; p < NP; ++p) {
      const size_t a = sidx(prm, o, p, j);
      const float e = P.E[a], sin_ = P.src_sin[a], sds = P.src_sds[a], snl = P.src_snl[a];
      const float c = prm.cth[p], s = prm.sth[p];
      ux = ux + e * (sds + sdt + sdv) * c * icp;
      uy = uy + e * (sds + sdt + sdv) * s * icp;
      if (o >= 2) {
        ux = ux - snl * wm * c * icp;
        uy = uy - snl * wm * s * icp;
      }
      bx = bx + e * sbf * c * icp;
      by = by + e * sbf * s * icp;
      if (o >= 2 && o < oc) {
        nx = nx + snl * wl * c * icp;
        ny = ny + snl * wl * s * icp;
      }
      ex = ex + e * sds * c;
      ey = ey + e * sds * s;
      if (o >= 2) {
        ex = ex - snl * wm * c;
        ey = ey - snl * wm * s;
      }
      ax = ax + e * sin_ * c;
      ay = ay + e * sin_ * s;
      const float dd = e * sin_ * icp * kdk;
      if (sin_ > 0.f) {
        f1x += dd * c; f1y += dd * s;
      } else if (cosf(wdir - prm.th[p]) < 0.f) {
        f2x += dd * c; f2y += dd * s;
      } else {
        f3x += dd * c; f3y += dd * s;
      }
    }
    top_x += ux * kdk; top_y += uy * kdk;
    bot_x += bx * kdk; bot_y += by * kdk;
    snl_x += nx * kdk; snl_y += ny * kdk;
    eo_x += ex * kdk; eo_y += ey * kdk;
    ea_x += ax * kdk; ea_y += ay * kdk;
    if (o == O - 1) {
      const float tl = stress_tail(P.wspd[ja], kk);
      tailx = ux * kk * tl * rhow * prm.dthg;
      taily = uy * kk * tl * rhow * prm.dthg;
    }
  }
  const float rg = rhow * prm.dthg;
  const size_t L = (size_t)prm.ldN;
  float* out = P.ocn;
  out[OCN_TAUX_TOP * L + j] = top_x * rg + tailx + P.taux_skin[j];
  out[OCN_TAUY_TOP * L + j] = top_y * rg + taily + P.tauy_skin[j];
  out[OCN_TAUX_BOT * L + j] = bot_x * rg;
  out[OCN_TAUY_BOT * L + j] = bot_y * rg;
  out[OCN_TAUX_SNL * L + j] = snl_x * rg;
  out[OCN_TAUY_SNL * L + j] = snl_y * rg;
  out[OCN_EPSX_OCN * L + j] = eo_x * rg;
  out[OCN_EPSY_OCN * L + j] = eo_y * rg;
  out[OCN_EPSX_ATM * L + j] = ea_x * rg;
  out[OCN_EPSY_ATM * L + j] = ea_y * rg;
  out[OCN_TAILX * L + j] = tailx;
  out[OCN_TAILY * L + j] = taily;
  out[OCN_TAUX1 * L + j] = f1x * rg;
  out[OCN_TAUY1 * L + j] = f1y * rg;
  out[OCN_TAUX2 * L + j] = f2x * rg;
  out[OCN_TAUY2 * L + j] = f2y * rg;
  out[OCN_TAUX3 * L + j] = f3x * rg;
  out[OCN_TAUY3 * L + j] = f3y * rg;
}

// Graph-driven inner loop: arm before the graph launch, then after each
// substep count it and set the while node's condition (another substep while
// a member is inside the dtg and the budget lasts).
__global__ void k_loop_arm(Global* g, int budget) {
  g->budget = budget;
  g->iters = 0;
}

__global__ void k_loop_cond(Global* g, cudaGraphConditionalHandle h) {
  g->iters += 1;
  if (g->budget > 0) g->budget -= 1;
  cudaGraphSetConditional(h, (g->not_done && g->budget != 0) ? 1u : 0u);
}

// Count the NaN/Inf values of a[0..n) into *count (option "check_finite").
__global__ void k_count_nonfinite(const float* __restrict__ a, size_t n, int* count) {
  int bad = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    bad += isfinite(a[i]) ? 0 : 1;
  bad = __syncthreads_count(bad > 0);
  if (threadIdx.x == 0 && bad) atomicAdd(count, bad);
}

__global__ void k_fill(float* a, size_t n, float v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = v;
}

static int grid_for(long n, int block) {
  long g = (n + block - 1) / block;
  if (g > 152L * 32) g = 152L * 32;
  return (int)(g < 1 ? 1 : g);
}

cudaError_t launch_prep(const Params& prm, const Ptrs& P, int compute_rot, int max_nm, cudaStream_t st) {
  dim3 grid(grid_for(max_nm, 256), prm.nmem);
  k_prep<<<grid, 256, 0, st>>>(prm, P, compute_rot);
  return cudaGetLastError();
}
cudaError_t launch_dts(const Params& prm, const Ptrs& P, int compute_rot, int first, cudaStream_t st) {
  k_dts<<<1, 256, 0, st>>>(prm, P, compute_rot, first);
  return cudaGetLastError();
}
cudaError_t launch_sice(const Params& prm, const Ptrs& P, cudaStream_t st) {
  k_sice<<<(prm.Ntot + 127) / 128, 128, 0, st>>>(prm, P);
  return cudaGetLastError();
}
cudaError_t launch_diag(const Params& prm, const Ptrs& P, cudaStream_t st) {
  k_diag<<<(prm.Ntot + 127) / 128, 128, 0, st>>>(prm, P);
  return cudaGetLastError();
}
cudaError_t launch_stokes(const Params& prm, const Ptrs& P, cudaStream_t st) {
  k_stokes<<<(prm.Ntot + 127) / 128, 128, 0, st>>>(prm, P);
  return cudaGetLastError();
}
cudaError_t launch_screen(const Params& prm, const Ptrs& P, cudaStream_t st) {
  k_screen<<<prm.nmem, 256, 0, st>>>(prm, P);
  return cudaGetLastError();
}
cudaError_t launch_to_ref(const Params& prm, const float* E, float* F, int off, int n, cudaStream_t st) {
  dim3 grid((prm.O * prm.P + 31) / 32, (n + 31) / 32), block(32, 8);
  k_to_ref<<<grid, block, 0, st>>>(prm, E, F, off, n);
  return cudaGetLastError();
}
cudaError_t launch_from_ref(const Params& prm, const float* F, float* E, int off, int n, cudaStream_t st) {
  dim3 grid((prm.O * prm.P + 31) / 32, (n + 31) / 32), block(32, 8);
  k_from_ref<<<grid, block, 0, st>>>(prm, F, E, off, n);
  return cudaGetLastError();
}
cudaError_t launch_begin_dtg(const Params& prm, cudaStream_t st) {
  k_begin_dtg<<<1, 256, 0, st>>>(prm);
  return cudaGetLastError();
}
cudaError_t launch_stress_ocn(const Params& prm, const Ptrs& P, cudaStream_t st) {
  k_stress_ocn<<<(prm.Ntot + 127) / 128, 128, 0, st>>>(prm, P);
  return cudaGetLastError();
}
cudaError_t launch_loop_arm(Global* g, int budget, cudaStream_t st) {
  k_loop_arm<<<1, 1, 0, st>>>(g, budget);
  return cudaGetLastError();
}
cudaError_t launch_loop_cond(Global* g, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_loop_cond<<<1, 1, 0, st>>>(g, h);
  return cudaGetLastError();
}
cudaError_t launch_count_nonfinite(const float* a, size_t n, int* count, cudaStream_t st) {
  k_count_nonfinite<<<grid_for((long)std::min<size_t>(n, 1u << 30), 256), 256, 0, st>>>(a, n, count);
  return cudaGetLastError();
}
cudaError_t launch_fill(float* a, size_t n, float v, cudaStream_t st) {
  k_fill<<<grid_for((long)std::min<size_t>(n, 1u << 30), 256), 256, 0, st>>>(a, n, v);
  return cudaGetLastError();
}

}  // namespace umwm
