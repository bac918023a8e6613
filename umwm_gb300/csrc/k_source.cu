// Source-term kernels: sin_d12, sds_d12, snl_d12, s_ice and source()
// (umwm_source_functions.F90:16-183, umwm_physics.F90:9-86).
//
// One CTA owns a tile of 32 consecutive wet points (lane = point, so every
// load of one (o,p) bin is a 128-byte line) and 4 warps split the pm
// directions into 4 contiguous groups of PW.  The frequency loop walks
// o = 1..om in order because the mean-square-slope adjustment of Sds is a
// prefix over o:
//   dummy(o,p) = dummy(o-1,p) + k3dk(o-1) * sum_pp e(o-1,pp) cth2pp(pp,p),
//   cth2pp(pp,p) = cos^2(th(pp)-th(p)) dth = dth/2 (1 + cos2th(pp)cos2th(p)
//                                                  + sin2th(pp)sin2th(p)),
// so dummy(o,.) = A + B cos2th(p) + C sin2th(p) with three running sums per
// point (exact algebra; replaces pm multiply-adds per bin by 2).
// Snl at level o needs Sds*e at o+1 and o+2, so the integration finishes
// level o two iterations after it was loaded.
//
// MODE_PHYS : per-point max |exponent argument| -> physics_time_step and the
//             global min for dts (umwm_physics.F90:18-41); optionally the
//             global max of the rotation rate for refraction's dtr
//             (umwm_advection.F90:125-154).
// MODE_INTEG: exponential integration (o <= oc), equilibrium tail (o > oc),
//             E* = (e + ef)/2 -> ES, ef -> EF (umwm_physics.F90:61-84).
#include "dev_common.cuh"
#include "kernels.hpp"

namespace umwm {

constexpr int NWARP = 4;

template <int PW, bool INTEG>
__global__ void __launch_bounds__(128) k_source(const Params prm, const Ptrs P, int compute_rot) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int N = prm.N, ldN = prm.ldN, O = prm.O, NP = prm.P;
  const int j = blockIdx.x * 32 + lane;
  const bool valid = j < N;
  const int jj = valid ? j : N;  // the ghost column keeps loads in bounds
  const int p0 = w * PW;
  __shared__ float4 part[2][NWARP][32];
  __shared__ float red[NWARP][32];

  const float dts = INTEG ? P.ctl->dts : 0.f;
  const float ustar = P.ustar[jj];
  const WindIn wi = load_wind(prm, P, jj, ustar);
  const float wdir = P.wdir[jj];
  const float sdtc = (prm.sdt_fac * sqrtf(P.rhorat[jj])) * ustar;
  const float sv = prm.ice_possible ? P.sice_v[jj] : 0.f;
  const float hdth = 0.5f * prm.dth;

  float cw[PW];
#pragma unroll
  for (int k = 0; k < PW; ++k) cw[k] = cosf(wdir - prm.th[p0 + k]);

  // rotation-rate inputs (refraction), only for MODE_PHYS with compute_rot
  int nie = N, niw = N, nin = N, nis = N;
  float vce = 0.f, vcw = 0.f, ucn = 0.f, ucs = 0.f, odx = 0.f, ody = 0.f;
  if (!INTEG && compute_rot) {
    nie = P.ie[jj]; niw = P.iw[jj]; nin = P.in[jj]; nis = P.is[jj];
    vce = P.vc[P.iie[jj]]; vcw = P.vc[P.iiw[jj]]; ucn = P.uc[P.iin[jj]]; ucs = P.uc[P.iis[jj]];
    odx = P.oneovdx[jj]; ody = P.oneovdy[jj];
  }

  float A = 0.f, B = 0.f, C = 0.f;        // dummy coefficients for the current level
  float A2 = 0.f, B2 = 0.f, C2 = 0.f;     // ... two levels back (tail of MODE_INTEG)
  float A1 = 0.f, B1 = 0.f, C1 = 0.f;     // ... one level back
  float eL1[PW], eL2[PW], sL1[PW], sL2[PW];
#pragma unroll
  for (int k = 0; k < PW; ++k) { eL1[k] = eL2[k] = sL1[k] = sL2[k] = 0.f; }
  float mx = 0.f, rmx = 0.f;

  const int OL = INTEG ? O + 2 : O;
  for (int o = 0; o < OL; ++o) {
    float ec[PW], sc[PW];
    if (o < O) {
      const float* Erow = P.E + ((size_t)o * NP + p0) * ldN + jj;
#pragma unroll
      for (int k = 0; k < PW; ++k) ec[k] = __ldg(Erow + (size_t)k * ldN);
      const float* T = P.TAB + (size_t)o * T_COUNT * ldN + jj;
      const float k4 = __ldg(T + T_K4 * ldN);
      float s0 = 0.f, sc2 = 0.f, ss2 = 0.f;
#pragma unroll
      for (int k = 0; k < PW; ++k) {
        s0 += ec[k];
        sc2 += ec[k] * prm.c2th[p0 + k];
        ss2 += ec[k] * prm.s2th[p0 + k];
      }
      part[o & 1][w][lane] = make_float4(s0, sc2, ss2, 0.f);
      const float sA = prm.twopisds_fac * prm.f[o];
#pragma unroll
      for (int k = 0; k < PW; ++k) {
        float chi = A + B * prm.c2th[p0 + k] + C * prm.s2th[p0 + k];
        float t = 1.f + prm.mss_fac * chi;
        sc[k] = (sA * (t * t)) * pow_pos(ec[k] * k4, prm.sds_power);
      }
      if (!INTEG) {
        if (o < wi.oc) {
          const float logl2z = __ldg(T + T_LOGL2Z * ldN), cp0 = __ldg(T + T_CP0 * ldN);
          const float fkovg = __ldg(T + T_FKOVG * ldN), cothkd = __ldg(T + T_COTHKD * ldN);
          const float sbf = __ldg(T + T_SBF * ldN), sdv = __ldg(T + T_SDV * ldN), kk = __ldg(T + T_K * ldN);
          const float snl_arg = 1.f - (__ldg(T + T_BF1R * ldN) + __ldg(T + T_BF2R * ldN));
          const float sdt = sdtc * kk;
          const float sice = sv != 0.f ? 2.f * __ldg(T + T_CG0 * ldN) * sv : 0.f;
#pragma unroll
          for (int k = 0; k < PW; ++k) {
            const int p = p0 + k;
            float s = sin_bin(prm, wi, cw[k], prm.cth[p], prm.sth[p], logl2z, cp0, fkovg, false);
            float a = s - (sc[k] * cothkd) * snl_arg - sbf - sdt - sdv + sice;
            mx = fmaxf(mx, fabsf(a));
          }
          if (compute_rot) {
            const float* CP = P.TAB + ((size_t)o * T_COUNT + T_CP0) * ldN;
            const float dcx = __ldg(CP + nie) - __ldg(CP + niw);
            const float dcy = __ldg(CP + nin) - __ldg(CP + nis);
#pragma unroll
            for (int k = 0; k < PW; ++k) {
              const int p = p0 + k;
              float r = 0.5f * ((dcx * prm.sth[p] + vce - vcw) * odx - (dcy * prm.cth[p] + ucn - ucs) * ody);
              rmx = fmaxf(rmx, r);
            }
          }
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < PW; ++k) { ec[k] = 0.f; sc[k] = 0.f; }
    }
    __syncthreads();
    float S0 = 0.f, SC = 0.f, SS = 0.f;
    if (o < O) {
#pragma unroll
      for (int q = 0; q < NWARP; ++q) {
        float4 v = part[o & 1][q][lane];
        S0 += v.x; SC += v.y; SS += v.z;
      }
    }
    if (INTEG && o >= 2) {
      // finish level L = o-2
      const int L = o - 2;
      const float* T = P.TAB + (size_t)L * T_COUNT * ldN + jj;
      const float logl2z = __ldg(T + T_LOGL2Z * ldN), cp0 = __ldg(T + T_CP0 * ldN);
      const float fkovg = __ldg(T + T_FKOVG * ldN), cothkd = __ldg(T + T_COTHKD * ldN);
      const float sbf = __ldg(T + T_SBF * ldN), sdv = __ldg(T + T_SDV * ldN), kk = __ldg(T + T_K * ldN);
      const float sdt = sdtc * kk;
      const float sice = sv != 0.f ? 2.f * __ldg(T + T_CG0 * ldN) * sv : 0.f;
      const bool prog = L < wi.oc;
      float* ESrow = P.ES + ((size_t)L * NP + p0) * ldN + j;
      float* EFrow = P.EF + ((size_t)L * NP + p0) * ldN + j;
      if (prog) {
        const float bf1r = __ldg(T + T_BF1R * ldN), bf2r = __ldg(T + T_BF2R * ldN);
#pragma unroll
        for (int k = 0; k < PW; ++k) {
          const int p = p0 + k;
          float s = sin_bin(prm, wi, cw[k], prm.cth[p], prm.sth[p], logl2z, cp0, fkovg, false);
          float snl = (bf1r * sL1[k]) * eL1[k] + (bf2r * sc[k]) * ec[k] - (prm.snl_fac * sL2[k]) * eL2[k];
          float S = s - sL2[k] * cothkd - sbf - sdt - sdv + sice;
          float ef = eL2[k] * __expf(dts * S) + dts * snl;
          if (valid) {
            ESrow[(size_t)k * ldN] = 0.5f * (eL2[k] + ef);
            EFrow[(size_t)k * ldN] = ef;
          }
        }
      } else {
        const float oneoverk4 = 1.f / __ldg(T + T_K4 * ldN);
        const float sAc = (prm.twopisds_fac * prm.f[L]);
#pragma unroll
        for (int k = 0; k < PW; ++k) {
          const int p = p0 + k;
          float s = sin_bin(prm, wi, cw[k], prm.cth[p], prm.sth[p], logl2z, cp0, fkovg, true);
          float num = s - sdt - sdv + sice;
          float ef = 0.f;
          if (num >= 0.f) {
            float chi = A2 + B2 * prm.c2th[p] + C2 * prm.s2th[p];
            float t = 1.f + prm.mss_fac * chi;
            float den = (sAc * (t * t)) * cothkd;
            ef = oneoverk4 * pow_pos(num / den, prm.inv_sds_power);
          }
          if (valid) {
            ESrow[(size_t)k * ldN] = 0.5f * (eL2[k] + ef);
            EFrow[(size_t)k * ldN] = ef;
          }
        }
      }
    }
    // advance the dummy coefficients: level o -> o+1
    A2 = A1; B2 = B1; C2 = C1;
    A1 = A; B1 = B; C1 = C;
    if (o < O) {
      const float h = __ldg(P.TAB + ((size_t)o * T_COUNT + T_K3DK) * ldN + jj) * hdth;
      A += h * S0; B += h * SC; C += h * SS;
    }
    if (INTEG) {
#pragma unroll
      for (int k = 0; k < PW; ++k) { eL2[k] = eL1[k]; sL2[k] = sL1[k]; eL1[k] = ec[k]; sL1[k] = sc[k]; }
    }
  }

  if (!INTEG) {
    // per-point max over the 4 direction groups, then explim / max
    red[w][lane] = mx;
    __syncthreads();
    if (w == 0) {
      float m = fmaxf(fmaxf(red[0][lane], red[1][lane]), fmaxf(red[2][lane], red[3][lane]));
      float ph = prm.explim / m;
      if (valid) P.phys[j] = ph;
      float bm = valid ? ph : __int_as_float(0x7f800000);
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) bm = fminf(bm, __shfl_xor_sync(0xffffffffu, bm, s));
      if (lane == 0) atomicMin(&P.ctl->minphys_enc, enc_ord_d(bm));
    }
    if (compute_rot) {
      __syncthreads();
      red[w][lane] = valid ? rmx : 0.f;
      __syncthreads();
      if (w == 0) {
        float m = fmaxf(fmaxf(red[0][lane], red[1][lane]), fmaxf(red[2][lane], red[3][lane]));
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
        if (lane == 0) atomicMax(&P.ctl->maxrot_enc, enc_ord_d(m));
      }
    }
  }
}

template <bool INTEG>
static cudaError_t launch_source_t(const Params& prm, const Ptrs& P, int compute_rot, cudaStream_t st) {
  const int PW = prm.P / NWARP;
  dim3 grid((prm.N + 31) / 32), block(128);
  switch (PW) {
#define CASE(X) \
  case X: k_source<X, INTEG><<<grid, block, 0, st>>>(prm, P, compute_rot); break;
    CASE(2) CASE(3) CASE(4) CASE(6) CASE(8) CASE(9) CASE(12) CASE(16) CASE(18)
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
  int pw = pm / NWARP;
  return pm % NWARP == 0 && (pw == 2 || pw == 3 || pw == 4 || pw == 6 || pw == 8 || pw == 9 || pw == 12 ||
                             pw == 16 || pw == 18);
}

}  // namespace umwm
