// Propagation, refraction, e = ef and stress('atm') in one pass
// (umwm_advection.F90:18-180, umwm_top.F90:113-115, umwm_stress.F90:17-264).
//
// Same tiling as the source kernels: 32 consecutive wet points per CTA
// (lane = point), 4 warps over contiguous direction groups.  E* (ES) is read
// at the point and its four unrolled neighbours; the east/west neighbours
// sit one wet column away (about nm indices) and are served from L2, which
// holds the few-MB window of rows that the CTAs in flight are working on.
// Refraction needs E* at p-1 and p+1; the group's two edge directions are
// loaded as well.  The rotation rate is recomputed from cp0 and the
// currents instead of being stored (it depends on no spectral value); when
// the reference would reuse the rotation of an earlier substep
// (currents = .F.) the mask o <= oc of that substep is kept in oc_rot.
// The wind stress sums e*Sin*cos/sin(th)/cp over the new spectrum while it
// is still in registers and the last warp-group finishes the per-point
// drag, skin-stress and ustar update.
#include "dev_common.cuh"
#include "kernels.hpp"

namespace umwm {

constexpr int NW = 4;

// stress_tail, umwm_stress.F90:300-311
__device__ __forceinline__ float stress_tail(float w, float kmax) {
  const float kcap = 1e3f, a = 0.000112f, b = -0.01451f, c = -1.0186f;
  float tail = a * (w * w) + b * w + c;
  float kpt = powf(kmax, tail);
  return (powf(kcap, tail + 1.f) - kmax * kpt) / (kpt * (tail + 1.f));
}

template <int PW>
__global__ void __launch_bounds__(128) k_advect(const Params prm, const Ptrs P) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int N = prm.N, ldN = prm.ldN, O = prm.O, NP = prm.P;
  const int j = blockIdx.x * 32 + lane;
  const bool valid = j < N;
  const int jj = valid ? j : N;
  const int p0 = w * PW;
  __shared__ float red[6][NW][32];

  const Ctl* ctl = P.ctl;
  const float dta = ctl->dta, dtr = ctl->dtr;
  const bool zerocur = ctl->zerocurrents != 0;

  const int ie = P.ie[jj], iw = P.iw[jj], in = P.in[jj], is = P.is[jj];
  const int oc = P.oc[jj], ocr = P.oc_rot[jj];
  const bool ice = P.fice[jj] > prm.fice_uth;
  const float oneovar = P.oneovar[jj], dxn = P.dxn[jj], dxs = P.dxs[jj], dye = P.dye[jj], dyw = P.dyw[jj];
  const float odx = P.oneovdx[jj], ody = P.oneovdy[jj];
  const float ustar = P.ustar[jj];
  const WindIn wi = load_wind(prm, P, jj, ustar);
  const float wdir = P.wdir[jj];

  // current advection coefficients, umwm_advection.F90:64-74
  float feup = 0.f, fedn = 0.f, fwup = 0.f, fwdn = 0.f, fnup = 0.f, fndn = 0.f, fsup = 0.f, fsdn = 0.f;
  const float uci = P.uc[jj], vci = P.vc[jj];
  const float uce = P.uc[P.iie[jj]], ucw = P.uc[P.iiw[jj]], ucn = P.uc[P.iin[jj]], ucs = P.uc[P.iis[jj]];
  const float vce = P.vc[P.iie[jj]], vcw = P.vc[P.iiw[jj]], vcn = P.vc[P.iin[jj]], vcs = P.vc[P.iis[jj]];
  if (!zerocur) {
    float ue = uci + uce, uw = uci + ucw, vn = vci + vcn, vs = vci + vcs;
    feup = (ue + fabsf(ue)) * dye; fedn = (ue - fabsf(ue)) * dye;
    fwup = (uw + fabsf(uw)) * dyw; fwdn = (uw - fabsf(uw)) * dyw;
    fnup = (vn + fabsf(vn)) * dxn; fndn = (vn - fabsf(vn)) * dxn;
    fsup = (vs + fabsf(vs)) * dxs; fsdn = (vs - fabsf(vs)) * dxs;
  }

  float cw[PW], cc[PW], sc[PW];
  const float cv = prm.curvilinear ? P.curv[jj] : 0.f;
#pragma unroll
  for (int k = 0; k < PW; ++k) {
    const int p = p0 + k;
    cw[k] = cosf(wdir - prm.th[p]);
    if (prm.curvilinear) { cc[k] = cosf(prm.th[p] + cv); sc[k] = sinf(prm.th[p] + cv); }
    else { cc[k] = prm.cth[p]; sc[k] = prm.sth[p]; }
  }
  // stress_vector_integral divides by cp0 of the previous unrolled point
  // (assumed-shape dummy with lower bound 1 over cp0(:,0:im)),
  // umwm_stress.F90:401, :495-513
  const int jprev = (jj == 0 || jj >= N) ? N : jj - 1;

  float sx = 0.f, sy = 0.f, dxs_ = 0.f, dys_ = 0.f, txom = 0.f, tyom = 0.f;
  const int pm1 = (p0 + NP - 1) % NP, ppw = (p0 + PW) % NP;

  for (int o = 0; o < O; ++o) {
    const float* T = P.TAB + (size_t)o * T_COUNT * ldN;
    const float* ESo = P.ES + (size_t)o * NP * ldN;
    const float* EFo = P.EF + (size_t)o * NP * ldN;
    float* Eo = P.E + (size_t)o * NP * ldN;
    float ef[PW];
#pragma unroll
    for (int k = 0; k < PW; ++k) ef[k] = __ldg(EFo + (size_t)(p0 + k) * ldN + jj);
    if (o < oc) {
      // ---- propagation, umwm_advection.F90:30-97
      const float* CG = T + T_CG0 * ldN;
      const float cgi = __ldg(CG + jj), cgE = __ldg(CG + ie), cgW = __ldg(CG + iw), cgN = __ldg(CG + in),
                  cgS = __ldg(CG + is);
      float es[PW + 2];
      es[0] = __ldg(ESo + (size_t)pm1 * ldN + jj);
#pragma unroll
      for (int k = 0; k < PW; ++k) es[k + 1] = __ldg(ESo + (size_t)(p0 + k) * ldN + jj);
      es[PW + 1] = __ldg(ESo + (size_t)ppw * ldN + jj);
#pragma unroll
      for (int k = 0; k < PW; ++k) {
        const float* row = ESo + (size_t)(p0 + k) * ldN;
        const float e0 = es[k + 1];
        const float ee = __ldg(row + ie), ew = __ldg(row + iw), en = __ldg(row + in), esn = __ldg(row + is);
        const float cge = cgi * cc[k] + cgE * cc[k];
        const float cgw = cgi * cc[k] + cgW * cc[k];
        const float cgs = cgi * sc[k] + cgS * sc[k];
        const float cgn = cgi * sc[k] + cgN * sc[k];
        float flux = (cge + fabsf(cge)) * dye * e0 + (cge - fabsf(cge)) * dye * ee -
                     (cgw + fabsf(cgw)) * dyw * ew - (cgw - fabsf(cgw)) * dyw * e0 +
                     (cgn + fabsf(cgn)) * dxn * e0 + (cgn - fabsf(cgn)) * dxn * en -
                     (cgs + fabsf(cgs)) * dxs * esn - (cgs - fabsf(cgs)) * dxs * e0;
        if (!zerocur)
          flux = flux + (feup * e0 + fedn * ee - fwup * ew - fwdn * e0 + fnup * e0 + fndn * en - fsup * esn -
                         fsdn * e0);
        ef[k] = ef[k] - 0.25f * dta * flux * oneovar;
        if (ice) ef[k] = 0.f;
      }
      // ---- refraction, umwm_advection.F90:122-178
      if (o < ocr) {
        const float* CP = T + T_CP0 * ldN;
        const float dcx = __ldg(CP + ie) - __ldg(CP + iw);
        const float dcy = __ldg(CP + in) - __ldg(CP + is);
        float r[PW + 2];
#pragma unroll
        for (int k = 0; k < PW + 2; ++k) {
          const int p = (k == 0) ? pm1 : (k == PW + 1 ? ppw : p0 + k - 1);
          r[k] = 0.5f * ((dcx * prm.sth[p] + vce - vcw) * odx - (dcy * prm.cth[p] + ucn - ucs) * ody);
        }
#pragma unroll
        for (int k = 0; k < PW; ++k) {
          const float rl = 0.5f * (r[k + 1] + r[k + 2]);  // pl(p) = p+1
          const float rr = 0.5f * (r[k + 1] + r[k]);      // pr(p) = p-1
          const float fl = 0.5f *
                           ((rl + fabsf(rl)) * es[k + 1] + (rl - fabsf(rl)) * es[k + 2] -
                            (rr + fabsf(rr)) * es[k] - (rr - fabsf(rr)) * es[k + 1]) *
                           prm.oneovdth;
          ef[k] = ef[k] - dtr * fl;
          if (ice) ef[k] = 0.f;
        }
      }
    }
    // ---- e = ef and the form-stress integrand
    const float logl2z = __ldg(T + T_LOGL2Z * ldN + jj), cp0 = __ldg(T + T_CP0 * ldN + jj);
    const float fkovg = __ldg(T + T_FKOVG * ldN + jj), kdk = __ldg(T + T_KDK * ldN + jj);
    const float icp = 1.f / __ldg(T + T_CP0 * ldN + jprev);
    const bool tail = o >= oc;
    float tx = 0.f, ty = 0.f;
#pragma unroll
    for (int k = 0; k < PW; ++k) {
      const int p = p0 + k;
      if (valid) Eo[(size_t)p * ldN + j] = ef[k];
      float s = sin_bin(prm, wi, cw[k], prm.cth[p], prm.sth[p], logl2z, cp0, fkovg, tail);
      float es_ = ef[k] * s;
      tx += es_ * prm.cth[p] * icp;
      ty += es_ * prm.sth[p] * icp;
    }
    sx += tx * kdk; sy += ty * kdk;
    if (o >= oc - 1) { dxs_ += tx * kdk; dys_ += ty * kdk; }
    if (o == O - 1) { txom = tx; tyom = ty; }
  }

  red[0][w][lane] = sx; red[1][w][lane] = sy; red[2][w][lane] = dxs_;
  red[3][w][lane] = dys_; red[4][w][lane] = txom; red[5][w][lane] = tyom;
  __syncthreads();
  if (w != 0 || !valid) return;
  float v[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) v[q] = ((red[q][0][lane] + red[q][1][lane]) + red[q][2][lane]) + red[q][3][lane];
  // ---- stress('atm') per point, umwm_stress.F90:216-262
  const float rhow = P.rhow[j], rhoa = P.rhoa[j], wspd = wi.wspd;
  const float kom = __ldg(P.TAB + ((size_t)(O - 1) * T_COUNT + T_K) * ldN + j);
  const float tail = stress_tail(wspd, kom);
  const float tax = v[4] * kom * tail * rhow * prm.dthg;
  const float tay = v[5] * kom * tail * rhow * prm.dthg;
  const float tfx = v[0] * rhow * prm.dthg + tax;
  const float tfy = v[1] * rhow * prm.dthg + tay;
  P.tailatmx[j] = tax; P.tailatmy[j] = tay;
  P.taux_form[j] = tfx; P.tauy_form[j] = tfy;
  P.taux_diag[j] = v[2] * rhow * prm.dthg;
  P.tauy_diag[j] = v[3] * rhow * prm.dthg;
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

cudaError_t launch_advect(const Params& prm, const Ptrs& P, cudaStream_t st) {
  const int PW = prm.P / NW;
  dim3 grid((prm.N + 31) / 32), block(128);
  switch (PW) {
#define CASE(X) \
  case X: k_advect<X><<<grid, block, 0, st>>>(prm, P); break;
    CASE(2) CASE(3) CASE(4) CASE(6) CASE(8) CASE(9) CASE(12) CASE(16) CASE(18)
#undef CASE
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

}  // namespace umwm
