// Device helpers shared by the kernel translation units.
#pragma once
#include <cuda_runtime.h>

#include "dev.cuh"

namespace umwm {

__device__ __forceinline__ unsigned enc_ord_d(float x) {
  unsigned u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float dec_ord_d(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// x^y for x >= 0 through the SFU (lg2/ex2); 0 for x == 0 (as pow does).
__device__ __forceinline__ float pow_pos(float x, float y) { return exp2f(y * __log2f(x)); }

// sheltering_coare35, umwm_sheltering.F90:49-79
__device__ __forceinline__ float shelter_coare35(float w) {
  const float x1 = 15.f, x2 = 33.f, x3 = 60.f, y1 = 0.10f, y2 = 0.09f, y3 = 0.06f;
  const float intercept = 0.04f, curvature = 0.65f, decay = 1.6f;
  float slope1 = (y1 - intercept) / x1;
  float slope2 = (y3 - y2) / (x3 - x2);
  float c = curvature * (slope2 - slope1) / (x2 - x1);
  float b = slope1 - 2.f * c * x1;
  float a = y1 - b * x1 - c * (x1 * x1);
  float s1 = a + b * x2 + c * (x2 * x2);
  if (w <= x1) return intercept + slope1 * w;
  if (w <= x2) return a + b * w + c * (w * w);
  return s1 * expf(-(w - x2) / (decay * w));
}

// Per-point inputs of the wind-input source term, sin_d12
// (umwm_source_functions.F90:16-82).
struct WindIn {
  float wspd, uc, vc, ustar25, shelt, c1;
  int oc;  // 1-based cut-off index; 0-based level o is prognostic when o < oc
};

// jj: global wet index; ja: its all-point index
__device__ __forceinline__ WindIn load_wind(const Params& prm, const Ptrs& P, int jj, int ja, float ustar) {
  WindIn w;
  w.wspd = P.wspd[ja];
  w.uc = P.uc[ja];
  w.vc = P.vc[ja];
  w.ustar25 = 2.5f * ustar;
  w.shelt = P.shelt[jj];
  // (1 - fice) * twopi * rhorat
  w.c1 = ((1.f - P.fice[ja]) * (2.f * 3.14159274f)) * P.rhorat[ja];
  w.oc = P.oc[jj];
  return w;
}

// all-point index of a wet (or ghost) point of member M
__device__ __forceinline__ int apt(const Member& M, int j) { return M.nmoff + (j - M.off); }

// max(x, 0) with NaN kept (max.NaN)
__device__ __forceinline__ float max_nan0(float x) {
  float r;
  asm("max.NaN.f32 %0, %1, 0f00000000;" : "=f"(r) : "f"(x));
  return r;
}

// Sin of one bin from x = U cos(wdir - th) - cp0 - uc cos th - vc sin th,
// umwm_source_functions.F90:39-80, with its factors folded: the reference
// forms sin_fac |x| x, then multiplies by shelt/sin_fac where positive, by
// fieldscale1 where negative and by fieldscale2 where still negative and
// cos(wdir - th) > 0, then by (1 - fice) 2 pi rhorat and fkovg.  Here
// (x |x|) is multiplied once by the factor its sign selects (shelt, or
// sin_fac fieldscale1 [fieldscale2], prm.sin_neg1/2) and once by
// gl = (1 - fice) 2 pi rhorat fkovg of the level: the same product in
// another order (a few ulp apart), in fewer instructions.
__device__ __forceinline__ float sin_fold(const Params& prm, float shelt, float x, float cw, float gl, bool tail) {
  const float a = x * fabsf(x);
  const float f = x > 0.f ? shelt : (cw > 0.f ? prm.sin_neg2 : prm.sin_neg1);
  float s = (a * f) * gl;
  if (tail) s = fmaxf(s, 0.f);
  return s;
}

// sin_fold of the two directions k, k+1 of one lane, with x formed as the
// scalar callers form it (U cw - cp0 - ucg cos th - vcg sin th) and the
// affine parts in packed f32x2 arithmetic (the integration's pairs: 2.29 ->
// 2.28 ms at 1000x1000; in the pre-pass and the propagation it measured no
// faster)
__device__ __forceinline__ float2 sin_fold2(const Params& prm, float shelt, float U, float2 cw, float ucg, float vcg,
                                            float2 cth, float2 sth, float cp0, float gl, bool tail) {
  float2 x = __ffma2_rn(make_float2(U, U), cw, make_float2(-cp0, -cp0));
  x = __ffma2_rn(make_float2(-ucg, -ucg), cth, x);
  x = __ffma2_rn(make_float2(-vcg, -vcg), sth, x);
  const float2 a = make_float2(x.x * fabsf(x.x), x.y * fabsf(x.y));
  const float2 f = make_float2(x.x > 0.f ? shelt : (cw.x > 0.f ? prm.sin_neg2 : prm.sin_neg1),
                               x.y > 0.f ? shelt : (cw.y > 0.f ? prm.sin_neg2 : prm.sin_neg1));
  float2 s = __fmul2_rn(__fmul2_rn(a, f), make_float2(gl, gl));
  if (tail) s = make_float2(fmaxf(s.x, 0.f), fmaxf(s.y, 0.f));
  return s;
}

#ifndef UMWM_PREFETCH_TAB
#define UMWM_PREFETCH_TAB 1  // the spectral kernels also prefetch the block's table rows with the spectrum
#endif

// 2^x through the SFU (ex2.approx.ftz)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 4-byte asynchronous copy global -> shared (cp.async), its group commit and
// wait (the wait ends when this thread's copies have landed)
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// stress_tail, umwm_stress.F90:300-311
__device__ __forceinline__ float stress_tail(float w, float kmax) {
  const float kcap = 1e3f, a = 0.000112f, b = -0.01451f, c = -1.0186f;
  float tail = a * (w * w) + b * w + c;
  float kpt = powf(kmax, tail);
  return (powf(kcap, tail + 1.f) - kmax * kpt) / (kpt * (tail + 1.f));
}

// 1-D bulk copies (TMA) into shared memory completing on an mbarrier, and
// the bounded wait for them (about 2 s of clock)
__device__ __forceinline__ uint32_t adv_smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void adv_mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void adv_mbar_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void adv_bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ bool adv_mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool adv_mbar_wait(uint32_t bar, uint32_t parity, long long limit_cycles) {
  if (adv_mbar_try(bar, parity)) return true;
  const long long t0 = clock64();
  while (!adv_mbar_try(bar, parity))
    if (clock64() - t0 > limit_cycles) return false;
  return true;
}

// Own-row staging of the TMA forms of the propagation and the dts pre-pass:
// each level's rows of the CTA's 64 points (two blocks, one contiguous
// region per array) land in shared memory by bulk copies issued one level
// ahead, into two alternating buffers, each completing on its own mbarrier.
struct OwnStage {
  float* buf;     // [2 buffers][arrays][2 blocks][P][32]
  uint32_t mbar;  // two mbarriers, 8 bytes apart
};


}  // namespace umwm
