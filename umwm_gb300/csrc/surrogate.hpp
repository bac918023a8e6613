// Learned source-term surrogate: an MLP that takes a point's log-spectrum
// (rotated into the wind frame) plus forcing and returns the point's
// source-term step as a log-tendency; a per-point energy-budget monitor
// sends points whose step leaves the budget back to the plain source
// integration.  Device kernels are in k_sur.cu, the GEMMs in k_mlp.cu, the
// host side in surrogate.cu.
//
// Features of a wet point j (row of the input matrix, bf16, width FPAD):
//   s      = index of the direction bin nearest to the wind direction wdir;
//            direction p' of the rotated frame is the model's direction
//            (p' + s) mod pm, so the wind always lies along p' = 0
//   x[o*pm + p'] = (ln(e(o, (p'+s) mod pm) + EPS) - LN_C0) / LN_C1
//   x[F0 + 0] = wspd / 25           x[F0 + 1] = (wdir - th(s)) / dth
//   x[F0 + 2] = ustar               x[F0 + 3] = ln(depth) / 8
//   x[F0 + 4] = dts / 60            x[F0 + 5] = current along the wind
//   x[F0 + 6] = current across      x[F0 + 7] = rhoa / rhow * 800
//   x[F0 + 8] = fice                the rest zero (F0 = om*pm)
// Output y (width FPAD, first F0 used) in the same rotated frame:
//   ef = max((e + EPS) exp(min(TS * y, dts max(Sin, 0) + 0.02)) - EPS, 0),
//   ES = (e + ef) / 2,   EF = ef
// i.e. the step the plain path takes in umwm_physics.F90:61-84, with growth
// capped by the bin's wind input Sin (sin_d12, umwm_source_functions.F90:39-80).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "dev.cuh"

namespace umwm {

int set_error(int code, const std::string& msg);  // umwm_gpu.cu

namespace sur {

constexpr int NEXTRA = 9;
constexpr int FPAD = 1344;   // padded feature / output width (multiple of 64)
constexpr int HID = 512;     // hidden width
constexpr float EPS = 1e-15f;
constexpr float LN_C0 = -15.f, LN_C1 = 8.f;
constexpr float TS = 2.f;    // tendency scale
// Energy weight of a target bin in the weighted loss, from its input feature
// x = (ln(e + EPS) - LN_C0) / LN_C1: a ramp in ln e from WL0 (e = 1e-9,
// weight WMIN) to WL1 (e = 1e-5, weight 1)
constexpr float WL0 = -20.7232658f, WL1 = -11.5129255f, WMIN = 0.01f;
__host__ __device__ inline float energy_weight(float x) {
  const float w = (x * LN_C1 + LN_C0 - WL0) / (WL1 - WL0);
  return w < WMIN ? WMIN : (w > 1.f ? 1.f : w);
}

// Device kernels (k_sur.cu) ---------------------------------------------------

// X rows for points pts[0..n) (pts == nullptr: row r is point r, n = ldN);
// invalid rows (padding, ghost, not running) are zero.  ecopy (optional, f32
// n x F0) receives e in the rotated frame; shift (optional) the rotation.
cudaError_t launch_features(const Params& prm, const Ptrs& P, const int* pts, int n, __nv_bfloat16* X,
                            float* ecopy, int* shift, cudaStream_t st);
// Targets of captured rows: t = (ln(ef + EPS) - ln(e + EPS)) / TS, bf16.
cudaError_t launch_targets(const Params& prm, const Ptrs& P, const int* pts, int n, const float* ecopy,
                           const int* shift, __nv_bfloat16* T, cudaStream_t st);
// Apply the predicted step (Y: ldN x FPAD bf16) to every running wet point
// whose energy budget passes: |ln(m1/m0)| <= tol, m = sum e k dk, and for
// every frequency level o holding more than 1e-4 of the point's largest
// level energy, |ln(L1_o/L0_o)| <= tol_level, L_o = sum_p e.  Failing points
// get fb_pt[j] = 1 and their tile fb_tile[t] = 1 and keep e; counts[0] +=
// points applied, [1] += points failing.
cudaError_t launch_apply(const Params& prm, const Ptrs& P, const __nv_bfloat16* Y, float tol, float tol_level,
                         unsigned char* fb_pt, int* fb_tile, unsigned long long* counts, cudaStream_t st);

// training helpers
cudaError_t launch_gather_rows(const __nv_bfloat16* src, const int* idx, int n, int width, __nv_bfloat16* dst,
                               cudaStream_t st);
cudaError_t launch_transpose(const __nv_bfloat16* src, int rows, int cols, __nv_bfloat16* dst, cudaStream_t st);
// dY = 2 w (Y - T) / (n * F0) over the first F0 columns (0 beyond);
// loss += sum w (Y-T)^2 / (n*F0).  w = 1, or with X (the batch's input rows)
// the energy weight of the bin, energy_weight(X): targets of nearly empty
// bins (whose log-tendency is noise at the EPS floor) count little
cudaError_t launch_loss(const float* Y, const __nv_bfloat16* T, const __nv_bfloat16* X, int n, int f0,
                        __nv_bfloat16* dY, float* loss, cudaStream_t st);
cudaError_t launch_colsum(const __nv_bfloat16* A, int rows, int cols, float* out, cudaStream_t st);
cudaError_t launch_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t st);
// bf16 copy of a rows x cols f32 matrix and (optional) its transpose
cudaError_t launch_to_bf16(const float* w, int rows, int cols, __nv_bfloat16* out, __nv_bfloat16* out_t,
                           cudaStream_t st);
cudaError_t launch_f32_to_bf16(const float* a, long n, __nv_bfloat16* out, cudaStream_t st);

// Hooks of the model driver (surrogate.cu) ------------------------------------

bool capturing();
bool active();
// wet: (first global index, count) of each member's wet points
int capture_before(const Params& prm, const Ptrs& P, const std::vector<std::pair<int, int>>& wet, cudaStream_t st);
int capture_after(const Params& prm, const Ptrs& P, cudaStream_t st);
// The surrogate source step of one substep; fills fbP (the Ptrs the
// fallback integration runs with: only flagged tiles and points).
int step(const Params& prm, const Ptrs& P, Ptrs& fbP, cudaStream_t st);
void release_model_buffers();  // model finalized
int set_option(const std::string& name, double value);  // "surrogate", "surrogate_tol"
double get_stat(const std::string& name);               // "surrogate_*"; -1 if unknown

}  // namespace sur
}  // namespace umwm
