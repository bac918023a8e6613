// Kernels of the source-term surrogate around the tensor-core GEMMs: input
// features from the spectrum, targets of captured training pairs, the
// apply step with its energy-budget monitor, and the training helpers
// (row gather, transpose, loss, column sums, Adam, bf16 conversion).
#include <cfloat>
#include <cstdint>

#include "dev_common.cuh"
#include "surrogate.hpp"

namespace umwm {
namespace sur {

namespace {

constexpr int UNR = 12;                // spectrum loads in flight per warp in the bin loops
constexpr int FLC = 8;                 // levels per chunk of k_features (one per warp)
constexpr int FPITCHW = FLC * MAX_PM / 2 + 1;  // words per row of k_features' chunk tile (odd)

struct PointInfo {
  int j, ok, s;
  float psi;
};

// Validity, rotation and wind direction of global point j.
__device__ __forceinline__ PointInfo point_info(const Params& prm, const Ptrs& P, int j) {
  PointInfo q{j, 0, 0, 0.f};
  if (j < 0 || j >= prm.Ntot) return q;
  const Member& M = prm.mem[prm.tile_mem[j / TILE]];
  if (j >= M.off + M.N || !M.ctl->running) return q;
  q.ok = 1;
  q.psi = P.wdir[apt(M, j)];
  int s = static_cast<int>(floorf((q.psi - prm.th[0]) / prm.dth + 0.5f)) % prm.P;
  if (s < 0) s += prm.P;
  q.s = s;
  return q;
}

__device__ __forceinline__ float feature(float e) { return (logf(fmaxf(e, 0.f) + EPS) - LN_C0) * (1.f / LN_C1); }

// Growth allowance of the surrogate step (k_apply): a bin's predicted
// log-tendency is capped by dts * max(Sin, 0) + GROWTH_SLACK.  Without wind
// input a bin cannot grow in the plain step, so the cap stops a network
// error from feeding energy into bins the forcing does not reach.
constexpr float GROWTH_SLACK = 0.02f;

}  // namespace

// Input rows of 32 points per CTA (8 warps).  Warp 0 finds each row's
// point, rotation and extra features.  The spectrum part goes level chunk
// by level chunk (FLC levels, FLC * pm columns of every row): warp w takes
// level w of the chunk, lane = row, and walks the directions (UNR loads in
// flight), writing the rotated bf16 features into a shared-memory tile; the
// tile's row segments then go out as 32-bit words, coalesced along each
// row.  For the inference rows (pts == nullptr, row r = point r) a level's
// row of 32 points is one 128-byte line per direction.
__global__ void __launch_bounds__(256) k_features(const Params prm, const Ptrs P, const int* pts, int n,
                                                  __nv_bfloat16* X, float* ecopy, int* shift) {
  __shared__ uint32_t tile[32 * FPITCHW];
  __shared__ int s_j[32], s_ok[32], s_s[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r0 = blockIdx.x * 32;
  const int NP = prm.P, F0 = prm.O * prm.P;
  if (warp == 0) {
    const int r = r0 + lane;
    PointInfo q{-1, 0, 0, 0.f};
    if (r < n) q = point_info(prm, P, pts ? pts[r] : r);
    s_j[lane] = q.j;
    s_ok[lane] = q.ok;
    s_s[lane] = q.s;
    if (shift && r < n) shift[r] = q.ok ? q.s : -1;
    float ex[NEXTRA] = {0.f};
    if (q.ok) {
      const int j = q.j;
      const Member& M = prm.mem[prm.tile_mem[j / TILE]];
      const int ja = apt(M, j);
      float d = q.psi - prm.th[q.s];
      d = d - 6.28318531f * floorf(d / 6.28318531f + 0.5f);
      const float cs = cosf(q.psi), sn = sinf(q.psi);
      ex[0] = P.wspd[ja] * (1.f / 25.f);
      ex[1] = d / prm.dth;
      ex[2] = P.ustar[j];
      ex[3] = logf(P.d[j]) * 0.125f;
      ex[4] = M.ctl->dts * (1.f / 60.f);
      ex[5] = P.uc[ja] * cs + P.vc[ja] * sn;
      ex[6] = -P.uc[ja] * sn + P.vc[ja] * cs;
      ex[7] = P.rhorat[ja] * 800.f;
      ex[8] = P.fice[ja];
    }
    if (r < n) {  // the extra features and the padding, straight to the row
      for (int c = F0; c < FPAD; ++c)
        X[(size_t)r * FPAD + c] = __float2bfloat16_rn(c - F0 < NEXTRA ? ex[c - F0] : 0.f);
    }
  }
  __syncthreads();
  const int j = s_j[lane], ok = s_ok[lane], s = s_s[lane];
  __nv_bfloat16* h = reinterpret_cast<__nv_bfloat16*>(tile + lane * FPITCHW);
  uint32_t* X32 = reinterpret_cast<uint32_t*>(X);
  for (int c0 = 0; c0 < prm.O; c0 += FLC) {
    const int nl = min(FLC, prm.O - c0);  // levels of this chunk
    const int o = c0 + warp;
    if (warp < nl) {
      const float* Er = ok ? P.E + sidx(prm, o, 0, j) : nullptr;  // direction p at Er[p * 32]
      int pr = s == 0 ? 0 : NP - s;                                  // rotated column of p = 0
      for (int p0 = 0; p0 < NP; p0 += UNR) {
        float ev[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) ev[u] = (ok && p0 + u < NP) ? __ldg(Er + (p0 + u) * 32) : 0.f;
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
          if (p0 + u >= NP) break;
          h[warp * NP + pr] = __float2bfloat16_rn(ok ? feature(ev[u]) : 0.f);
          if (ecopy && r0 + lane < n) ecopy[(size_t)(r0 + lane) * F0 + o * NP + pr] = ev[u];
          pr = pr + 1 == NP ? 0 : pr + 1;
        }
      }
    }
    __syncthreads();
    // rows r0..r0+31, columns c0 * NP .. (c0 + nl) * NP, as words
    const int nw = nl * NP / 2;
    for (int rr = warp; rr < 32; rr += 8) {
      if (r0 + rr >= n) break;
      uint32_t* dst = X32 + ((size_t)(r0 + rr) * FPAD + (size_t)c0 * NP) / 2;
      for (int k = lane; k < nw; k += 32) dst[k] = tile[rr * FPITCHW + k];
    }
    __syncthreads();
  }
}

__global__ void k_targets(const Params prm, const Ptrs P, const int* pts, int n, const float* ecopy,
                          const int* shift, __nv_bfloat16* T) {
  const int NP = prm.P, F0 = prm.O * prm.P;
  const size_t total = (size_t)n * FPAD;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = static_cast<int>(idx / FPAD), c = static_cast<int>(idx % FPAD);
    float t = 0.f;
    const int s = shift[r];
    if (c < F0 && s >= 0) {
      const int o = c / NP, pr = c - o * NP;
      int p = pr + s;
      if (p >= NP) p -= NP;
      // ef after the integration: at propagated levels 2 E* - e (e left in place)
      const size_t a = sidx(prm, o, p, pts[r]);
      const float ef = o < P.oc[pts[r]] ? 2.f * P.ES[a] - P.EF[a] : P.EF[a];
      t = (logf(fmaxf(ef, 0.f) + EPS) - logf(fmaxf(ecopy[(size_t)r * F0 + c], 0.f) + EPS)) * (1.f / TS);
    }
    T[idx] = __float2bfloat16_rn(t);
  }
}

// Apply step of one 32-point block (lane = point).  Each warp takes every
// eighth frequency level: it stages the level's row segment of each point's
// network output in shared memory (the rotation by the point's wind bin is
// then a shared-memory index), reads the level's table values once, and
// sums the level's energy before and after in registers, so no level sum
// needs an atomic.  Pass 1 forms ef for every bin and writes E* = (e + ef)/2
// and the monitor's sums; the points that pass get ef at the levels above
// the cut-off in pass 2 (E* of the failing points is rewritten by the
// fallback integration).
__global__ void __launch_bounds__(256) k_apply(const Params prm, const Ptrs P, const __nv_bfloat16* Y, float tol,
                                               float tol_level, unsigned char* fb_pt, int* fb_tile,
                                               unsigned long long* counts) {
  extern __shared__ uint32_t dyn[];
  __shared__ float red0[8][32], red1[8][32], red2[8][32], red3[8][32];
  __shared__ float lev0[MAX_OM][32], lev1[MAX_OM][32];  // energy of each frequency level before / after
  __shared__ int s_ok[32], s_s[32], s_pass[32];
  __shared__ WindIn s_wi[32];
  __shared__ float s_dts[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int jb = blockIdx.x, j = jb * 32 + lane;
  const int NP = prm.P, O = prm.O;
  const int YP = NP | 1;  // staged row pitch (odd: conflict-free columns)
  float* cwt = reinterpret_cast<float*>(dyn);                                  // [NP][32]
  uint16_t* yb = reinterpret_cast<uint16_t*>(dyn + NP * 32) + warp * 32 * YP;  // this warp's [32][YP]
  if (warp == 0) {
    const PointInfo q = point_info(prm, P, j);
    s_ok[lane] = q.ok;
    s_s[lane] = q.s;
    if (q.ok) {
      const Member& M = prm.mem[prm.tile_mem[j / TILE]];
      s_wi[lane] = load_wind(prm, P, j, apt(M, j), P.ustar[j]);
      s_dts[lane] = M.ctl->dts;
    }
    for (int p = 0; p < NP; ++p) cwt[p * 32 + lane] = q.ok ? cosf(q.psi - prm.th[p]) : 0.f;
  }
  __syncthreads();
  const int ok = s_ok[lane], s = s_s[lane];
  const WindIn wi = s_wi[lane];
  const float dts = s_dts[lane];
  const uint16_t* Yr = reinterpret_cast<const uint16_t*>(Y) + (size_t)j * FPAD;  // this point's output row
  // stage this point's output at level o (NP bf16, 4-byte aligned: NP is even)
  auto stage = [&](int o) {
    __syncwarp();
    const uint32_t* src = reinterpret_cast<const uint32_t*>(Yr + o * NP);
    for (int k = 0; k < NP / 2; ++k) {
      const uint32_t v = ok ? src[k] : 0u;
      yb[lane * YP + 2 * k] = (uint16_t)(v & 0xffffu);
      yb[lane * YP + 2 * k + 1] = (uint16_t)(v >> 16);
    }
    __syncwarp();
  };
  // ef of bin (o, p): the predicted log-tendency, capped above by the growth
  // the wind input allows over dts
  auto step = [&](int p, float e, float logl2z, float cp0, float fkovg, bool tail, float& sp) {
    int pr = p - s;
    if (pr < 0) pr += NP;
    const float y = __uint_as_float((uint32_t)yb[lane * YP + pr] << 16);
    const float cw = cwt[p * 32 + lane];
    const float x = (wi.wspd + wi.ustar25 * logl2z) * cw - cp0 - wi.uc * prm.cth[p] - wi.vc * prm.sth[p];
    sp = fmaxf(sin_fold(prm, wi.shelt, x, cw, wi.c1 * fkovg, tail), 0.f);
    const float d = fminf(TS * y, dts * sp + GROWTH_SLACK);
    return fmaxf((fmaxf(e, 0.f) + EPS) * ex2_approx(d * 1.44269504f) - EPS, 0.f);  // e^d through the SFU
  };
  float m0 = 0.f, m1 = 0.f, w0 = 0.f, w1 = 0.f;  // energy, and energy where the wind feeds (weight Sin)
  for (int o = warp; o < O; o += 8) {
    stage(o);
    const float* T = P.TAB + tidx(prm, o, 0, j);
    const float kdk = T[T_KDK * 32], logl2z = T[T_LOGL2Z * 32], cp0 = T[T_CP0 * 32], fkovg = T[T_FKOVG * 32];
    const bool tail = o >= wi.oc;
    float lv0 = 0.f, lv1 = 0.f;
    for (int p0 = 0; p0 < NP; p0 += UNR) {
      float ev[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) ev[u] = (p0 + u < NP) ? P.E[sidx(prm, o, p0 + u, j)] : 0.f;
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const int p = p0 + u;
        if (p >= NP) break;
        const float e = ev[u];
        float sp;
        const float ef = step(p, e, logl2z, cp0, fkovg, tail, sp);
        m0 += e * kdk;
        m1 += ef * kdk;
        w0 += fmaxf(e, 0.f) * sp * kdk;
        w1 += ef * sp * kdk;
        lv0 += fmaxf(e, 0.f);
        lv1 += ef;
        if (ok) P.ES[sidx(prm, o, p, j)] = 0.5f * (e + ef);
      }
    }
    lev0[o][lane] = lv0;
    lev1[o][lane] = lv1;
  }
  red0[warp][lane] = m0;
  red1[warp][lane] = m1;
  red2[warp][lane] = w0;
  red3[warp][lane] = w1;
  __syncthreads();
  if (warp == 0) {
    float a = 0.f, b = 0.f, wa = 0.f, wb = 0.f;
    for (int w = 0; w < 8; ++w) {
      a += red0[w][lane];
      b += red1[w][lane];
      wa += red2[w][lane];
      wb += red3[w][lane];
    }
    // total energy (sum e k dk, as Hs^2) within tol, and every frequency
    // level holding more than 1e-4 of the largest level's energy within
    // tol_level (the total alone hardly sees the low frequencies)
    // the wind-weighted energy (sum e max(Sin,0) k dk, which sets the form
    // stress and so ustar) within tol_level as well
    bool pass = ok && isfinite(b) && fabsf(logf((b + 1e-30f) / (a + 1e-30f))) <= tol &&
                isfinite(wb) && fabsf(logf((wb + 1e-30f) / (wa + 1e-30f))) <= tol_level;
    if (pass) {
      float lmax = 0.f;
      for (int o = 0; o < O; ++o) lmax = fmaxf(lmax, lev0[o][lane]);
      const float floor_ = 1e-4f * lmax + 1e-30f;
      for (int o = 0; o < O; ++o)
        if (!(fabsf(logf((lev1[o][lane] + floor_) / (lev0[o][lane] + floor_))) <= tol_level)) pass = false;
    }
    s_pass[lane] = pass ? 1 : 0;
    if (j < prm.Ntot) fb_pt[j] = (ok && !pass) ? 1 : 0;
    const unsigned fails = __ballot_sync(0xffffffffu, ok && !pass);
    const unsigned passes = __ballot_sync(0xffffffffu, pass);
    if (lane == 0) {
      if (fails) fb_tile[(jb * 32) / TILE] = 1;
      if (passes) atomicAdd(&counts[0], (unsigned long long)__popc(passes));
      if (fails) atomicAdd(&counts[1], (unsigned long long)__popc(fails));
    }
  }
  __syncthreads();
  // pass 2: ef above the cut-off of the passing points (as the integration:
  // E* only at the propagated levels); lanes of failing points idle in it
  const bool pass = s_pass[lane] != 0;
  if (!__any_sync(0xffffffffu, pass)) return;
  for (int o = warp; o < O; o += 8) {
    if (!__any_sync(0xffffffffu, pass && o >= wi.oc)) continue;
    stage(o);
    if (!(pass && o >= wi.oc)) continue;
    const float* T = P.TAB + tidx(prm, o, 0, j);
    const float logl2z = T[T_LOGL2Z * 32], cp0 = T[T_CP0 * 32], fkovg = T[T_FKOVG * 32];
    for (int p = 0; p < NP; ++p) {
      const size_t k = sidx(prm, o, p, j);
      float sp;
      P.EF[k] = step(p, P.E[k], logl2z, cp0, fkovg, true, sp);
    }
  }
}

// ---- training helpers ---------------------------------------------------------

__global__ void k_gather_rows(const uint4* src, const int* idx, int n, int w16, uint4* dst) {
  const size_t total = (size_t)n * w16;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = i / w16, c = i % w16;
    dst[i] = src[(size_t)idx[r] * w16 + c];
  }
}

__global__ void k_transpose(const __nv_bfloat16* src, int rows, int cols, __nv_bfloat16* dst) {
  __shared__ __nv_bfloat16 t[32][34];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[k][threadIdx.x] = src[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[(size_t)c * rows + r] = t[threadIdx.x][k];
  }
}

__global__ void k_loss(const float* Y, const __nv_bfloat16* T, const __nv_bfloat16* X, int n, int f0,
                       __nv_bfloat16* dY, float* loss) {
  __shared__ float red[256];
  const size_t total = (size_t)n * FPAD;
  const float inv = 1.f / ((float)n * f0);
  float acc = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = static_cast<int>(i % FPAD);
    const float d = c < f0 ? Y[i] - __bfloat162float(T[i]) : 0.f;
    const float w = (X && c < f0) ? energy_weight(__bfloat162float(X[i])) : 1.f;
    acc += w * (d * d);
    dY[i] = __float2bfloat16_rn(2.f * (w * d) * inv);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] * inv);
}

__global__ void k_colsum(const __nv_bfloat16* A, int rows, int cols, float* out) {
  const int c = blockIdx.x * 32 + threadIdx.x;
  const int r0 = blockIdx.y * 256;
  if (c >= cols) return;
  float acc = 0.f;
  for (int r = r0 + threadIdx.y; r < min(rows, r0 + 256); r += blockDim.y) acc += __bfloat162float(A[(size_t)r * cols + c]);
  atomicAdd(&out[c], acc);
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_to_bf16(const float* w, int rows, int cols, __nv_bfloat16* out, __nv_bfloat16* out_t) {
  const long total = (long)rows * cols;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
    out[i] = b;
    if (out_t) {
      const long r = i / cols, c = i % cols;
      out_t[c * rows + r] = b;
    }
  }
}

// ---- launchers ----------------------------------------------------------------

static int grid_for(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  if (g > 152u * 32) g = 152u * 32;
  return static_cast<int>(g < 1 ? 1 : g);
}

cudaError_t launch_features(const Params& prm, const Ptrs& P, const int* pts, int n, __nv_bfloat16* X,
                            float* ecopy, int* shift, cudaStream_t st) {
  if (prm.O * prm.P + NEXTRA > FPAD || prm.P % 2) return cudaErrorInvalidValue;
  if (n <= 0) return cudaSuccess;
  k_features<<<(n + 31) / 32, 256, 0, st>>>(prm, P, pts, n, X, ecopy, shift);
  return cudaGetLastError();
}

cudaError_t launch_targets(const Params& prm, const Ptrs& P, const int* pts, int n, const float* ecopy,
                           const int* shift, __nv_bfloat16* T, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_targets<<<grid_for((size_t)n * FPAD, 256), 256, 0, st>>>(prm, P, pts, n, ecopy, shift, T);
  return cudaGetLastError();
}

cudaError_t launch_apply(const Params& prm, const Ptrs& P, const __nv_bfloat16* Y, float tol, float tol_level,
                         unsigned char* fb_pt, int* fb_tile, unsigned long long* counts, cudaStream_t st) {
  // direction cosines [pm][32] and each warp's staged row segments [32][pm|1]
  const int smem = prm.P * 32 * 4 + 8 * 32 * (prm.P | 1) * 2;
  if (smem > 48 * 1024 || prm.P % 2) return cudaErrorInvalidConfiguration;
  k_apply<<<prm.NB, 256, smem, st>>>(prm, P, Y, tol, tol_level, fb_pt, fb_tile, counts);
  return cudaGetLastError();
}

cudaError_t launch_gather_rows(const __nv_bfloat16* src, const int* idx, int n, int width, __nv_bfloat16* dst,
                               cudaStream_t st) {
  if (width % 8) return cudaErrorInvalidValue;
  const int w16 = width / 8;
  k_gather_rows<<<grid_for((size_t)n * w16, 256), 256, 0, st>>>(reinterpret_cast<const uint4*>(src), idx, n, w16,
                                                                reinterpret_cast<uint4*>(dst));
  return cudaGetLastError();
}

cudaError_t launch_transpose(const __nv_bfloat16* src, int rows, int cols, __nv_bfloat16* dst, cudaStream_t st) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  k_transpose<<<grid, block, 0, st>>>(src, rows, cols, dst);
  return cudaGetLastError();
}

cudaError_t launch_loss(const float* Y, const __nv_bfloat16* T, const __nv_bfloat16* X, int n, int f0,
                        __nv_bfloat16* dY, float* loss, cudaStream_t st) {
  k_loss<<<grid_for((size_t)n * FPAD, 256), 256, 0, st>>>(Y, T, X, n, f0, dY, loss);
  return cudaGetLastError();
}

cudaError_t launch_colsum(const __nv_bfloat16* A, int rows, int cols, float* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, (size_t)cols * sizeof(float), st);
  if (e != cudaSuccess) return e;
  dim3 grid((cols + 31) / 32, (rows + 255) / 256), block(32, 8);
  k_colsum<<<grid, block, 0, st>>>(A, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2, float eps,
                        float c1, float c2, cudaStream_t st) {
  k_adam<<<grid_for((size_t)n, 256), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* w, int rows, int cols, __nv_bfloat16* out, __nv_bfloat16* out_t,
                           cudaStream_t st) {
  k_to_bf16<<<grid_for((size_t)rows * cols, 256), 256, 0, st>>>(w, rows, cols, out, out_t);
  return cudaGetLastError();
}

cudaError_t launch_f32_to_bf16(const float* a, long n, __nv_bfloat16* out, cudaStream_t st) {
  k_to_bf16<<<grid_for((size_t)n, 256), 256, 0, st>>>(a, 1, (int)n, out, nullptr);
  return cudaGetLastError();
}

}  // namespace sur
}  // namespace umwm
