// Host side of the source-term surrogate (see surrogate.hpp): parameters and
// Adam state on the device, the store of captured (state, next-step) pairs,
// training on the GPU with the tensor-core GEMMs, inference inside a model
// substep, and the C ABI entry points umwm_gpu_surrogate_*.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/umwm_gpu.h"
#include "mlp.hpp"
#include "surrogate.hpp"

namespace umwm {
namespace sur {
namespace {

using bf16 = __nv_bfloat16;

// parameter layout (f32, contiguous): W1 [HID x FPAD], b1 [HID], W2 [HID x HID],
// b2 [HID], W3 [FPAD x HID], b3 [FPAD]
constexpr long OFF_W1 = 0;
constexpr long OFF_B1 = OFF_W1 + (long)HID * FPAD;
constexpr long OFF_W2 = OFF_B1 + HID;
constexpr long OFF_B2 = OFF_W2 + (long)HID * HID;
constexpr long OFF_W3 = OFF_B2 + HID;
constexpr long OFF_B3 = OFF_W3 + (long)FPAD * HID;
constexpr long NPARAM = OFF_B3 + FPAD;
constexpr int ROW_CHUNK = 4 << 20;  // GEMM rows per launch (grid y <= 65535 tiles)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  ~DevBuf() { release(); }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct State {
  bool init = false;
  int O = 0, P = 0, F0 = 0;
  long adam_t = 0;
  DevBuf w, g, m, v;             // f32 parameters, gradients, Adam moments
  DevBuf W1, W2, W3, W2t, W3t;   // bf16 copies
  int* d_err = nullptr;          // GEMM wait timeout flag
  cudaStream_t st = nullptr;     // stream of standalone calls (training, forward, grad)
  // pair store
  DevBuf sX, sT;
  long cap = 0, count = 0;
  long holdout = 0;  // trailing stored pairs kept out of training
  bool loss_weighted = false;  // option "surrogate_loss_weight": energy-weighted loss
  int per_substep = 0;
  bool capture_on = false;
  DevBuf c_pts, c_shift, c_ecopy;
  std::vector<int> h_pts;
  int c_n = 0;
  uint64_t rng = 0x9e3779b97f4a7c15ull;
  // inference inside the model
  bool active = false;
  float tol = 0.02f;        // total-energy budget per substep (ln)
  float tol_level = 0.1f;   // per-level energy budget per substep (ln)
  DevBuf iX, iH1, iH2, fb_pt, fb_tile, counts;
  unsigned long long applied = 0, fallback = 0;
  // per-stage CUDA-event timing of the surrogate step (option "surrogate_timing")
  bool timing = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ev_pending = false;
  double ms_features = 0, ms_gemm = 0, ms_apply = 0;
  long long timed_steps = 0;
  long long rows_gemm = 0;
  // training batch buffers
  DevBuf bX, bT, Z1, H1, Z2, H2, Yf, dY, dZ2, dZ1, dYt, H2t, dZ2t, H1t, dZ1t, Xt, bidx, loss;
};

State S;

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double uniform(uint64_t& x) { return ((splitmix(x) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
double normal(uint64_t& x) {
  const double u1 = uniform(x), u2 = uniform(x);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

int cuda_fail(cudaError_t e, const char* what) {
  return set_error(UMWM_ERR_CUDA, std::string("surrogate: ") + what + ": " + cudaGetErrorString(e));
}

#define SCU(x)                                   \
  do {                                           \
    cudaError_t e_ = (x);                        \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x); \
  } while (0)

int ensure_common() {
  if (!S.st) SCU(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
  if (!S.d_err) {
    SCU(cudaMalloc(&S.d_err, sizeof(int)));
    SCU(cudaMemset(S.d_err, 0, sizeof(int)));
  }
  return UMWM_OK;
}

int check_err() {
  int h = 0;
  SCU(cudaMemcpy(&h, S.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    cudaMemset(S.d_err, 0, sizeof(int));
    return set_error(UMWM_ERR_TIMEOUT, "surrogate: a bounded wait of the tensor-core GEMM gave up");
  }
  return UMWM_OK;
}

// bf16 copies of the weights (and the transposes the backward pass uses)
int refresh_bf16(cudaStream_t st) {
  const float* w = S.w.as<float>();
  SCU(launch_to_bf16(w + OFF_W1, HID, FPAD, S.W1.as<bf16>(), nullptr, st));
  SCU(launch_to_bf16(w + OFF_W2, HID, HID, S.W2.as<bf16>(), S.W2t.as<bf16>(), st));
  SCU(launch_to_bf16(w + OFF_W3, FPAD, HID, S.W3.as<bf16>(), S.W3t.as<bf16>(), st));
  return UMWM_OK;
}

int gemm(const bf16* A, const bf16* B, int M, int N, int K, int epi, void* out, int ldo, const float* bias,
         const bf16* zin, bf16* zout, int ldz, cudaStream_t st) {
  // rows in chunks: the launch grid holds at most 65535 row tiles
  for (int r0 = 0; r0 < M; r0 += ROW_CHUNK) {
    const int m = std::min(ROW_CHUNK, M - r0);
    tc::EpiArgs ep{};
    const size_t esz = (epi == tc::EPI_F32 || epi == tc::EPI_F32_ACC) ? 4 : 2;
    ep.out = static_cast<char*>(out) + (size_t)r0 * ldo * esz;
    ep.ldo = ldo;
    ep.bias = bias;
    ep.zin = zin ? zin + (size_t)r0 * ldz : nullptr;
    ep.zout = zout ? zout + (size_t)r0 * ldz : nullptr;
    ep.ldz = ldz;
    SCU(gemm_bf16(A + (size_t)r0 * K, B, m, N, K, epi, ep, S.d_err, st));
  }
  return UMWM_OK;
}

// Forward pass over n rows of X (bf16, n x FPAD).  Training: keeps Z1, Z2
// and writes f32 outputs to Yf; inference: bf16 outputs to Ybf.
int forward(const bf16* X, int n, bf16* H1, bf16* H2, bf16* Z1, bf16* Z2, float* Yf, bf16* Ybf, cudaStream_t st) {
  const float* w = S.w.as<float>();
  int rc;
  if ((rc = gemm(X, S.W1.as<bf16>(), n, HID, FPAD, tc::EPI_BF16_GELU, H1, HID, w + OFF_B1, nullptr, Z1, HID, st)))
    return rc;
  if ((rc = gemm(H1, S.W2.as<bf16>(), n, HID, HID, tc::EPI_BF16_GELU, H2, HID, w + OFF_B2, nullptr, Z2, HID, st)))
    return rc;
  if (Yf) return gemm(H2, S.W3.as<bf16>(), n, FPAD, HID, tc::EPI_F32, Yf, FPAD, w + OFF_B3, nullptr, nullptr, 0, st);
  return gemm(H2, S.W3.as<bf16>(), n, FPAD, HID, tc::EPI_BF16, Ybf, FPAD, w + OFF_B3, nullptr, nullptr, 0, st);
}

int ensure_batch(int B) {
  const size_t b = (size_t)B;
  SCU(S.bX.ensure(b * FPAD * 2));
  SCU(S.bT.ensure(b * FPAD * 2));
  for (DevBuf* d : {&S.Z1, &S.H1, &S.Z2, &S.H2, &S.dZ2, &S.dZ1, &S.H2t, &S.dZ2t, &S.H1t, &S.dZ1t})
    SCU(d->ensure(b * HID * 2));
  SCU(S.Yf.ensure(b * FPAD * 4));
  SCU(S.dY.ensure(b * FPAD * 2));
  SCU(S.dYt.ensure(b * FPAD * 2));
  SCU(S.Xt.ensure(b * FPAD * 2));
  SCU(S.loss.ensure(sizeof(float)));
  return UMWM_OK;
}

// Loss and gradients of the batch in bX/bT (B rows) into S.g; loss added to *dloss.
int backward(int B, float* dloss, cudaStream_t st) {
  int rc;
  float* g = S.g.as<float>();
  if ((rc = forward(S.bX.as<bf16>(), B, S.H1.as<bf16>(), S.H2.as<bf16>(), S.Z1.as<bf16>(), S.Z2.as<bf16>(),
                    S.Yf.as<float>(), nullptr, st)))
    return rc;
  SCU(launch_loss(S.Yf.as<float>(), S.bT.as<bf16>(), S.loss_weighted ? S.bX.as<bf16>() : nullptr, B, S.F0,
                  S.dY.as<bf16>(), dloss, st));
  // layer 3
  SCU(launch_transpose(S.dY.as<bf16>(), B, FPAD, S.dYt.as<bf16>(), st));
  SCU(launch_transpose(S.H2.as<bf16>(), B, HID, S.H2t.as<bf16>(), st));
  if ((rc = gemm(S.dYt.as<bf16>(), S.H2t.as<bf16>(), FPAD, HID, B, tc::EPI_F32, g + OFF_W3, HID, nullptr, nullptr,
                 nullptr, 0, st)))
    return rc;
  SCU(launch_colsum(S.dY.as<bf16>(), B, FPAD, g + OFF_B3, st));
  if ((rc = gemm(S.dY.as<bf16>(), S.W3t.as<bf16>(), B, HID, FPAD, tc::EPI_BF16_DGELU, S.dZ2.as<bf16>(), HID, nullptr,
                 S.Z2.as<bf16>(), nullptr, HID, st)))
    return rc;
  // layer 2
  SCU(launch_transpose(S.dZ2.as<bf16>(), B, HID, S.dZ2t.as<bf16>(), st));
  SCU(launch_transpose(S.H1.as<bf16>(), B, HID, S.H1t.as<bf16>(), st));
  if ((rc = gemm(S.dZ2t.as<bf16>(), S.H1t.as<bf16>(), HID, HID, B, tc::EPI_F32, g + OFF_W2, HID, nullptr, nullptr,
                 nullptr, 0, st)))
    return rc;
  SCU(launch_colsum(S.dZ2.as<bf16>(), B, HID, g + OFF_B2, st));
  if ((rc = gemm(S.dZ2.as<bf16>(), S.W2t.as<bf16>(), B, HID, HID, tc::EPI_BF16_DGELU, S.dZ1.as<bf16>(), HID, nullptr,
                 S.Z1.as<bf16>(), nullptr, HID, st)))
    return rc;
  // layer 1
  SCU(launch_transpose(S.dZ1.as<bf16>(), B, HID, S.dZ1t.as<bf16>(), st));
  SCU(launch_transpose(S.bX.as<bf16>(), B, FPAD, S.Xt.as<bf16>(), st));
  if ((rc = gemm(S.dZ1t.as<bf16>(), S.Xt.as<bf16>(), HID, FPAD, B, tc::EPI_F32, g + OFF_W1, FPAD, nullptr, nullptr,
                 nullptr, 0, st)))
    return rc;
  SCU(launch_colsum(S.dZ1.as<bf16>(), B, HID, g + OFF_B1, st));
  return UMWM_OK;
}

// accumulate the stage times of the last timed step (its events are complete
// once the stream has been synchronised)
void collect_timing() {
  if (!S.ev_pending) return;
  if (cudaEventSynchronize(S.ev[3]) != cudaSuccess) return;
  float a = 0, b = 0, c = 0;
  cudaEventElapsedTime(&a, S.ev[0], S.ev[1]);
  cudaEventElapsedTime(&b, S.ev[1], S.ev[2]);
  cudaEventElapsedTime(&c, S.ev[2], S.ev[3]);
  S.ms_features += a;
  S.ms_gemm += b;
  S.ms_apply += c;
  S.timed_steps += 1;
  S.ev_pending = false;
}

int need_init() {
  if (!S.init) return set_error(UMWM_ERR_STATE, "surrogate: call umwm_gpu_surrogate_init first");
  return UMWM_OK;
}

}  // namespace

// ---- hooks of the model driver ----------------------------------------------

bool capturing() { return S.init && S.capture_on && S.count < S.cap; }
bool active() { return S.init && S.active; }

int capture_before(const Params& prm, const Ptrs& P, const std::vector<std::pair<int, int>>& wet, cudaStream_t st) {
  S.c_n = 0;
  if (!capturing()) return UMWM_OK;
  if (prm.O != S.O || prm.P != S.P)
    return set_error(UMWM_ERR_UNSUPPORTED, "surrogate: spectral grid differs from the network's");
  long total = 0;
  for (auto& r : wet) total += r.second;
  if (total <= 0) return UMWM_OK;
  const int n = (int)std::min<long>(S.per_substep, S.cap - S.count);
  S.h_pts.resize(n);
  for (int i = 0; i < n; ++i) {
    long k = (long)(uniform(S.rng) * total);
    if (k >= total) k = total - 1;
    for (auto& r : wet) {
      if (k < r.second) {
        S.h_pts[i] = r.first + (int)k;
        break;
      }
      k -= r.second;
    }
  }
  SCU(S.c_pts.ensure((size_t)n * 4));
  SCU(S.c_shift.ensure((size_t)n * 4));
  SCU(S.c_ecopy.ensure((size_t)n * S.F0 * 4));
  SCU(cudaMemcpyAsync(S.c_pts.p, S.h_pts.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
  SCU(launch_features(prm, P, S.c_pts.as<int>(), n, S.sX.as<bf16>() + (size_t)S.count * FPAD, S.c_ecopy.as<float>(),
                      S.c_shift.as<int>(), st));
  SCU(cudaStreamSynchronize(st));  // h_pts is reused by the next capture
  S.c_n = n;
  return UMWM_OK;
}

int capture_after(const Params& prm, const Ptrs& P, cudaStream_t st) {
  if (S.c_n <= 0) return UMWM_OK;
  SCU(launch_targets(prm, P, S.c_pts.as<int>(), S.c_n, S.c_ecopy.as<float>(), S.c_shift.as<int>(),
                     S.sT.as<bf16>() + (size_t)S.count * FPAD, st));
  S.count += S.c_n;
  S.c_n = 0;
  return UMWM_OK;
}

int step(const Params& prm, const Ptrs& P, Ptrs& fbP, cudaStream_t st) {
  if (prm.O != S.O || prm.P != S.P)
    return set_error(UMWM_ERR_UNSUPPORTED, "surrogate: spectral grid differs from the network's");
  const size_t n = (size_t)prm.ldN;
  SCU(S.iX.ensure(n * FPAD * 2));
  SCU(S.iH1.ensure(n * HID * 2));
  SCU(S.iH2.ensure(n * HID * 2));
  SCU(S.fb_pt.ensure(n));
  SCU(S.fb_tile.ensure((size_t)prm.ntiles * 4));
  if (!S.counts.p) {
    SCU(S.counts.ensure(2 * sizeof(unsigned long long)));
    SCU(cudaMemsetAsync(S.counts.p, 0, 2 * sizeof(unsigned long long), st));
  }
  collect_timing();
  if (S.timing && !S.ev[0])
    for (cudaEvent_t& e : S.ev) SCU(cudaEventCreate(&e));
  if (S.timing) SCU(cudaEventRecord(S.ev[0], st));
  SCU(launch_features(prm, P, nullptr, (int)n, S.iX.as<bf16>(), nullptr, nullptr, st));
  if (S.timing) SCU(cudaEventRecord(S.ev[1], st));
  int rc = forward(S.iX.as<bf16>(), (int)n, S.iH1.as<bf16>(), S.iH2.as<bf16>(), nullptr, nullptr, nullptr,
                   S.iX.as<bf16>(), st);  // outputs overwrite the inputs
  if (rc) return rc;
  if (S.timing) SCU(cudaEventRecord(S.ev[2], st));
  SCU(cudaMemsetAsync(S.fb_tile.p, 0, (size_t)prm.ntiles * 4, st));
  SCU(launch_apply(prm, P, S.iX.as<bf16>(), S.tol, S.tol_level, S.fb_pt.as<unsigned char>(), S.fb_tile.as<int>(),
                   S.counts.as<unsigned long long>(), st));
  if (S.timing) {
    SCU(cudaEventRecord(S.ev[3], st));
    S.ev_pending = true;
    S.rows_gemm = (long long)n;
  }
  fbP = P;
  fbP.fb_tile = S.fb_tile.as<int>();
  fbP.fb_pt = S.fb_pt.as<unsigned char>();
  return UMWM_OK;
}

void release_model_buffers() {
  for (DevBuf* d : {&S.iX, &S.iH1, &S.iH2, &S.fb_pt, &S.fb_tile, &S.c_pts, &S.c_shift, &S.c_ecopy}) d->release();
}

int set_option(const std::string& name, double value) {
  if (name == "surrogate") {
    if (value != 0 && !S.init) return need_init();
    S.active = value != 0;
    return UMWM_OK;
  }
  if (name == "surrogate_timing") {
    collect_timing();
    S.timing = value != 0;
    S.ms_features = S.ms_gemm = S.ms_apply = 0;
    S.timed_steps = 0;
    return UMWM_OK;
  }
  if (name == "surrogate_loss_weight") {  // 1: energy-weighted training loss (energy_weight)
    S.loss_weighted = value != 0;
    return UMWM_OK;
  }
  if (name == "surrogate_holdout") {
    if (value < 0) return set_error(UMWM_ERR_ARG, "surrogate_holdout must be >= 0");
    S.holdout = (long)value;
    return UMWM_OK;
  }
  if (name == "surrogate_tol_level") {
    if (!(value > 0)) return set_error(UMWM_ERR_ARG, "surrogate_tol_level must be > 0");
    S.tol_level = (float)value;
    return UMWM_OK;
  }
  if (name == "surrogate_tol") {
    if (!(value > 0)) return set_error(UMWM_ERR_ARG, "surrogate_tol must be > 0");
    S.tol = (float)value;
    return UMWM_OK;
  }
  return set_error(UMWM_ERR_ARG, "set_option: unknown option " + name);
}

double get_stat(const std::string& name) {
  if (name == "surrogate_nparams") return (double)NPARAM;
  if (name == "surrogate_pairs") return (double)S.count;
  if (name == "surrogate_width") return (double)FPAD;
  if (name.compare(0, 13, "surrogate_ms_") == 0 || name == "surrogate_timed_steps" || name == "surrogate_rows") {
    collect_timing();
    if (name == "surrogate_ms_features") return S.ms_features;
    if (name == "surrogate_ms_gemm") return S.ms_gemm;
    if (name == "surrogate_ms_apply") return S.ms_apply;
    if (name == "surrogate_rows") return (double)S.rows_gemm;
    return (double)S.timed_steps;
  }
  if (name == "surrogate_points" || name == "surrogate_fallback") {
    if (S.counts.p) {
      unsigned long long c[2] = {0, 0};
      if (cudaMemcpy(c, S.counts.p, sizeof(c), cudaMemcpyDeviceToHost) == cudaSuccess) {
        S.applied = c[0];
        S.fallback = c[1];
      }
    }
    return name == "surrogate_points" ? (double)(S.applied + S.fallback) : (double)S.fallback;
  }
  return -1.0;
}

}  // namespace sur
}  // namespace umwm

using namespace umwm;
using namespace umwm::sur;

extern "C" {

int umwm_gpu_surrogate_init(int om, int pm, unsigned long long seed) {
  if (om <= 0 || pm <= 0 || om * pm + NEXTRA > FPAD)
    return set_error(UMWM_ERR_UNSUPPORTED, "surrogate_init: om*pm + 9 must be <= 1344");
  int rc = ensure_common();
  if (rc) return rc;
  S.O = om;
  S.P = pm;
  S.F0 = om * pm;
  S.adam_t = 0;
  for (DevBuf* d : {&S.w, &S.g, &S.m, &S.v}) SCU(d->ensure(NPARAM * 4));
  SCU(S.W1.ensure((size_t)HID * FPAD * 2));
  SCU(S.W2.ensure((size_t)HID * HID * 2));
  SCU(S.W2t.ensure((size_t)HID * HID * 2));
  SCU(S.W3.ensure((size_t)FPAD * HID * 2));
  SCU(S.W3t.ensure((size_t)FPAD * HID * 2));
  // He initialisation for the GELU layers, a small output layer (the
  // untrained network predicts a near-zero tendency)
  std::vector<float> h(NPARAM, 0.f);
  uint64_t r = seed ^ 0x5851f42d4c957f2dull;
  const int fin1 = S.F0 + NEXTRA;
  for (int o = 0; o < HID; ++o)
    for (int i = 0; i < fin1; ++i) h[OFF_W1 + (long)o * FPAD + i] = (float)(normal(r) * std::sqrt(2.0 / fin1));
  for (long i = 0; i < (long)HID * HID; ++i) h[OFF_W2 + i] = (float)(normal(r) * std::sqrt(2.0 / HID));
  for (int o = 0; o < S.F0; ++o)
    for (int i = 0; i < HID; ++i) h[OFF_W3 + (long)o * HID + i] = (float)(normal(r) * 0.1 * std::sqrt(1.0 / HID));
  SCU(cudaMemcpy(S.w.p, h.data(), NPARAM * 4, cudaMemcpyHostToDevice));
  SCU(cudaMemset(S.m.p, 0, NPARAM * 4));
  SCU(cudaMemset(S.v.p, 0, NPARAM * 4));
  SCU(cudaMemset(S.g.p, 0, NPARAM * 4));
  if ((rc = refresh_bf16(S.st))) return rc;
  SCU(cudaStreamSynchronize(S.st));
  S.init = true;
  return UMWM_OK;
}

int umwm_gpu_surrogate_get_params(float* out, long n) {
  int rc = need_init();
  if (rc) return rc;
  if (!out || n != NPARAM) return set_error(UMWM_ERR_ARG, "surrogate_get_params: n must equal the parameter count");
  SCU(cudaMemcpy(out, S.w.p, NPARAM * 4, cudaMemcpyDeviceToHost));
  return UMWM_OK;
}

int umwm_gpu_surrogate_set_params(const float* in, long n) {
  int rc = need_init();
  if (rc) return rc;
  if (!in || n != NPARAM) return set_error(UMWM_ERR_ARG, "surrogate_set_params: n must equal the parameter count");
  SCU(cudaMemcpy(S.w.p, in, NPARAM * 4, cudaMemcpyHostToDevice));
  if ((rc = refresh_bf16(S.st))) return rc;
  SCU(cudaStreamSynchronize(S.st));
  return UMWM_OK;
}

int umwm_gpu_surrogate_capture(long capacity, int points_per_substep) {
  int rc = need_init();
  if (rc) return rc;
  if (capacity < 0 || points_per_substep < 0) return set_error(UMWM_ERR_ARG, "surrogate_capture: negative size");
  if (capacity == 0) {
    S.capture_on = false;
    return UMWM_OK;
  }
  if (capacity != S.cap) {
    SCU(S.sX.ensure((size_t)capacity * FPAD * 2));
    SCU(S.sT.ensure((size_t)capacity * FPAD * 2));
    S.cap = capacity;
    S.count = 0;
  }
  S.per_substep = points_per_substep;
  S.capture_on = points_per_substep > 0;
  return UMWM_OK;
}

int umwm_gpu_surrogate_train(int steps, int batch, double lr, unsigned long long seed, float* losses) {
  int rc = need_init();
  if (rc) return rc;
  if (steps <= 0 || batch <= 0 || batch % 128) return set_error(UMWM_ERR_ARG, "surrogate_train: batch % 128 != 0");
  const long ntrain = S.count - std::min(S.holdout, S.count);
  if (ntrain < batch) return set_error(UMWM_ERR_STATE, "surrogate_train: fewer training pairs than one batch");
  if ((rc = ensure_batch(batch))) return rc;
  SCU(S.bidx.ensure((size_t)batch * 4));
  DevBuf dl;
  SCU(dl.ensure((size_t)steps * 4));
  SCU(cudaMemsetAsync(dl.p, 0, (size_t)steps * 4, S.st));
  std::vector<int> idx(batch);
  int* hidx = nullptr;
  SCU(cudaMallocHost(&hidx, (size_t)batch * 4 * 2));
  uint64_t r = seed;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int s = 0; s < steps && rc == UMWM_OK; ++s) {
    int* hb = hidx + (s & 1) * batch;  // double-buffered host indices
    if (s >= 2) {
      cudaError_t e = cudaStreamSynchronize(S.st);
      if (e != cudaSuccess) { rc = cuda_fail(e, "train sync"); break; }
    }
    for (int i = 0; i < batch; ++i) hb[i] = (int)std::min<long>((long)(uniform(r) * ntrain), ntrain - 1);
    cudaError_t e = cudaMemcpyAsync(S.bidx.p, hb, (size_t)batch * 4, cudaMemcpyHostToDevice, S.st);
    if (e == cudaSuccess) e = launch_gather_rows(S.sX.as<bf16>(), S.bidx.as<int>(), batch, FPAD, S.bX.as<bf16>(), S.st);
    if (e == cudaSuccess) e = launch_gather_rows(S.sT.as<bf16>(), S.bidx.as<int>(), batch, FPAD, S.bT.as<bf16>(), S.st);
    if (e != cudaSuccess) { rc = cuda_fail(e, "train gather"); break; }
    if ((rc = backward(batch, dl.as<float>() + s, S.st))) break;
    ++S.adam_t;
    const float c1 = 1.f - std::pow(b1, (float)S.adam_t), c2 = 1.f - std::pow(b2, (float)S.adam_t);
    e = launch_adam(S.w.as<float>(), S.g.as<float>(), S.m.as<float>(), S.v.as<float>(), NPARAM, (float)lr, b1, b2,
                    1e-8f, c1, c2, S.st);
    if (e != cudaSuccess) { rc = cuda_fail(e, "adam"); break; }
    rc = refresh_bf16(S.st);
  }
  cudaError_t e = cudaStreamSynchronize(S.st);
  cudaFreeHost(hidx);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "train");
  if ((rc = check_err())) return rc;
  if (losses) SCU(cudaMemcpy(losses, dl.p, (size_t)steps * 4, cudaMemcpyDeviceToHost));
  dl.release();
  return UMWM_OK;
}

int umwm_gpu_surrogate_eval(long first, long count, double* loss) {
  int rc = need_init();
  if (rc) return rc;
  if (!loss || first < 0 || count <= 0 || first + count > S.count)
    return set_error(UMWM_ERR_ARG, "surrogate_eval: rows outside the stored pairs");
  const int B = 8192;
  if ((rc = ensure_batch(B))) return rc;
  DevBuf dl, idx;
  const long nb = (count + B - 1) / B;
  SCU(dl.ensure((size_t)nb * 4));
  SCU(idx.ensure((size_t)B * 4));
  SCU(cudaMemsetAsync(dl.p, 0, (size_t)nb * 4, S.st));
  std::vector<int> h(B);
  for (long b = 0; b < nb; ++b) {
    const int n = (int)std::min<long>(B, count - b * B);
    for (int i = 0; i < n; ++i) h[i] = (int)(first + b * B + i);
    SCU(cudaMemcpyAsync(idx.p, h.data(), (size_t)n * 4, cudaMemcpyHostToDevice, S.st));
    SCU(launch_gather_rows(S.sX.as<bf16>(), idx.as<int>(), n, FPAD, S.bX.as<bf16>(), S.st));
    SCU(launch_gather_rows(S.sT.as<bf16>(), idx.as<int>(), n, FPAD, S.bT.as<bf16>(), S.st));
    if ((rc = forward(S.bX.as<bf16>(), n, S.H1.as<bf16>(), S.H2.as<bf16>(), S.Z1.as<bf16>(), S.Z2.as<bf16>(),
                      S.Yf.as<float>(), nullptr, S.st)))
      return rc;
    SCU(launch_loss(S.Yf.as<float>(), S.bT.as<bf16>(), S.loss_weighted ? S.bX.as<bf16>() : nullptr, n, S.F0,
                    S.dY.as<bf16>(), dl.as<float>() + b, S.st));
    SCU(cudaStreamSynchronize(S.st));  // h is reused
  }
  std::vector<float> l(nb);
  SCU(cudaMemcpy(l.data(), dl.p, (size_t)nb * 4, cudaMemcpyDeviceToHost));
  double acc = 0;
  for (long b = 0; b < nb; ++b) acc += (double)l[b] * std::min<long>(B, count - b * B);
  *loss = acc / count;
  return check_err();
}

int umwm_gpu_surrogate_forward(const float* X, int n, float* Y) {
  int rc = need_init();
  if (rc) return rc;
  if (!X || !Y || n <= 0) return set_error(UMWM_ERR_ARG, "surrogate_forward: bad arguments");
  if ((rc = ensure_batch(n))) return rc;
  DevBuf xf;
  SCU(xf.ensure((size_t)n * FPAD * 4));
  SCU(cudaMemcpyAsync(xf.p, X, (size_t)n * FPAD * 4, cudaMemcpyHostToDevice, S.st));
  SCU(launch_f32_to_bf16(xf.as<float>(), (long)n * FPAD, S.bX.as<bf16>(), S.st));
  if ((rc = forward(S.bX.as<bf16>(), n, S.H1.as<bf16>(), S.H2.as<bf16>(), S.Z1.as<bf16>(), S.Z2.as<bf16>(),
                    S.Yf.as<float>(), nullptr, S.st)))
    return rc;
  SCU(cudaMemcpyAsync(Y, S.Yf.p, (size_t)n * FPAD * 4, cudaMemcpyDeviceToHost, S.st));
  SCU(cudaStreamSynchronize(S.st));
  xf.release();
  return check_err();
}

int umwm_gpu_surrogate_grad(const float* X, const float* T, int n, float* loss, float* grad) {
  int rc = need_init();
  if (rc) return rc;
  if (!X || !T || n <= 0 || n % 64) return set_error(UMWM_ERR_ARG, "surrogate_grad: n must be a multiple of 64");
  if ((rc = ensure_batch(n))) return rc;
  DevBuf xf;
  SCU(xf.ensure((size_t)n * FPAD * 4));
  SCU(cudaMemcpyAsync(xf.p, X, (size_t)n * FPAD * 4, cudaMemcpyHostToDevice, S.st));
  SCU(launch_f32_to_bf16(xf.as<float>(), (long)n * FPAD, S.bX.as<bf16>(), S.st));
  SCU(cudaMemcpyAsync(xf.p, T, (size_t)n * FPAD * 4, cudaMemcpyHostToDevice, S.st));
  SCU(launch_f32_to_bf16(xf.as<float>(), (long)n * FPAD, S.bT.as<bf16>(), S.st));
  SCU(cudaMemsetAsync(S.loss.p, 0, sizeof(float), S.st));
  if ((rc = backward(n, S.loss.as<float>(), S.st))) return rc;
  if (loss) SCU(cudaMemcpyAsync(loss, S.loss.p, sizeof(float), cudaMemcpyDeviceToHost, S.st));
  if (grad) SCU(cudaMemcpyAsync(grad, S.g.p, NPARAM * 4, cudaMemcpyDeviceToHost, S.st));
  SCU(cudaStreamSynchronize(S.st));
  xf.release();
  return check_err();
}

int umwm_gpu_gemm_bf16(const unsigned short* A, const unsigned short* B, float* C, int M, int N, int K) {
  if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || K % 64 || N % 32)
    return set_error(UMWM_ERR_ARG, "gemm_bf16: K % 64 == 0 and N % 32 == 0 required");
  int rc = ensure_common();
  if (rc) return rc;
  DevBuf a, b, c;
  SCU(a.ensure((size_t)M * K * 2));
  SCU(b.ensure((size_t)N * K * 2));
  SCU(c.ensure((size_t)M * N * 4));
  SCU(cudaMemcpyAsync(a.p, A, (size_t)M * K * 2, cudaMemcpyHostToDevice, S.st));
  SCU(cudaMemcpyAsync(b.p, B, (size_t)N * K * 2, cudaMemcpyHostToDevice, S.st));
  if ((rc = gemm(a.as<bf16>(), b.as<bf16>(), M, N, K, tc::EPI_F32, c.p, N, nullptr, nullptr, nullptr, 0, S.st)))
    return rc;
  SCU(cudaMemcpyAsync(C, c.p, (size_t)M * N * 4, cudaMemcpyDeviceToHost, S.st));
  SCU(cudaStreamSynchronize(S.st));
  a.release();
  b.release();
  c.release();
  return check_err();
}

}  // extern "C"
