// C ABI of the GB300 UMWM library (include/umwm_gpu.h): the umwm_top entry
// points, the in-memory stand-ins for the reference's input files, and the
// device-resident model.  The outer dtg loop and the inner dynamic-dts loop
// of umwm_run (umwm_top.F90:68-192) are driven from here; every per-substep
// quantity (dts, sumt, dtr, the rotation max, the screen line) stays in a
// device control block, and the host reads back one flag per substep to
// end the inner loop, or none at all when the loop runs as a CUDA graph
// with a device-side while node.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <map>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/umwm_gpu.h"
#include "host_model.hpp"
#include "kernels.hpp"
#include "ncfile.hpp"
#include "surrogate.hpp"

namespace umwm {
namespace {

std::string g_err;
Inputs g_inputs;
int g_device = -1;  // set_option("device", n) before initialize

// Per-kernel CUDA-event timing on the launching stream (option "kernel_timing").
enum KName { K_PREP, K_SICE, K_PHYS, K_DTS, K_INTEG, K_ADVECT, K_DIAG, K_SCREEN, K_STOKES, K_NK };
const char* const KNAMES[K_NK] = {"prep", "sice", "phys", "dts", "integ", "advect", "diag", "screen", "stokes"};

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CU(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) return fail(UMWM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

unsigned enc_ord_h(float x) {
  unsigned u;
  std::memcpy(&u, &x, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct Dev {
  std::vector<void*> bufs;
  template <typename T>
  cudaError_t alloc(T** p, size_t n, bool zero = true) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    bufs.push_back(q);
    if (zero) e = cudaMemset(q, 0, std::max<size_t>(n, 1) * sizeof(T));
    *p = (T*)q;
    return e;
  }
  ~Dev() {
    for (void* q : bufs) cudaFree(q);
  }
};

// One member of the model (a single domain is a one-member ensemble).
struct MemberHost {
  HostModel H;
  Inputs in;              // this member's stand-ins for the reference's files
  bool readfile = false;  // any forcing variable comes from the input files
  int off = 0, N = 0, ghost = 0, padded = 0, nmoff = 0, NM = 0;
  Ctl* ctl = nullptr;
  double* log = nullptr;
  int log_cap = 0;
  int *mi = nullptr, *ni = nullptr;
  float *uwb = nullptr, *uwf = nullptr, *vwb = nullptr, *vwf = nullptr, *ucb = nullptr, *ucf = nullptr,
        *vcb = nullptr, *vcf = nullptr, *rhoab = nullptr, *rhoaf = nullptr, *rhowb = nullptr, *rhowf = nullptr,
        *ficeb = nullptr, *ficef = nullptr;
  size_t screen_printed = 0;
  int substep_mark = 0;  // member substep counter at the start of the last run
};

// Online autotuner of the three spectral kernels' launch configuration.
//
// Each kernel (dts pre-pass, integration, propagation) has a candidate list
// of (direction mapping, resident CTAs per SM, prefetch distance).  While the
// tuner is active the inner loop runs host-driven and substep s launches each
// kernel with its candidate s mod n (round-robin, `reps` times each), timed
// with CUDA events on the model's stream; once a kernel has all its samples
// it keeps the candidate with the smallest median time (timing noise only
// adds time, and the interleaving spreads drift over all candidates).  The
// tuner measures the
// model's real substeps, so tuning costs no extra work.  Register budgets and
// prefetch distances do not change any result (mode 1); the direction mapping
// changes the summation order of the partial sums (mode 2, results differ by
// rounding: both mappings meet the parity bars).  Choices are cached per
// domain signature for the life of the process.
struct TuneCand {
  int g4, minb, pf;  // quarter-turn groups, CTAs per SM (0: default instance), levels prefetched
  int tma = 0;       // own rows staged by bulk copies (propagation 1: E* and e, 2: E*; pre-pass 1: e)
};
struct KernelTune {
  std::vector<TuneCand> cands;
  std::vector<std::vector<float>> ms;  // samples per candidate
  int best = -1;
};
enum { TK_PHYS = 0, TK_INTEG, TK_ADVECT, TK_N };
struct Tuner {
  int mode = 0;         // 0 off, 1 register budgets and prefetch, 2 also the direction mapping
  bool active = false;  // measuring
  bool done = false;    // a choice is in place (tuned or from the cache)
  int reps = 5;  // samples per candidate; the median decides (timing noise only adds time)
  int step = 0;         // substeps measured so far
  KernelTune k[TK_N];
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> kev;  // pending (kernel, events)
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  ~Tuner() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};
std::map<std::string, std::array<TuneCand, TK_N>> g_tune_cache;

struct Model {
  std::vector<MemberHost> mem;
  bool on_device = false;
  Params prm{};
  Ptrs P{};
  std::unique_ptr<Dev> dev;
  Member* d_mem = nullptr;
  int* d_tile_mem = nullptr;
  Global* d_glob = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Global* flag_h = nullptr;  // pinned read-back of the Global block
  cudaGraph_t graph = nullptr;          // inner loop as a while node (option "use_graph")
  cudaGraphExec_t graph_exec = nullptr;
  bool first = true;
  long long substeps = 0, max_substeps = -1;
  bool verbose = false, check_finite = false, use_graph = false;
  unsigned gust_seed = 1;  // seed of the wind gust draws (option "gust_seed")
  // spectrum output (output_spectrum_nc): the points of namelists/spectrum.nml,
  // read at the first output, the time of that output (the files' names) and
  // the records written so far per point (each call rewrites the files)
  struct SpecPoint {
    std::string id;
    int m, n, i;  // grid cell and wet index (1-based)
  };
  struct SpecRec {
    float wspd, wdir;
    std::vector<float> F, Sin, Sds, Snl, Sdt;
  };
  bool spec_read = false;
  std::vector<SpecPoint> spec_pts;
  std::string spec_time;
  std::vector<std::vector<SpecRec>> spec_recs;
  bool ocn_every = false;  // stress('ocn') after every outer step (option "stress_ocn")
  double last_gpu_ms = 0, last_bins = 0;
  long long launches = 0;
  int sel = 0;      // member the getters and setters act on
  std::vector<std::pair<int, int>> wet_ranges;  // (off, N) of each member
  int max_nm = 0;   // largest all-point range of a member
  bool ktime = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> kev;  // pending (kernel, events)
  std::vector<cudaEvent_t> evpool;
  size_t evused = 0;
  double kms[K_NK] = {0};
  long long kcnt[K_NK] = {0};
  float *E = nullptr, *ES = nullptr, *TAB = nullptr;
  Tuner tune;
  // persistent substep kernel (option "persistent"): its launch captured in a
  // graph once per launch configuration (pgraph_state 1), or launched
  // directly where the capture is refused (-1); 0: not tried yet
  bool persistent = false;
  int stall_test = 0;  // option "persistent_stall_test": the next launch's barrier waits run out
  cudaGraph_t pgraph = nullptr;
  cudaGraphExec_t pgraph_exec = nullptr;
  int pgraph_state = 0;

  ~Model() {
    for (cudaEvent_t e : evpool) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (flag_h) cudaFreeHost(flag_h);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    if (pgraph_exec) cudaGraphExecDestroy(pgraph_exec);
    if (pgraph) cudaGraphDestroy(pgraph);
  }
};

std::unique_ptr<Model> g_model;

struct Pending {  // a member added with umwm_gpu_ensemble_add, not yet initialized
  std::string nml;
  Inputs in;
};
std::vector<Pending> g_pending;

cudaEvent_t next_event(Model& M) {
  if (M.evused == M.evpool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    M.evpool.push_back(e);
  }
  return M.evpool[M.evused++];
}

// Launch wrapper: brackets the launch with events when kernel timing is on.
template <typename F>
cudaError_t timed(Model& M, int kname, F&& launch) {
  if (!M.ktime) return launch();
  cudaEvent_t a = next_event(M), b = next_event(M);
  cudaEventRecord(a, M.st);
  cudaError_t e = launch();
  cudaEventRecord(b, M.st);
  M.kev.push_back({kname, {a, b}});
  return e;
}

// Collect the timings of completed launches (call after a stream sync).
void collect_timings(Model& M) {
  for (auto& k : M.kev) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, k.second.first, k.second.second) == cudaSuccess) {
      M.kms[k.first] += ms;
      M.kcnt[k.first] += 1;
    }
  }
  M.kev.clear();
  M.evused = 0;
}

// ---- autotuner --------------------------------------------------------------
void drop_graph(Model& M) {  // the captured inner loop holds the old launch configuration
  if (M.graph_exec) { cudaGraphExecDestroy(M.graph_exec); M.graph_exec = nullptr; }
  if (M.graph) { cudaGraphDestroy(M.graph); M.graph = nullptr; }
  if (M.pgraph_exec) { cudaGraphExecDestroy(M.pgraph_exec); M.pgraph_exec = nullptr; }
  if (M.pgraph) { cudaGraphDestroy(M.pgraph); M.pgraph = nullptr; }
  if (M.pgraph_state == 1) M.pgraph_state = 0;
}

// One launch of the persistent substep kernel (budget armed before): the
// graph holding it, captured on first use, or a direct cooperative launch
// when the capture is refused or the stall test is armed.
int persist_launch(Model& M) {
  if (M.stall_test) {
    M.stall_test = 0;
    CU(launch_persist(M.prm, M.P, 1, M.st));
    return UMWM_OK;
  }
  if (M.pgraph_state == 0) {
    cudaError_t e = cudaStreamBeginCapture(M.st, cudaStreamCaptureModeThreadLocal);
    cudaError_t el = e == cudaSuccess ? launch_persist(M.prm, M.P, 0, M.st) : e;
    cudaGraph_t g = nullptr;
    cudaError_t ec = e == cudaSuccess ? cudaStreamEndCapture(M.st, &g) : e;
    cudaError_t ei = (el == cudaSuccess && ec == cudaSuccess) ? cudaGraphInstantiate(&M.pgraph_exec, g, 0) : el;
    if (el == cudaSuccess && ec == cudaSuccess && ei == cudaSuccess) {
      M.pgraph = g;
      M.pgraph_state = 1;
    } else {
      if (g) cudaGraphDestroy(g);
      M.pgraph_exec = nullptr;
      cudaGetLastError();  // the refused capture is not an error of the run
      M.pgraph_state = -1;
    }
  }
  if (M.pgraph_state == 1) {
    CU(cudaGraphLaunch(M.pgraph_exec, M.st));
  } else {
    CU(launch_persist(M.prm, M.P, 0, M.st));
  }
  return UMWM_OK;
}

std::string tune_key(const Model& M) {
  const Params& p = M.prm;
  return std::to_string(p.ntiles) + "/" + std::to_string(p.O) + "/" + std::to_string(p.P) + "/" +
         std::to_string(p.nmem) + "/" + std::to_string(p.curvilinear) + "/" + std::to_string(M.tune.mode);
}

// the launch configuration of kernel k in M.prm
TuneCand tune_get(const Params& p, int k) {
  if (k == TK_PHYS) return {p.groups4_phys, p.minb_phys, p.pf_phys, p.phys_tma};
  if (k == TK_INTEG) return {p.groups4, p.minb_integ, p.pf_integ};
  return {p.adv_groups4, p.minb_adv, p.pf_adv, p.adv_tma};
}
void tune_set(Params& p, int k, const TuneCand& c) {
  if (k == TK_PHYS) { p.groups4_phys = c.g4; p.minb_phys = c.minb; p.pf_phys = c.pf; p.phys_tma = c.tma; }
  else if (k == TK_INTEG) { p.groups4 = c.g4; p.minb_integ = c.minb; p.pf_integ = c.pf; }
  else { p.adv_groups4 = c.g4; p.minb_adv = c.minb; p.pf_adv = c.pf; p.adv_tma = c.tma; }
}

// Candidate lists.  Register budgets have kernel instances only for the
// 36-direction mappings (the integration's two-group shared memory allows at
// most 4 CTAs; the propagation's tuned instances are for plain grids).
void tune_start(Model& M, int mode) {
  Tuner& T = M.tune;
  T.mode = mode;
  T.active = T.done = false;
  T.step = 0;
  if (mode == 0) return;
  const Params& p = M.prm;
  auto it = g_tune_cache.find(tune_key(M));
  if (it != g_tune_cache.end()) {
    for (int k = 0; k < TK_N; ++k) tune_set(M.prm, k, it->second[k]);
    T.done = true;
    drop_graph(M);
    return;
  }
  const bool d36 = p.P == 36;
  for (int k = 0; k < TK_N; ++k) {
    KernelTune& K = T.k[k];
    K.cands.clear();
    const TuneCand cur = tune_get(p, k);
    std::vector<int> g4s = {cur.g4};
    if (mode == 2 && quarter_groups(p.P)) g4s = {0, 1};
    for (int g4 : g4s) {
      std::vector<int> minbs = {0}, pfs;
      if (k == TK_PHYS) {
        if (d36) minbs = g4 ? std::vector<int>{4, 5, 6} : std::vector<int>{5, 6, 7};
        pfs = {1, 2, 3};
      } else if (k == TK_INTEG) {
        if (d36) minbs = g4 ? std::vector<int>{3, 4, 5} : std::vector<int>{3, 4};
        pfs = {1, 2};
      } else {
        if (d36 && !p.curvilinear) minbs = {3, 4, 5};
        pfs = {1, 2};
      }
      for (int mb : minbs)
        for (int pf : pfs) K.cands.push_back({g4, mb, pf, 0});
      // the propagation (3 CTAs per SM) and the dts pre-pass (5) with their
      // own rows staged by bulk copies
      if (k == TK_ADVECT && d36 && !p.curvilinear && !g4)
        for (int pf : pfs) {
          K.cands.push_back({0, 3, pf, 1});  // E* and e staged
          K.cands.push_back({0, 4, pf, 2});  // E* staged
        }
      if (k == TK_PHYS && d36 && !g4)
        for (int pf : {1, 2}) K.cands.push_back({0, 5, pf, 1});
    }
    K.ms.assign(K.cands.size(), {});
    K.best = -1;
  }
  T.active = true;
  drop_graph(M);
}

// configuration of the next measured substep
void tune_apply(Model& M) {
  Tuner& T = M.tune;
  for (int k = 0; k < TK_N; ++k) {
    const KernelTune& K = T.k[k];
    const int c = K.best >= 0 ? K.best : (int)(T.step % K.cands.size());
    tune_set(M.prm, k, K.cands[c]);
  }
}

cudaEvent_t tune_event(Tuner& T) {
  if (T.used == T.pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    T.pool.push_back(e);
  }
  return T.pool[T.used++];
}

// after the substep's stream synchronisation: book its times
void tune_collect(Model& M) {
  Tuner& T = M.tune;
  if (!T.active || T.kev.empty()) return;
  for (auto& kv : T.kev) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, kv.second.first, kv.second.second) != cudaSuccess) continue;
    KernelTune& K = T.k[kv.first];
    if (K.best >= 0) continue;
    const int c = (int)(T.step % K.cands.size());
    K.ms[c].push_back(ms);
  }
  T.kev.clear();
  T.used = 0;
  T.step++;
  bool all = true;
  for (int k = 0; k < TK_N; ++k) {
    KernelTune& K = T.k[k];
    if (K.best >= 0) continue;
    if (T.step < (int)K.cands.size() * T.reps) { all = false; continue; }
    double bm = 1e300;
    for (size_t c = 0; c < K.cands.size(); ++c) {
      std::vector<float> v = K.ms[c];
      if (v.empty()) continue;
      std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
      if (v[v.size() / 2] < bm) { bm = v[v.size() / 2]; K.best = (int)c; }
    }
    if (K.best < 0) K.best = 0;
  }
  if (!all) return;
  std::array<TuneCand, TK_N> choice;
  for (int k = 0; k < TK_N; ++k) {
    choice[k] = T.k[k].cands[T.k[k].best];
    tune_set(M.prm, k, choice[k]);
  }
  g_tune_cache[tune_key(M)] = choice;
  T.active = false;
  T.done = true;
  drop_graph(M);
}

// Launch wrapper of the tuned kernels: events for the tuner while it
// measures, else the kernel-timing wrapper.
template <typename F>
cudaError_t tuned(Model& M, int tk, int kname, F&& launch) {
  if (!M.tune.active) return timed(M, kname, launch);
  cudaEvent_t a = tune_event(M.tune), b = tune_event(M.tune);
  cudaEventRecord(a, M.st);
  cudaError_t e = launch();
  cudaEventRecord(b, M.st);
  M.tune.kev.push_back({tk, {a, b}});
  return e;
}

// per-(o,i) tables in the blocked device layout [o][j/32][t][32], one member
// at a time (host memory of one member).  A member's ghost point holds the
// ghost values of cp0/cg0; padding points get finite throw-away values (k = 1)
// so that idle lanes stay finite.  Members start on a tile boundary, so for
// each o a member's blocks are one contiguous range.
int upload_tables(Model& M, const MemberHost& mh) {
  const Params& prm = M.prm;
  const int O = prm.O;
  const HostModel& H = mh.H;
  const std::vector<float>* src[T_COUNT] = {};
  src[T_K] = &H.k, src[T_CP0] = &H.cp0, src[T_CG0] = &H.cg0, src[T_LOGL2Z] = &H.logl2overz;
  src[T_FKOVG] = &H.fkovg, src[T_KDK] = &H.kdk, src[T_K4] = &H.k4, src[T_K3DK] = &H.k3dk;
  src[T_COTHKD] = &H.cothkd, src[T_SBF] = &H.sbf, src[T_SDV] = &H.sdv, src[T_BF1R] = &H.bf1r;
  src[T_BF2R] = &H.bf2r;
  const size_t per_o = (size_t)mh.padded * T_COUNT;  // floats of one level of this member
  std::vector<float> T(per_o);
  for (int o = 1; o <= O; ++o) {
    for (int t = 0; t < T_COUNT; ++t) {
      const bool ghost = (t == T_CP0 || t == T_CG0);
      for (int j = 0; j < mh.padded; ++j) {
        float v;
        if (j < mh.N) v = (*src[t])[H.oi(o, j + 1)];
        else if (ghost) v = (*src[t])[H.oi(o, 0)];
        else v = (t == T_K || t == T_K4 || t == T_KDK || t == T_COTHKD) ? 1.f : 0.f;
        T[((size_t)(j >> 5) * T_COUNT + t) * 32 + (j & 31)] = v;
      }
    }
    CU(cudaMemcpy(M.TAB + tidx(prm, o - 1, 0, mh.off), T.data(), per_o * 4, cudaMemcpyHostToDevice));
  }
  return UMWM_OK;
}

int set_forcing_constants(Model& M, MemberHost& mh) {
  // input_nc without file variables: umwm_io.F90:39-83
  const HostModel& H = mh.H;
  const size_t NM = mh.NM, a = mh.nmoff;
  if (!H.winds) {
    CU(launch_fill(M.P.wspd + a, NM, H.wspd0, M.st));
    CU(launch_fill(M.P.wdir + a, NM, H.wdir0, M.st));
  }
  if (!H.currents) {
    CU(launch_fill(M.P.uc + a, NM, H.uc0, M.st));
    CU(launch_fill(M.P.vc + a, NM, H.vc0, M.st));
  }
  if (!H.seaice) CU(launch_fill(M.P.fice + a, NM, H.fice0, M.st));
  if (!H.air_density) CU(launch_fill(M.P.rhoa + a, NM, H.rhoa0, M.st));
  if (!H.water_density) CU(launch_fill(M.P.rhow + a, NM, H.rhow0, M.st));
  return UMWM_OK;
}

// input_nc(timestr) file variables into the n+1 level, umwm_io.F90:13-93
int read_forcing(Model& M, MemberHost& mh, const std::string& key, std::vector<float>* uwf_host = nullptr,
                 std::vector<float>* vwf_host = nullptr) {
  const HostModel& H = mh.H;
  if (!mh.readfile) return UMWM_OK;
  auto it = mh.in.forcing.find(key);
  if (it == mh.in.forcing.end()) {
    // nothing staged: the reference's file input/umwmin_<time>.nc (umwm_io.F90:20-26)
    const std::string path = "input/umwmin_" + key + ".nc";
    std::map<std::string, std::vector<float>> vars;
    const std::pair<bool, const char*> want[] = {{H.winds, "uw"}, {H.winds, "vw"}, {H.currents, "uc"},
                                                 {H.currents, "vc"}, {H.seaice, "fice"},
                                                 {H.air_density, "rhoa"}, {H.water_density, "rhow"}};
    for (auto& w : want) {
      if (!w.first) continue;
      std::vector<size_t> sh;
      std::string err;
      if (!nc::read_float(path, w.second, sh, vars[w.second], err))
        return fail(UMWM_ERR_INPUT, "input_nc: no forcing staged for " + key + " and " + err);
    }
    it = mh.in.forcing.emplace(key, std::move(vars)).first;
  }
  const size_t n2 = (size_t)H.mm * H.nm;
  auto get = [&](const char* var, float* dst, bool zero_land, std::vector<float>* keep) -> int {
    auto v = it->second.find(var);
    if (v == it->second.end()) return fail(UMWM_ERR_INPUT, std::string("input_nc: variable ") + var + " missing for " + key);
    if (v->second.size() != n2) return fail(UMWM_ERR_INPUT, std::string("input_nc: variable ") + var + " has the wrong size");
    const float* src = v->second.data();
    std::vector<float> tmp;
    if (zero_land) {
      tmp = v->second;
      for (size_t q = 0; q < n2; ++q) if (H.mask[q] == 0) tmp[q] = 0.f;
      src = tmp.data();
    }
    if (keep) keep->assign(src, src + n2);
    CU(cudaMemcpyAsync(dst, src, n2 * 4, cudaMemcpyHostToDevice, M.st));
    CU(cudaStreamSynchronize(M.st));
    return UMWM_OK;
  };
  int rc;
  if (H.winds) {
    if ((rc = get("uw", mh.uwf, false, uwf_host))) return rc;
    if ((rc = get("vw", mh.vwf, false, vwf_host))) return rc;
  }
  if (H.currents) {
    if ((rc = get("uc", mh.ucf, true, nullptr))) return rc;
    if ((rc = get("vc", mh.vcf, true, nullptr))) return rc;
  }
  if (H.seaice && (rc = get("fice", mh.ficef, false, nullptr))) return rc;
  if (H.air_density && (rc = get("rhoa", mh.rhoaf, false, nullptr))) return rc;
  if (H.water_density && (rc = get("rhow", mh.rhowf, false, nullptr))) return rc;
  return UMWM_OK;
}

// forcinginput, umwm_forcing.F90:11-37
int forcing_input(Model& M, MemberHost& mh, const std::string& key) {
  const HostModel& H = mh.H;
  const size_t b = (size_t)H.mm * H.nm * 4;
  auto cp = [&](float* d, const float* s_) { return cudaMemcpyAsync(d, s_, b, cudaMemcpyDeviceToDevice, M.st); };
  if (H.winds) { CU(cp(mh.uwb, mh.uwf)); CU(cp(mh.vwb, mh.vwf)); }
  if (H.currents) { CU(cp(mh.ucb, mh.ucf)); CU(cp(mh.vcb, mh.vcf)); }
  if (H.air_density) CU(cp(mh.rhoab, mh.rhoaf));
  if (H.water_density) CU(cp(mh.rhowb, mh.rhowf));
  if (H.seaice) CU(cp(mh.ficeb, mh.ficef));
  int rc = read_forcing(M, mh, key);
  if (rc) return rc;
  if (mh.readfile) return set_forcing_constants(M, mh);
  return UMWM_OK;
}

// Parameters shared by all members; members must agree on them.
int setup_params(Model& M) {
  const HostModel& H = M.mem[0].H;
  for (size_t m = 1; m < M.mem.size(); ++m) {
    const HostModel& G = M.mem[m].H;
    const bool same =
        G.om == H.om && G.pm == H.pm && G.fmin == H.fmin && G.fmax == H.fmax && G.fprog == H.fprog && G.dtg == H.dtg &&
        G.g == H.g && G.nu_air == H.nu_air && G.nu_water == H.nu_water && G.sfct == H.sfct && G.kappa == H.kappa &&
        G.z == H.z && G.explim == H.explim && G.sin_fac == H.sin_fac && G.sin_diss1 == H.sin_diss1 &&
        G.sin_diss2 == H.sin_diss2 && G.sds_fac == H.sds_fac && G.sds_power == H.sds_power && G.mss_fac == H.mss_fac &&
        G.snl_fac == H.snl_fac && G.sdt_fac == H.sdt_fac && G.sbf_fac == H.sbf_fac && G.sbp_fac == H.sbp_fac &&
        G.winds == H.winds && G.currents == H.currents && G.air_density == H.air_density &&
        G.water_density == H.water_density && G.seaice == H.seaice && G.restart == H.restart && G.stokes == H.stokes &&
        G.fice_lth == H.fice_lth && G.fice_uth == H.fice_uth && G.rhow0 == H.rhow0 && G.depth == H.depth &&
        G.starttimestr == H.starttimestr;
    if (!same)
      return fail(UMWM_ERR_UNSUPPORTED, "ensemble members must share the spectral grid, physics, forcing switches, "
                                        "dtg, start time and Stokes depths; member " + std::to_string(m) + " differs");
  }
  if (H.om > MAX_OM) return fail(UMWM_ERR_UNSUPPORTED, "om > 64 is not supported");
  if (H.pm > MAX_PM || !supported_pm(H.pm))
    return fail(UMWM_ERR_UNSUPPORTED, "pm must be 4*k with k in {2,3,4,6,8,9,12}");
  if (H.lm > MAX_LM) return fail(UMWM_ERR_UNSUPPORTED, "more than 100 Stokes depths");
  for (const MemberHost& mh : M.mem)
    if (mh.H.gustiness != M.mem[0].H.gustiness)
      return fail(UMWM_ERR_UNSUPPORTED, "ensemble members must share gustiness");
  Params& p = M.prm;
  // layout: each member's wet points, its ghost, padding to a tile
  int off = 0, nmoff = 0;
  M.max_nm = 0;
  M.wet_ranges.clear();
  for (MemberHost& mh : M.mem) {
    mh.N = mh.H.im;
    mh.off = off;
    M.wet_ranges.push_back({off, mh.N});
    mh.ghost = off + mh.N;
    mh.padded = (mh.N + 1 + TILE - 1) / TILE * TILE;
    off += mh.padded;
    mh.NM = mh.H.imm;
    mh.nmoff = nmoff;
    nmoff += mh.NM;
    M.max_nm = std::max(M.max_nm, mh.NM);
    mh.readfile = mh.H.winds || mh.H.currents || mh.H.air_density || mh.H.water_density || mh.H.seaice;
  }
  p.Ntot = off;
  p.NB = off / 32;
  p.ldN = off;
  p.NMtot = nmoff;
  p.ntiles = off / TILE;
  p.nmem = (int)M.mem.size();
  p.O = H.om; p.P = H.pm; p.lm = H.lm;
  p.g = H.g; p.explim = H.explim; p.sin_fac = H.sin_fac; p.fieldscale1 = H.fieldscale1;
  p.fieldscale2 = H.fieldscale2; p.twopisds_fac = H.twopisds_fac; p.sds_power = H.sds_power;
  p.inv_sds_power = H.inv_sds_power; p.mss_fac = H.mss_fac; p.snl_fac = H.snl_fac; p.sdt_fac = H.sdt_fac;
  p.bf1 = H.bf1; p.bf2 = H.bf2;
  p.gustiness = H.gustiness;
  p.gust_seed = M.gust_seed;
  p.sin_neg1 = H.sin_fac * H.fieldscale1;
  // fieldscale2 applies where x fieldscale1 is still negative
  p.sin_neg2 = H.fieldscale1 > 0.f ? (H.sin_fac * H.fieldscale1) * H.fieldscale2 : p.sin_neg1;
  p.z = H.z; p.nu_air = H.nu_air; p.kappa = H.kappa; p.fprog = H.fprog; p.dth = H.dth; p.dthg = H.dthg;
  p.oneovdth = H.oneovdth; p.dtg = H.dtg; p.fice_lth = H.fice_lth; p.fice_uth = H.fice_uth;
  p.eulerinv = H.eulerinv; p.rhow0 = H.rhow0;
  p.winds = H.winds; p.currents = H.currents; p.air_density = H.air_density; p.water_density = H.water_density;
  p.seaice = H.seaice; p.restart = H.restart;
  p.curvilinear = 0; p.isglobal = 0; p.ice_possible = 0;
  for (const MemberHost& mh : M.mem) {
    p.curvilinear |= mh.H.curvilinear;
    p.isglobal |= mh.H.isglobal;
    p.ice_possible |= (mh.H.seaice || (mh.H.fice0 > mh.H.fice_lth));
  }
  for (int o = 0; o < H.om; ++o) { p.f[o] = H.f[o]; p.dom[o] = H.dom[o]; }
  // the two-group flux of pm % 4 == 0 grids takes one upwind term per slot
  // pair (adv_body.cuh): the grid th(p) = (p - (pm + 1) / 2) dth gives the
  // first pm/2 directions sin th < 0 and cos th < 0 exactly below pm/4
  p.swsign = H.pm % 4 == 0;
  for (int q = 0; q < H.pm / 2; ++q)
    if (!(H.sth[q] < 0.f) || !(q < H.pm / 4 ? H.cth[q] < 0.f : H.cth[q] > 0.f)) p.swsign = 0;
  if (H.pm % 4 == 0 && !p.swsign) return fail(UMWM_ERR_NAMELIST, "direction grid without the expected signs");
  for (int q = 0; q < H.pm; ++q) {
    p.th[q] = H.th[q]; p.cth[q] = H.cth[q]; p.sth[q] = H.sth[q];
    p.cthp[q] = std::max(H.cth[q], 0.f); p.cthm[q] = std::min(H.cth[q], 0.f);
    const int q1 = (q + 1) % H.pm;
    p.shs[q] = 0.5f * (H.sth[q] + H.sth[q1]);
    p.chs[q] = 0.5f * (H.cth[q] + H.cth[q1]);
    p.sthp[q] = std::max(H.sth[q], 0.f); p.sthm[q] = std::min(H.sth[q], 0.f);
    p.c2th[q] = (float)std::cos(2.0 * (double)H.th[q]);
    p.s2th[q] = (float)std::sin(2.0 * (double)H.th[q]);
  }
  for (int l = 0; l < H.lm; ++l) p.depth[l] = H.depth[l];
  // launch configuration: default register budgets (0) and prefetch distances
  p.minb_phys = p.minb_integ = p.minb_adv = 0;
  p.count_cut = 0;
  p.adv_tma = 0;
  p.phys_tma = 0;
  p.pf_phys = UMWM_PF_DIST_PHYS;
  p.pf_integ = UMWM_PF_DIST_INTEG;
  p.pf_adv = UMWM_PF_DIST_ADV;
  return UMWM_OK;
}

#ifndef UMWM_AUTO_G4_TILES
#define UMWM_AUTO_G4_TILES 3
#endif

int init_device(Model& M) {
  int rc = setup_params(M);
  if (rc) return rc;
  Params& p = M.prm;
  const int ldN = p.ldN;
  const size_t spec = (size_t)p.O * p.P * ldN;
  if (g_device >= 0) CU(cudaSetDevice(g_device));
  // Small domains: with fewer than UMWM_AUTO_G4_TILES 64-point tiles per SM
  // the half-turn mapping leaves SMs idle, and four quarter-turn groups (32
  // points per CTA) double the CTAs: measured 1.4x at 9.6 k wet points,
  // 1.3x at 17.7 k, even at 31 k (3.2 tiles per SM), 0.95x at 71 k.  The
  // options direction_groups / advect_groups override this.
  {
    int dev = 0, nsm = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (quarter_groups(p.P) && (long)p.ntiles < (long)UMWM_AUTO_G4_TILES * nsm)
      p.groups4 = p.groups4_phys = p.adv_groups4 = 1;
  }
  M.dev.reset(new Dev());
  Dev& D = *M.dev;
  CU(cudaStreamCreateWithFlags(&M.st, cudaStreamNonBlocking));
  CU(cudaEventCreate(&M.ev0));
  CU(cudaEventCreate(&M.ev1));
  CU(cudaMallocHost(&M.flag_h, sizeof(Global)));
  Ptrs& P = M.P;
  CU(D.alloc(&M.E, spec, false));
  CU(D.alloc(&M.ES, spec, false));
  P.E = M.E; P.ES = M.ES;
  P.EF = M.E;  // ef overwrites e bin by bin (source integration), e overwrites ef (advection)
  CU(D.alloc(&M.TAB, (size_t)p.O * T_COUNT * ldN, true));
  P.TAB = M.TAB;
  for (const MemberHost& mh : M.mem)
    if ((rc = upload_tables(M, mh))) return rc;
  // per-point arrays in the common index space
  auto upload_i = [&](const int** dst, std::vector<int>(HostModel::*field), bool aliased) -> int {
    std::vector<int> h(ldN, 0);
    for (const MemberHost& mh : M.mem) {
      const std::vector<int>& src = mh.H.*field;
      for (int j = 0; j < mh.padded; ++j) {
        int v;
        if (j < mh.N) {
          const int r = src[j + 1];
          v = aliased ? (r == 0 ? mh.ghost : mh.off + r - 1) : mh.nmoff + r - 1;
        } else {
          v = aliased ? mh.ghost : mh.nmoff + mh.N;  // the member's ghost / a land point
        }
        h[mh.off + j] = v;
      }
    }
    int* d = nullptr;
    CU(D.alloc(&d, ldN));
    CU(cudaMemcpy(d, h.data(), (size_t)ldN * 4, cudaMemcpyHostToDevice));
    *dst = d;
    return UMWM_OK;
  };
  if ((rc = upload_i(&P.ie, &HostModel::ie, true)) || (rc = upload_i(&P.iw, &HostModel::iw, true)) ||
      (rc = upload_i(&P.in, &HostModel::in, true)) || (rc = upload_i(&P.is, &HostModel::is, true)) ||
      (rc = upload_i(&P.iie, &HostModel::iie, false)) || (rc = upload_i(&P.iiw, &HostModel::iiw, false)) ||
      (rc = upload_i(&P.iin, &HostModel::iin, false)) || (rc = upload_i(&P.iis, &HostModel::iis, false)))
    return rc;
  auto upload_f = [&](const float** dst, std::vector<float>(HostModel::*field)) -> int {
    std::vector<float> h(ldN, 1.f);
    for (const MemberHost& mh : M.mem) {
      const std::vector<float>& src = mh.H.*field;
      for (int i = 1; i <= mh.N; ++i) h[mh.off + i - 1] = src[i];
    }
    float* d = nullptr;
    CU(D.alloc(&d, ldN));
    CU(cudaMemcpy(d, h.data(), (size_t)ldN * 4, cudaMemcpyHostToDevice));
    *dst = d;
    return UMWM_OK;
  };
  if ((rc = upload_f(&P.oneovar, &HostModel::oneovar)) || (rc = upload_f(&P.oneovdx, &HostModel::oneovdx)) ||
      (rc = upload_f(&P.oneovdy, &HostModel::oneovdy)) || (rc = upload_f(&P.dxn, &HostModel::dxn)) ||
      (rc = upload_f(&P.dxs, &HostModel::dxs)) || (rc = upload_f(&P.dye, &HostModel::dye)) ||
      (rc = upload_f(&P.dyw, &HostModel::dyw)) || (rc = upload_f(&P.d, &HostModel::d)) ||
      (rc = upload_f(&P.curv, &HostModel::curv_i)))
    return rc;
  {
    std::vector<int> ones(ldN, 1);
    CU(D.alloc(&P.oc, ldN)); CU(D.alloc(&P.oc_rot, ldN));
    CU(cudaMemcpy(P.oc, ones.data(), (size_t)ldN * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(P.oc_rot, ones.data(), (size_t)ldN * 4, cudaMemcpyHostToDevice));
  }
  for (float** q : {&P.ustar, &P.cd, &P.taux, &P.tauy, &P.taux_form, &P.tauy_form, &P.taux_skin, &P.tauy_skin,
                    &P.taux_diag, &P.tauy_diag, &P.tailatmx, &P.tailatmy, &P.shelt, &P.fcutoff, &P.phys, &P.sice_v,
                    &P.ds, &P.ht, &P.mwp, &P.mwd, &P.mss, &P.mwl, &P.dwd, &P.dwl, &P.dwp, &P.dcp0, &P.dcp, &P.dcg0,
                    &P.dcg, &P.momx, &P.momy, &P.cgmxx, &P.cgmxy, &P.cgmyy})
    CU(D.alloc(q, ldN));
  for (float** q : {&P.wspd, &P.wdir, &P.uc, &P.vc, &P.rhoa, &P.rhow, &P.rhorat, &P.fice}) CU(D.alloc(q, p.NMtot));
  CU(D.alloc(&P.us, (size_t)std::max(1, p.lm) * ldN));
  CU(D.alloc(&P.vs, (size_t)std::max(1, p.lm) * ldN));
  CU(D.alloc(&M.d_glob, 1));
  P.glob = M.d_glob;
  // per-member device pieces
  Ctl* ctls = nullptr;
  CU(D.alloc(&ctls, M.mem.size()));
  std::vector<Member> hm(M.mem.size());
  for (size_t m = 0; m < M.mem.size(); ++m) {
    MemberHost& mh = M.mem[m];
    const HostModel& H = mh.H;
    mh.ctl = ctls + m;
    mh.log_cap = M.mem.size() > 1 ? (1 << 14) : (1 << 20);
    CU(D.alloc(&mh.log, (size_t)mh.log_cap * 8));
    std::vector<int> mi(mh.NM), ni(mh.NM);
    for (int i = 1; i <= mh.NM; ++i) { mi[i - 1] = H.mi[i]; ni[i - 1] = H.ni[i]; }
    CU(D.alloc(&mh.mi, mh.NM)); CU(D.alloc(&mh.ni, mh.NM));
    CU(cudaMemcpy(mh.mi, mi.data(), (size_t)mh.NM * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(mh.ni, ni.data(), (size_t)mh.NM * 4, cudaMemcpyHostToDevice));
    const size_t n2 = (size_t)H.mm * H.nm;
    auto lev = [&](bool on, float** b, float** f) -> int {
      if (!on) return UMWM_OK;
      CU(D.alloc(b, n2)); CU(D.alloc(f, n2));
      return UMWM_OK;
    };
    if ((rc = lev(H.winds, &mh.uwb, &mh.uwf)) || (rc = lev(H.winds, &mh.vwb, &mh.vwf)) ||
        (rc = lev(H.currents, &mh.ucb, &mh.ucf)) || (rc = lev(H.currents, &mh.vcb, &mh.vcf)) ||
        (rc = lev(H.air_density, &mh.rhoab, &mh.rhoaf)) || (rc = lev(H.water_density, &mh.rhowb, &mh.rhowf)) ||
        (rc = lev(H.seaice, &mh.ficeb, &mh.ficef)))
      return rc;
    Member& d = hm[m];
    d.off = mh.off; d.N = mh.N; d.ghost = mh.ghost; d.nmoff = mh.nmoff; d.NM = mh.NM; d.mm = H.mm; d.nm = H.nm;
    d.iip = (H.iip >= 1 && H.iip <= H.im) ? mh.off + H.iip - 1 : -1;
    d.dtamin = H.dtamin;
    d.ctl = mh.ctl;
    d.log = mh.log;
    d.log_cap = mh.log_cap;
    d.mi = mh.mi; d.ni = mh.ni;
    d.uwb = mh.uwb; d.uwf = mh.uwf; d.vwb = mh.vwb; d.vwf = mh.vwf; d.ucb = mh.ucb; d.ucf = mh.ucf;
    d.vcb = mh.vcb; d.vcf = mh.vcf; d.rhoab = mh.rhoab; d.rhoaf = mh.rhoaf; d.rhowb = mh.rhowb; d.rhowf = mh.rhowf;
    d.ficeb = mh.ficeb; d.ficef = mh.ficef;
    Ctl c{};
    c.minphys_enc = enc_ord_h(std::numeric_limits<float>::infinity());
    c.maxrot_enc = enc_ord_h(0.f);
    c.first = 1;
    c.zerocurrents = 1;
    CU(cudaMemcpy(mh.ctl, &c, sizeof c, cudaMemcpyHostToDevice));
  }
  CU(D.alloc(&M.d_mem, M.mem.size()));
  CU(cudaMemcpy(M.d_mem, hm.data(), hm.size() * sizeof(Member), cudaMemcpyHostToDevice));
  {
    std::vector<int> tm(p.ntiles, 0);
    for (size_t m = 0; m < M.mem.size(); ++m)
      for (int t = M.mem[m].off / TILE; t < (M.mem[m].off + M.mem[m].padded) / TILE; ++t) tm[t] = (int)m;
    CU(D.alloc(&M.d_tile_mem, p.ntiles));
    CU(cudaMemcpy(M.d_tile_mem, tm.data(), (size_t)p.ntiles * 4, cudaMemcpyHostToDevice));
  }
  p.mem = M.d_mem;
  p.tile_mem = M.d_tile_mem;

  // e = tiny(e), umwm_init.F90:1182 (spectrum and the ghost points of E*)
  const float tiny = std::numeric_limits<float>::min();
  CU(launch_fill(M.E, spec, tiny, M.st));
  CU(launch_fill(M.ES, spec, tiny, M.st));

  // input_nc(starttimestr), umwm_top.F90:25, and init's first guess of the
  // drag and friction velocity, umwm_init.F90:1350-1365
  std::vector<float> ust(ldN, 0.f), cd(ldN, 0.f);
  for (MemberHost& mh : M.mem) {
    const HostModel& H = mh.H;
    std::vector<float> uwf_h, vwf_h;
    if ((rc = set_forcing_constants(M, mh))) return rc;
    rc = read_forcing(M, mh, time_key(H.starttimestr.c_str()), &uwf_h, &vwf_h);
    if (rc) return rc;
    std::vector<float> wspd(mh.N + 1, H.wspd0);
    if (H.winds)
      for (int i = 1; i <= mh.N; ++i) {
        size_t q = H.i2(H.mi[i], H.ni[i]);
        wspd[i] = std::sqrt(uwf_h[q] * uwf_h[q] + vwf_h[q] * vwf_h[q]);
      }
    for (int i = 1; i <= mh.N; ++i) {
      float c_ = 1.2e-3f;
      if (wspd[i] > 11) c_ = (0.49f + 0.065f * wspd[i]) * 1e-3f;
      cd[mh.off + i - 1] = c_;
      ust[mh.off + i - 1] = std::sqrt(c_) * wspd[i];
    }
    if (H.seaice) {  // init copies ficef into fice, umwm_init.F90:1351
      std::vector<float> fi(mh.NM, 0.f);
      const std::vector<float>& src = mh.in.forcing.find(time_key(H.starttimestr.c_str()))->second.at("fice");
      for (int i = 1; i <= mh.NM; ++i) fi[i - 1] = src[H.i2(H.mi[i], H.ni[i])];
      CU(cudaMemcpy(P.fice + mh.nmoff, fi.data(), (size_t)mh.NM * 4, cudaMemcpyHostToDevice));
    }
  }
  CU(cudaMemcpy(P.ustar, ust.data(), (size_t)ldN * 4, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(P.cd, cd.data(), (size_t)ldN * 4, cudaMemcpyHostToDevice));
  // stokes_drift('init'), umwm_top.F90:27
  if (p.lm > 0) CU(launch_stokes(M.prm, P, M.st));
  CU(cudaStreamSynchronize(M.st));
  M.first = true;
  M.on_device = true;
  return UMWM_OK;
}

int set_state_member(Model& M, int m, const float* F, const float* ust) {
  const Params& p = M.prm;
  const MemberHost& mh = M.mem[m];
  if (F) {
    const size_t n = (size_t)p.O * p.P * mh.N;
    float* tmp = nullptr;
    CU(cudaMalloc(&tmp, n * 4));
    cudaError_t e = cudaMemcpy(tmp, F, n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_from_ref(p, tmp, M.E, mh.off, mh.N, M.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M.st);
    cudaFree(tmp);
    CU(e);
  }
  if (ust) CU(cudaMemcpy(M.P.ustar + mh.off, ust, (size_t)mh.N * 4, cudaMemcpyHostToDevice));
  return UMWM_OK;
}

// Restart file name of a member: restart/umwmrst_<time>.nc as the reference
// names it (umwm_restart.F90:28-31, :70); ensemble members add _m<member>.
std::string restart_path(const Model& M, int m, const std::string& key) {
  std::string p = "restart/umwmrst_" + key;
  if (M.mem.size() > 1) p += "_m" + std::to_string(m);
  return p + ".nc";
}

// restart_read, umwm_restart.F90:19-56: the staged restart for the time key,
// else the file restart/umwmrst_<key>.nc (F and ust).
int restart_read(Model& M, int m, const std::string& key) {
  MemberHost& mh = M.mem[m];
  auto it = mh.in.restarts.find(key);
  if (it == mh.in.restarts.end()) {
    const std::string path = restart_path(M, m, key);
    std::vector<size_t> shF, shU;
    std::vector<float> F, U;
    std::string err;
    if (!nc::read_float(path, "F", shF, F, err) || !nc::read_float(path, "ust", shU, U, err))
      return fail(UMWM_ERR_INPUT, "restart_read: no restart staged for " + key + " and " + err);
    const std::vector<size_t> wantF = {(size_t)mh.N, (size_t)M.prm.P, (size_t)M.prm.O};
    if (shF != wantF || shU != std::vector<size_t>{(size_t)mh.N})
      return fail(UMWM_ERR_INPUT, "restart_read: " + path + " does not match the grid (x, th, f)");
    return set_state_member(M, m, F.data(), U.data());
  }
  const size_t nF = (size_t)M.prm.O * M.prm.P * mh.N;
  if (it->second.first.size() != nF || it->second.second.size() != (size_t)mh.N)
    return fail(UMWM_ERR_INPUT, "restart_read: restart arrays have the wrong size");
  return set_state_member(M, m, it->second.first.data(), it->second.second.data());
}

// restart_write, umwm_restart.F90:59-154: dimensions x (wet points), f, th;
// variables lon, lat, frequency, theta, ust, wavenumber (x, f) and F
// (x, th, f), with the reference's descriptions and units.
int restart_write(Model& M, int m, const std::string& path) {
  const Params& p = M.prm;
  const MemberHost& mh = M.mem[m];
  const HostModel& H = mh.H;
  const int N = mh.N;
  const size_t R = (size_t)p.O * p.P;
  CU(cudaStreamSynchronize(M.st));
  std::vector<float> lon(N), lat(N), ust(N);
  for (int i = 1; i <= N; ++i) {
    lon[i - 1] = H.lon[H.i2(H.mi[i], H.ni[i])];
    lat[i - 1] = H.lat[H.i2(H.mi[i], H.ni[i])];
  }
  CU(cudaMemcpy(ust.data(), M.P.ustar + mh.off, (size_t)N * 4, cudaMemcpyDeviceToHost));
  auto from = [](const float* v) {
    return [v](size_t first, size_t n, float* out) {
      std::memcpy(out, v + first, n * 4);
      return true;
    };
  };
  // F streams through a device buffer of whole points
  const int chunk_pts = 2048;
  float* dtmp = nullptr;
  CU(cudaMalloc(&dtmp, (size_t)chunk_pts * R * 4));
  std::vector<float> hbuf((size_t)chunk_pts * R);
  long cached = -1;  // first point held in hbuf
  bool dev_ok = true;
  auto fillF = [&](size_t first, size_t n, float* out) {
    while (n > 0) {
      const long pt = (long)(first / R);
      if (cached < 0 || pt < cached || pt >= cached + chunk_pts) {
        const int cnt = (int)std::min<long>(chunk_pts, N - pt);
        cudaError_t e = launch_to_ref(p, M.E, dtmp, mh.off + (int)pt, cnt, M.st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(M.st);
        if (e == cudaSuccess) e = cudaMemcpy(hbuf.data(), dtmp, (size_t)cnt * R * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
          dev_ok = false;
          return false;
        }
        cached = pt;
      }
      const size_t off = first - (size_t)cached * R;
      const size_t take = std::min(n, (size_t)chunk_pts * R - off);
      std::memcpy(out, hbuf.data() + off, take * 4);
      out += take;
      first += take;
      n -= take;
    }
    return true;
  };
  const std::vector<std::pair<std::string, size_t>> dims = {{"x", (size_t)N}, {"f", (size_t)p.O}, {"th", (size_t)p.P}};
  std::vector<nc::Var> vars = {
      {"lon", {0}, {{"description", "longitude"}, {"units", "degrees east"}}, from(lon.data())},
      {"lat", {0}, {{"description", "latitude"}, {"units", "degrees north"}}, from(lat.data())},
      {"frequency", {1}, {{"description", "frequency"}, {"units", "hz"}}, from(H.f.data())},
      {"theta", {2}, {{"description", "directions"}, {"units", "rad"}}, from(H.th.data())},
      {"ust", {0}, {{"description", "friction velocity"}, {"units", "m s^-1"}}, from(ust.data())},
      {"wavenumber", {0, 1}, {{"description", "wavenumber"}, {"units", "rad m^-1"}}, from(H.k.data() + p.O)},
      {"F", {0, 2, 1}, {{"description", "wave energy spectrum"}, {"units", "m^4 rad^-1"}}, fillF}};
  std::string err;
  const bool ok = nc::write(path, dims, vars, err);
  cudaFree(dtmp);
  if (!dev_ok) return fail(UMWM_ERR_CUDA, "restart_write: device copy failed");
  if (!ok) return fail(UMWM_ERR_INPUT, "restart_write: " + err);
  return UMWM_OK;
}

// output_grid_nc, umwm_io.F90:317-854: output/umwmout_<time>.nc with the
// reference's dimensions (x, y, f, th, time as the record dimension, z with
// the Stokes drift) and variables, in its order.  Wet-point fields go to
// their (m, n) cell and land cells are NaN, as gatherfield leaves them
// (umwm_io.F90:856-901); psim is 0 as in the reference (umwm_init.F90:341-342).
int output_grid(Model& M, const std::string& path) {
  const Params& p = M.prm;
  const MemberHost& mh = M.mem[0];
  const HostModel& H = mh.H;
  const Ptrs& P = M.P;
  const int N = mh.N, mm = H.mm, nm = H.nm;
  const size_t n2 = (size_t)mm * nm;
  CU(cudaStreamSynchronize(M.st));
  const float nan = std::numeric_limits<float>::quiet_NaN();
  // a wet-point field (device, wet points first) spread on the grid
  auto spread = [&](const float* dev, std::vector<float>& out) -> bool {
    std::vector<float> w(N);
    if (cudaMemcpy(w.data(), dev, (size_t)N * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    out.assign(n2, nan);
    for (int i = 1; i <= N; ++i) out[H.i2(H.mi[i], H.ni[i])] = w[i - 1];
    return true;
  };
  struct Field {
    const char *name, *desc, *units;
    std::function<bool(std::vector<float>&)> make;  // the whole variable
    int kind;  // 0: (time, y, x), 1: (f), 2: (th), 3: (z), 4: (time, z, y, x)
    bool is_int;
  };
  auto wet = [&](const float* dev) { return [&, dev](std::vector<float>& o) { return spread(dev + mh.off, o); }; };
  auto allp = [&](const float* dev) { return [&, dev](std::vector<float>& o) { return spread(dev + mh.nmoff, o); }; };
  auto ocn = [&](int q) {
    return [&, q](std::vector<float>& o) { return spread(P.ocn + (size_t)q * p.ldN + mh.off, o); };
  };
  auto host2d = [&](const std::vector<float>& v) { return [&v](std::vector<float>& o) { o = v; return true; }; };
  auto stokes = [&](const float* dev) {
    return [&, dev](std::vector<float>& o) {
      o.assign((size_t)H.lm * n2, nan);
      std::vector<float> lev;
      for (int l = 0; l < H.lm; ++l) {
        if (!spread(dev + (size_t)l * p.ldN + mh.off, lev)) return false;
        std::copy(lev.begin(), lev.end(), o.begin() + (size_t)l * n2);
      }
      return true;
    };
  };
  std::vector<float> mask_f(H.mask.begin(), H.mask.end());
  std::vector<float> depth_lm(H.depth.begin(), H.depth.end());
  std::vector<Field> F;
  if (H.stokes && H.lm > 0) {
    F.push_back({"z", "depth", "m", host2d(depth_lm), 3, false});
    F.push_back({"u_stokes", "stokes drift x-component", "m/s", stokes(P.us), 4, false});
    F.push_back({"v_stokes", "stokes drift y-component", "m/s", stokes(P.vs), 4, false});
    F.push_back({"d_stokes", "stokes drift e-folding depth", "m", wet(P.ds), 0, false});
  }
  F.push_back({"frequency", "frequency", "hz", host2d(H.f), 1, false});
  F.push_back({"theta", "directions", "rad", host2d(H.th), 2, false});
  F.push_back({"lon", "longitude", "degrees east", host2d(H.lon), 0, false});
  F.push_back({"lat", "latitude", "degrees north", host2d(H.lat), 0, false});
  F.push_back({"seamask", "seamask", "non-dimensional", host2d(mask_f), 0, true});
  F.push_back({"depth", "ocean depth", "m", host2d(H.d_2d), 0, false});
  F.push_back({"wspd", "wind speed", "m/s", allp(P.wspd), 0, false});
  F.push_back({"wdir", "wind direction", "rad", allp(P.wdir), 0, false});
  F.push_back({"uc", "ocean current, x-component", "m/s", allp(P.uc), 0, false});
  F.push_back({"vc", "ocean current, y-component", "m/s", allp(P.vc), 0, false});
  F.push_back({"rhoa", "air density", "kg/m^3", allp(P.rhoa), 0, false});
  F.push_back({"rhow", "water density", "kg/m^3", allp(P.rhow), 0, false});
  F.push_back({"fice", "seaice fraction", "non-dimensional", allp(P.fice), 0, false});
  F.push_back({"psim", "universal stability function for momentum", "non-dimensional",
               [&](std::vector<float>& o) {
                 o.assign(n2, nan);
                 for (int i = 1; i <= N; ++i) o[H.i2(H.mi[i], H.ni[i])] = 0.f;
                 return true;
               }, 0, false});
  F.push_back({"momx", "momentum, x-component", "kgm/s", wet(P.momx), 0, false});
  F.push_back({"momy", "momentum, y-component", "kgm/s", wet(P.momy), 0, false});
  F.push_back({"cgmxx", "cg*momentum, xx-component", "kgm^2/s^2", wet(P.cgmxx), 0, false});
  F.push_back({"cgmxy", "cg*momentum, xy-component", "kgm^2/s^2", wet(P.cgmxy), 0, false});
  F.push_back({"cgmyy", "cg*momentum, yy-component", "kgm^2/s^2", wet(P.cgmyy), 0, false});
  F.push_back({"shelt", "sheltering coefficient", "non-dimensional", wet(P.shelt), 0, false});
  F.push_back({"epsx_atm", "wave energy growth flux, x-component", "kg/s^3", ocn(OCN_EPSX_ATM), 0, false});
  F.push_back({"epsy_atm", "wave energy growth flux, y-component", "kg/s^3", ocn(OCN_EPSY_ATM), 0, false});
  F.push_back({"epsx_ocn", "wave energy dissipation flux, x-component", "kg/s^3", ocn(OCN_EPSX_OCN), 0, false});
  F.push_back({"epsy_ocn", "wave energy dissipation flux, y-component", "kg/s^3", ocn(OCN_EPSY_OCN), 0, false});
  F.push_back({"taux_form", "form drag, x-component", "n/m^2", wet(P.taux_form), 0, false});
  F.push_back({"tauy_form", "form drag, y-component", "n/m^2", wet(P.tauy_form), 0, false});
  F.push_back({"taux_form_1", "form drag, part 1, x-component", "n/m^2", ocn(OCN_TAUX1), 0, false});
  F.push_back({"tauy_form_1", "form drag, part 1, y-component", "n/m^2", ocn(OCN_TAUY1), 0, false});
  F.push_back({"taux_form_2", "form drag, part 2, x-component", "n/m^2", ocn(OCN_TAUX2), 0, false});
  F.push_back({"tauy_form_2", "form drag, part 2, y-component", "n/m^2", ocn(OCN_TAUY2), 0, false});
  F.push_back({"taux_form_3", "form drag, part 3, x-component", "n/m^2", ocn(OCN_TAUX3), 0, false});
  F.push_back({"tauy_form_3", "form drag, part 3, y-component", "n/m^2", ocn(OCN_TAUY3), 0, false});
  F.push_back({"taux_skin", "skin drag, x-component", "n/m^2", wet(P.taux_skin), 0, false});
  F.push_back({"tauy_skin", "skin drag, y-component", "n/m^2", wet(P.tauy_skin), 0, false});
  F.push_back({"taux_diag", "diagnostic form drag, x-component", "n/m^2", wet(P.taux_diag), 0, false});
  F.push_back({"tauy_diag", "diagnostic form drag, y-component", "n/m^2", wet(P.tauy_diag), 0, false});
  F.push_back({"taux_ocn", "momentum flux from breaking waves to ocean top, x-component", "n/m^2",
               ocn(OCN_TAUX_TOP), 0, false});
  F.push_back({"tauy_ocn", "momentum flux from breaking waves to ocean top, y-component", "n/m^2",
               ocn(OCN_TAUY_TOP), 0, false});
  F.push_back({"taux_bot", "momentum flux from waves to ocean bottom, x-component", "n/m^2", ocn(OCN_TAUX_BOT), 0,
               false});
  F.push_back({"tauy_bot", "momentum flux from waves to ocean bottom, y-component", "n/m^2", ocn(OCN_TAUY_BOT), 0,
               false});
  F.push_back({"taux_snl", "momentum flux due to snl, x-component", "n/m^2", ocn(OCN_TAUX_SNL), 0, false});
  F.push_back({"tauy_snl", "momentum flux due to snl, y-component", "n/m^2", ocn(OCN_TAUY_SNL), 0, false});
  F.push_back({"tailatmx", "atmosphere tail stress part, x-component", "n/m^2", wet(P.tailatmx), 0, false});
  F.push_back({"tailatmy", "atmosphere tail stress part, y-component", "n/m^2", wet(P.tailatmy), 0, false});
  F.push_back({"tailocnx", "ocean tail stress part, x-component", "n/m^2", ocn(OCN_TAILX), 0, false});
  F.push_back({"tailocny", "ocean tail stress part, y-component", "n/m^2", ocn(OCN_TAILY), 0, false});
  F.push_back({"cd", "drag coefficient of air", "non-dimensional", wet(P.cd), 0, false});
  F.push_back({"ust", "friction velocity of air", "m/s", wet(P.ustar), 0, false});
  F.push_back({"swh", "significant wave height", "m", wet(P.ht), 0, false});
  F.push_back({"mss", "mean-squared slope", "non-dimensional", wet(P.mss), 0, false});
  F.push_back({"mwp", "mean wave period", "s", wet(P.mwp), 0, false});
  F.push_back({"mwl", "mean wavelength", "m", wet(P.mwl), 0, false});
  F.push_back({"mwd", "mean wave direction", "rad", wet(P.mwd), 0, false});
  F.push_back({"dwp", "dominant wave period", "s", wet(P.dwp), 0, false});
  F.push_back({"dwl", "dominant wavelength", "m", wet(P.dwl), 0, false});
  F.push_back({"dwd", "dominant wave direction", "rad", wet(P.dwd), 0, false});
  F.push_back({"dcp0", "dominant phase speed, intrinsic", "m/s", wet(P.dcp0), 0, false});
  F.push_back({"dcg0", "dominant group speed, intrinsic", "m/s", wet(P.dcg0), 0, false});
  F.push_back({"dcp", "dominant phase speed", "m/s", wet(P.dcp), 0, false});
  F.push_back({"dcg", "dominant group speed", "m/s", wet(P.dcg), 0, false});
  F.push_back({"physics_time_step", "Physics time step", "s", wet(P.phys), 0, false});

  std::vector<std::pair<std::string, size_t>> dims = {
      {"x", (size_t)mm}, {"y", (size_t)nm}, {"f", (size_t)p.O}, {"th", (size_t)p.P}, {"time", 0}};
  const int X = 0, Y = 1, FD = 2, TH = 3, T = 4;
  if (H.stokes && H.lm > 0) dims.push_back({"z", (size_t)H.lm});
  const int Z = 5;
  std::vector<nc::Var> vars;
  std::vector<std::vector<float>> cache(F.size());
  bool ok = true;
  for (size_t q = 0; q < F.size(); ++q) {
    nc::Var v;
    v.name = F[q].name;
    v.atts = {{"description", F[q].desc}, {"units", F[q].units}};
    v.is_int = F[q].is_int;
    switch (F[q].kind) {
      case 1: v.dims = {FD}; break;
      case 2: v.dims = {TH}; break;
      case 3: v.dims = {Z}; break;
      case 4: v.dims = {T, Z, Y, X}; break;
      default: v.dims = {T, Y, X}; break;
    }
    v.fill = [&, q](size_t first, size_t n, float* out) {
      if (first == 0 && !F[q].make(cache[q])) {
        ok = false;
        return false;
      }
      if (first + n > cache[q].size()) return false;
      std::memcpy(out, cache[q].data() + first, n * 4);
      if (first + n == cache[q].size()) std::vector<float>().swap(cache[q]);
      return true;
    };
    vars.push_back(std::move(v));
  }
  std::string err;
  if (!nc::write(path, dims, vars, err)) return fail(ok ? UMWM_ERR_INPUT : UMWM_ERR_CUDA, "output_grid_nc: " + err);
  return UMWM_OK;
}

// The points of namelists/spectrum.nml, umwm_io.F90:178-227: a first line
// "xy" (grid indices m n, inside the open boundary) or "ll" (longitude,
// latitude: the nearest cell, the first in column-major order), then one
// point per line with its identifier.  A missing file means no points; land
// cells and boundary cells are kept and skipped at output (:229).
int spectrum_points(Model& M) {
  M.spec_read = true;
  M.spec_pts.clear();
  const HostModel& H = M.mem[0].H;
  std::FILE* f = std::fopen("namelists/spectrum.nml", "r");
  if (!f) return UMWM_OK;
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
  std::fclose(f);
  std::vector<std::string> lines;
  size_t a = 0;
  while (a <= text.size()) {
    size_t b = text.find('\n', a);
    if (b == std::string::npos) b = text.size();
    lines.push_back(text.substr(a, b - a));
    a = b + 1;
  }
  auto fields = [](const std::string& l) {  // list-directed: blanks and commas separate
    std::vector<std::string> out;
    std::string cur;
    for (char c : l) {
      if (c == ' ' || c == '\t' || c == ',' || c == '\r') {
        if (!cur.empty()) out.push_back(cur);
        cur.clear();
      } else {
        cur += c;
      }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
  };
  const std::string mode = lines.empty() ? "" : lines[0].substr(0, std::min<size_t>(2, lines[0].size()));
  const bool xy = mode == "xy" || mode == "XY", ll = mode == "ll" || mode == "LL";
  if (!xy && !ll)
    return fail(UMWM_ERR_INPUT, "output_spectrum_nc: first line in namelists/spectrum.nml must contain "
                                "\"xy\" (or \"XY\") or \"ll\" (or \"LL\")");
  for (size_t l = 1; l < lines.size(); ++l) {
    const std::vector<std::string> w = fields(lines[l]);
    if (w.size() < 3) continue;
    Model::SpecPoint sp;
    sp.id = w[2].substr(0, 40);
    if (xy) {
      sp.m = std::atoi(w[0].c_str());
      sp.n = std::atoi(w[1].c_str());
      if (sp.m < 2 || sp.m > H.mm - 1 || sp.n < 2 || sp.n > H.nm - 1)
        return fail(UMWM_ERR_INPUT, "output_spectrum_nc: a requested point in spectrum.nml is out of bounds");
    } else {
      const float lo = (float)std::atof(w[0].c_str()), la = (float)std::atof(w[1].c_str());
      float best = std::numeric_limits<float>::infinity();
      sp.m = sp.n = 1;
      for (int nn = 1; nn <= H.nm; ++nn)
        for (int mm = 1; mm <= H.mm; ++mm) {
          const float dx = lo - H.lon[H.i2(mm, nn)], dy = la - H.lat[H.i2(mm, nn)];
          const float d2 = dx * dx + dy * dy;
          if (d2 < best) {
            best = d2;
            sp.m = mm;
            sp.n = nn;
          }
        }
    }
    sp.i = H.ii[H.i2(sp.m, sp.n)];
    M.spec_pts.push_back(sp);
  }
  M.spec_recs.assign(M.spec_pts.size(), {});
  return UMWM_OK;
}

// output_spectrum_nc, umwm_io.F90:150-314: per wet point of spectrum.nml
// one file output/umwmspc_<id>_<time of the first output>.nc, one record per
// output (spectrum F, Sin, Sds after cothkd, Snl and Sdt of the last
// substep, wspd, wdir) with the static frequency, wavenumber, direction,
// position, Sdv and Sbf.  The records are kept on the host and each call
// writes the file again.
int output_spectrum(Model& M, int64_t t) {
  int rc;
  if (!M.spec_read && (rc = spectrum_points(M))) return rc;
  if (M.spec_time.empty()) M.spec_time = time_to_string(t, '_');
  const Params& p = M.prm;
  const MemberHost& mh = M.mem[0];
  const HostModel& H = mh.H;
  const int O = p.O, NPd = p.P;
  const size_t nb = (size_t)O * NPd;
  const size_t tstride = (size_t)p.NB * T_COUNT * 32;
  CU(cudaStreamSynchronize(M.st));
  float* tmp = nullptr;
  CU(cudaMalloc(&tmp, nb * 4));
  auto spectrum = [&](const float* src, int j, std::vector<float>& out) {
    out.resize(nb);
    cudaError_t e = launch_to_ref(p, src, tmp, j, 1, M.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M.st);
    if (e == cudaSuccess) e = cudaMemcpy(out.data(), tmp, nb * 4, cudaMemcpyDeviceToHost);
    return e;
  };
  auto row = [&](int t_, int j, std::vector<float>& out) {  // table row over o at point j
    out.resize(O);
    return cudaMemcpy2D(out.data(), 4, M.P.TAB + tidx(p, 0, t_, j), tstride * 4, 4, O, cudaMemcpyDeviceToHost);
  };
  cudaError_t e = cudaSuccess;
  for (size_t s = 0; s < M.spec_pts.size() && e == cudaSuccess; ++s) {
    const Model::SpecPoint& sp = M.spec_pts[s];
    if (sp.i < 1 || sp.i > mh.N) continue;  // land or boundary cell (ispec outside istart..iend)
    const int j = mh.off + sp.i - 1, ja = mh.nmoff + sp.i - 1;
    Model::SpecRec r;
    std::vector<float> k, sdv, sbf;
    float ust = 0.f, rhorat = 0.f;
    if ((e = spectrum(M.E, j, r.F)) || (e = spectrum(M.P.src_sin, j, r.Sin)) ||
        (e = spectrum(M.P.src_sds, j, r.Sds)) || (e = spectrum(M.P.src_snl, j, r.Snl)) || (e = row(T_K, j, k)) ||
        (e = row(T_SDV, j, sdv)) || (e = row(T_SBF, j, sbf)) ||
        (e = cudaMemcpy(&ust, M.P.src_ust + j, 4, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(&rhorat, M.P.rhorat + ja, 4, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(&r.wspd, M.P.wspd + ja, 4, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(&r.wdir, M.P.wdir + ja, 4, cudaMemcpyDeviceToHost)))
      break;
    // Sdt, umwm_source_functions.F90:179-181, with the ustar of that substep
    const float sdtc = (H.sdt_fac * std::sqrt(rhorat)) * ust;
    r.Sdt.resize(O);
    for (int o = 0; o < O; ++o) r.Sdt[o] = sdtc * k[o];
    M.spec_recs[s].push_back(std::move(r));
    const std::vector<Model::SpecRec>& recs = M.spec_recs[s];
    const std::string path = "output/umwmspc_" + sp.id + "_" + M.spec_time + ".nc";
    std::vector<std::pair<std::string, size_t>> dims = {
        {"scalar", 1}, {"frequency", (size_t)O}, {"direction", (size_t)NPd}, {"time", 0}};
    std::vector<nc::Var> vars;
    auto fixed = [&](const char* name, int dim, std::vector<float> v) {
      nc::Var x;
      x.name = name;
      x.dims = {dim};
      x.fill = [v](size_t first, size_t n, float* out) {
        if (first + n > v.size()) return false;
        std::memcpy(out, v.data() + first, n * 4);
        return true;
      };
      vars.push_back(std::move(x));
    };
    // a record variable from a per-record vector (size per record: n1)
    auto recvar = [&](const char* name, std::vector<int> d, size_t n1, std::function<const float*(const Model::SpecRec&)> get) {
      nc::Var x;
      x.name = name;
      x.dims = d;
      x.fill = [&recs, n1, get](size_t first, size_t n, float* out) {
        for (size_t q = 0; q < n; ++q) {
          const size_t g = first + q, r = g / n1;
          if (r >= recs.size()) return false;
          out[q] = get(recs[r])[g % n1];
        }
        return true;
      };
      vars.push_back(std::move(x));
    };
    fixed("frequency", 1, std::vector<float>(H.f.begin(), H.f.begin() + O));
    fixed("wavenumber", 1, k);
    fixed("direction", 2, std::vector<float>(H.th.begin(), H.th.begin() + NPd));
    fixed("longitude", 0, {H.lon[H.i2(sp.m, sp.n)]});
    fixed("latitude", 0, {H.lat[H.i2(sp.m, sp.n)]});
    recvar("wspd", {3, 0}, 1, [](const Model::SpecRec& x) { return &x.wspd; });
    recvar("wdir", {3, 0}, 1, [](const Model::SpecRec& x) { return &x.wdir; });
    recvar("F", {3, 2, 1}, nb, [](const Model::SpecRec& x) { return x.F.data(); });
    recvar("Sin", {3, 2, 1}, nb, [](const Model::SpecRec& x) { return x.Sin.data(); });
    recvar("Sds", {3, 2, 1}, nb, [](const Model::SpecRec& x) { return x.Sds.data(); });
    recvar("Sdt", {3, 1}, (size_t)O, [](const Model::SpecRec& x) { return x.Sdt.data(); });
    fixed("Sdv", 1, sdv);
    fixed("Sbf", 1, sbf);
    recvar("Snl", {3, 2, 1}, nb, [](const Model::SpecRec& x) { return x.Snl.data(); });
    std::string err;
    if (!nc::write(path, dims, vars, err, recs.size())) {
      std::fprintf(stderr, "umwm: output_spectrum_nc: %s not written (%s)\n", path.c_str(), err.c_str());
    } else if (M.verbose) {
      std::printf("umwm: output_spectrum_nc: spectrum written to %s\n", path.c_str());
    }
  }
  cudaFree(tmp);
  CU(e);
  return UMWM_OK;
}

// output/umwmout_<time>.nc; a file that cannot be written is reported and
// the run goes on, as the reference ignores the netCDF status there
void write_output_file(Model& M, int64_t t) {
  const std::string path = "output/umwmout_" + time_to_string(t, '_') + ".nc";
  if (output_grid(M, path) != UMWM_OK) {
    std::fprintf(stderr, "umwm: output_grid_nc: %s not written (%s)\n", path.c_str(), g_err.c_str());
    g_err.clear();
  } else if (M.verbose) {
    std::printf("umwm: output_grid_nc: written to %s\n", path.c_str());
  }
}

int check_ctl(Model& M) {
  std::vector<Ctl> c(M.mem.size());
  CU(cudaMemcpy(c.data(), M.mem[0].ctl, c.size() * sizeof(Ctl), cudaMemcpyDeviceToHost));
  for (auto& x : c)
    if (x.err) return fail(UMWM_ERR_TIMEOUT, "a device-side wait gave up");
  return UMWM_OK;
}

bool dir_exists(const char* path) {
  struct stat st;
  return ::stat(path, &st) == 0 && S_ISDIR(st.st_mode);
}

// Buffers of stress('ocn'): the last substep's source terms and the outputs.
// Allocated on first use; a captured inner loop holds the old pointers and is
// rebuilt.
int ensure_ocn(Model& M) {
  if (M.P.src_sin) return UMWM_OK;
  const size_t spec = (size_t)M.prm.O * M.prm.P * M.prm.ldN;
  Dev& D = *M.dev;
  CU(D.alloc(&M.P.src_sin, spec, false));
  CU(D.alloc(&M.P.src_sds, spec, false));
  CU(D.alloc(&M.P.src_snl, spec, false));
  CU(D.alloc(&M.P.src_ust, (size_t)M.prm.ldN));
  CU(D.alloc(&M.P.ocn, (size_t)OCN_COUNT * M.prm.ldN));
  if (M.graph_exec) { cudaGraphExecDestroy(M.graph_exec); M.graph_exec = nullptr; }
  if (M.graph) { cudaGraphDestroy(M.graph); M.graph = nullptr; }
  return UMWM_OK;
}

// Enqueue the launches of one substep: prep, [sice], phys, dts, integ,
// advect, [diag on the first substep of a run], screen.
int enqueue_substep(Model& M, int compute_rot, int first, bool diag) {
  const Params& prm = M.prm;
  const Ptrs& P = M.P;
  CU(timed(M, K_PREP, [&] { return launch_prep(prm, P, compute_rot, M.max_nm, M.st); }));
  if (prm.ice_possible) CU(timed(M, K_SICE, [&] { return launch_sice(prm, P, M.st); }));
  CU(tuned(M, TK_PHYS, K_PHYS, [&] { return launch_source_phys(prm, P, compute_rot, M.st); }));
  CU(timed(M, K_DTS, [&] { return launch_dts(prm, P, compute_rot, first, M.st); }));
  int rc;
  if (sur::active()) {
    // learned source step; points outside its energy budget fall back to
    // the plain integration (flagged tiles and points only)
    Ptrs fbP;
    if ((rc = sur::step(prm, P, fbP, M.st))) return rc;
    CU(timed(M, K_INTEG, [&] { return launch_source_integ(prm, fbP, M.st); }));
  } else {
    if (sur::capturing() && (rc = sur::capture_before(prm, P, M.wet_ranges, M.st))) return rc;
    CU(tuned(M, TK_INTEG, K_INTEG, [&] { return launch_source_integ(prm, P, M.st); }));
    if (sur::capturing() && (rc = sur::capture_after(prm, P, M.st))) return rc;
  }
  CU(tuned(M, TK_ADVECT, K_ADVECT, [&] { return launch_advect(prm, P, M.st); }));
  if (diag) CU(timed(M, K_DIAG, [&] { return launch_diag(prm, P, M.st); }));
  CU(timed(M, K_SCREEN, [&] { return launch_screen(prm, P, M.st); }));
  return UMWM_OK;
}

int substep_launches(const Model& M, bool diag) { return 6 + (M.prm.ice_possible ? 1 : 0) + (diag ? 1 : 0); }

int substep(Model& M) {
  const bool first = M.first;
  // the tuner measures from the second substep of the model on
  if (M.tune.active && first) {
    for (int k = 0; k < TK_N; ++k) tune_set(M.prm, k, M.tune.k[k].cands[0]);
    M.tune.active = false;  // not measured: the first substep also runs diag
    int rc = enqueue_substep(M, (M.prm.currents || first) ? 1 : 0, 1, true);
    M.tune.active = true;
    if (rc) return rc;
    M.launches += substep_launches(M, true);
    M.first = false;
    M.substeps++;
    return UMWM_OK;
  }
  if (M.tune.active) tune_apply(M);
  int rc = enqueue_substep(M, (M.prm.currents || first) ? 1 : 0, first ? 1 : 0, first);
  if (rc) return rc;
  M.launches += substep_launches(M, first);
  M.first = false;
  M.substeps++;
  return UMWM_OK;
}

// The inner loop of umwm_run as a CUDA graph: one while node whose body is a
// substep (after the first of a run: compute_rot = currents, first = 0)
// followed by k_loop_cond, which keeps the loop going while a member is
// inside the dtg and the armed budget lasts.  Launch parameters are fixed
// after initialize (forcing updates are device copies into fixed buffers), so
// the graph is built once per model.
int build_graph(Model& M) {
  if (M.graph_exec) return UMWM_OK;
  CU(cudaGraphCreate(&M.graph, 0));
  cudaGraphConditionalHandle h;
  CU(cudaGraphConditionalHandleCreate(&h, M.graph, 1u, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CU(cudaGraphAddNode(&node, M.graph, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CU(cudaStreamBeginCaptureToGraph(M.st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const bool kt = M.ktime;
  M.ktime = false;
  int rc = enqueue_substep(M, M.prm.currents ? 1 : 0, 0, false);
  cudaError_t e = rc ? cudaSuccess : launch_loop_cond(M.d_glob, h, M.st);
  M.ktime = kt;
  cudaGraph_t captured = nullptr;
  cudaError_t ec = cudaStreamEndCapture(M.st, &captured);
  if (rc) return rc;
  CU(e);
  CU(ec);
  CU(cudaGraphInstantiate(&M.graph_exec, M.graph, 0));
  return UMWM_OK;
}

// Substeps one graph launch may run before control returns to the host,
// which then relaunches it (bounded device-side loop).
constexpr int GRAPH_CHUNK = 4096;

void print_screen(Model& M) {
  MemberHost& mh = M.mem[0];
  int cnt = 0;
  if (cudaMemcpy(&cnt, &mh.ctl->log_count, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return;
  if ((size_t)cnt <= mh.screen_printed) return;
  std::vector<double> rows((size_t)(cnt - mh.screen_printed) * 8);
  cudaMemcpy(rows.data(), mh.log + mh.screen_printed * 8, rows.size() * 8, cudaMemcpyDeviceToHost);
  for (size_t r = 0; r < rows.size() / 8; ++r) {
    const double* L = &rows[r * 8];
    std::printf("  %4.2f  %8.3f %9.6f %9.6f %9.6f %9.6f %9.6f %9.6f\n", L[0], L[1], L[2], L[3], L[4], L[5], L[6], L[7]);
  }
  mh.screen_printed = cnt;
  std::fflush(stdout);
}

int member_substeps(Model& M, std::vector<int>& out) {
  std::vector<Ctl> c(M.mem.size());
  CU(cudaMemcpy(c.data(), M.mem[0].ctl, c.size() * sizeof(Ctl), cudaMemcpyDeviceToHost));
  out.resize(c.size());
  for (size_t m = 0; m < c.size(); ++m) out[m] = c[m].substep;
  return UMWM_OK;
}

int finish_run(Model& M) {
  CU(cudaEventRecord(M.ev1, M.st));
  CU(cudaEventSynchronize(M.ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, M.ev0, M.ev1);
  M.last_gpu_ms = ms;
  std::vector<int> sub;
  int rc = member_substeps(M, sub);
  if (rc) return rc;
  double bins = 0;
  for (size_t m = 0; m < M.mem.size(); ++m)
    bins += (double)(sub[m] - M.mem[m].substep_mark) * M.mem[m].N * M.prm.O * M.prm.P;
  M.last_bins = bins;
  collect_timings(M);
  return check_ctl(M);
}

int run_impl(Model& M, const std::string& start, const std::string& stop) {
  int64_t t0, t1;
  if (!time_from_string(start, t0) || !time_from_string(stop, t1))
    return fail(UMWM_ERR_ARG, "umwm_run: times must be 'YYYY-MM-DD hh:mm:ss'");
  int rc;
  if (M.first && M.prm.restart)
    for (size_t m = 0; m < M.mem.size(); ++m)
      if ((rc = restart_read(M, (int)m, time_key(start.c_str()))) != UMWM_OK) return rc;
  {
    std::vector<int> sub;
    if ((rc = member_substeps(M, sub))) return rc;
    for (size_t m = 0; m < M.mem.size(); ++m) M.mem[m].substep_mark = sub[m];
  }
  // the first substep of a model also writes output/umwmout_<start>.nc
  // (umwm_top.F90:121-127), without stress('ocn'): its fields are zero
  bool first_out = M.first && M.mem[0].H.outgrid > 0 && M.mem.size() == 1 && dir_exists("output");
  if (first_out && (rc = ensure_ocn(M))) return rc;
  // and output/umwmspc_*.nc with that substep's source terms (umwm_top.F90:128)
  bool first_spec = M.first && M.mem[0].H.outspec > 0 && M.mem.size() == 1 && dir_exists("output");
  if (first_spec) {
    if ((rc = ensure_ocn(M))) return rc;
    static const int one = 1;
    CU(cudaMemcpyAsync(&M.d_glob->save_src, &one, sizeof(int), cudaMemcpyHostToDevice, M.st));
  }
  CU(cudaEventRecord(M.ev0, M.st));
  int64_t now = t0;
  while (now < t1) {
    now += std::llround((double)M.prm.dtg);
    const std::string cur = time_to_string(now, '_');
    if (M.verbose) std::printf("umwm: solver: integrating to time: %s\n", cur.c_str());
    for (MemberHost& mh : M.mem)
      if ((rc = forcing_input(M, mh, cur))) return rc;
    CU(launch_begin_dtg(M.prm, M.st));  // sumt = 0, done = 0 for every member
    // stress('ocn') is due after this step (umwm_top.F90:160-171)
    const HostModel& H0 = M.mem[0].H;
    const int64_t sod = now % 86400;
    const bool grid_due = (H0.outgrid > 0 && (sod / 3600) % H0.outgrid == 0 && sod % 3600 == 0) || H0.outgrid == -1;
    // gridded output goes to output/umwmout_<time>.nc when that directory
    // exists (the reference's nf90_create fails there silently otherwise);
    // ensembles write none
    const bool grid_write = grid_due && M.mem.size() == 1 && dir_exists("output");
    // spectrum output at the times outspec asks for (umwm_top.F90:175-181)
    const bool spec_due = (H0.outspec > 0 && (sod / 3600) % H0.outspec == 0 && sod % 3600 == 0) || H0.outspec == -1;
    const bool spec_write = spec_due && M.mem.size() == 1 && dir_exists("output");
    const bool ocn_due = M.ocn_every || grid_write || spec_write;
    if (ocn_due) {
      if ((rc = ensure_ocn(M))) return rc;
      static const int one = 1;
      CU(cudaMemcpyAsync(&M.d_glob->save_src, &one, sizeof(int), cudaMemcpyHostToDevice, M.st));
    }
    for (long long inner = 0;;) {
      if (inner > 10000000LL) return fail(UMWM_ERR_TIMEOUT, "umwm_run: more than 1e7 substeps in one dtg (dts stuck at 0?)");
      if (M.max_substeps >= 0 && M.substeps >= M.max_substeps) return finish_run(M);
      if (M.persistent && !M.first && !M.ktime && !M.tune.active && !sur::active() && !sur::capturing() &&
          persist_supported(M.prm)) {
        long long budget = GRAPH_CHUNK;
        if (M.max_substeps >= 0) budget = std::min(budget, M.max_substeps - M.substeps);
        CU(launch_loop_arm(M.d_glob, (int)budget, M.st));
        if ((rc = persist_launch(M))) return rc;
        CU(cudaMemcpyAsync(M.flag_h, M.d_glob, sizeof(Global), cudaMemcpyDeviceToHost, M.st));
        CU(cudaStreamSynchronize(M.st));
        if (M.flag_h->bar_err)
          return fail(UMWM_ERR_TIMEOUT, "umwm_run: a grid barrier wait of the persistent substep kernel ran out");
        const int it = M.flag_h->iters;
        M.substeps += it;
        M.launches += 3;
        inner += it;
        if (M.flag_h->not_done == 0) break;
        continue;
      }
      if (M.use_graph && !M.first && !M.ktime && !M.tune.active && !sur::active() && !sur::capturing()) {
        if ((rc = build_graph(M))) return rc;
        long long budget = GRAPH_CHUNK;
        if (M.max_substeps >= 0) budget = std::min(budget, M.max_substeps - M.substeps);
        CU(launch_loop_arm(M.d_glob, (int)budget, M.st));
        CU(cudaGraphLaunch(M.graph_exec, M.st));
        CU(cudaMemcpyAsync(M.flag_h, M.d_glob, sizeof(Global), cudaMemcpyDeviceToHost, M.st));
        CU(cudaStreamSynchronize(M.st));
        const int it = M.flag_h->iters;
        M.substeps += it;
        M.launches += 1 + (long long)it * (substep_launches(M, false) + 1);
        inner += it;
        if (M.flag_h->not_done == 0) break;
        continue;
      }
      if ((rc = substep(M))) return rc;
      ++inner;
      if (first_out) {
        first_out = false;
        write_output_file(M, t0);
      }
      if (first_spec) {
        first_spec = false;
        if ((rc = output_spectrum(M, t0))) return rc;
        const int keep = ocn_due ? 1 : 0;  // the step's own stress('ocn') or output still needs them
        CU(cudaMemcpy(&M.d_glob->save_src, &keep, sizeof(int), cudaMemcpyHostToDevice));
      }
      CU(cudaMemcpyAsync(M.flag_h, M.d_glob, sizeof(Global), cudaMemcpyDeviceToHost, M.st));
      CU(cudaStreamSynchronize(M.st));
      collect_timings(M);
      tune_collect(M);
      if (M.flag_h->not_done == 0) break;
    }
    if (M.mem[0].H.stokes && M.prm.lm > 0) {
      CU(timed(M, K_STOKES, [&] { return launch_stokes(M.prm, M.P, M.st); }));
      M.launches++;
    }
    CU(timed(M, K_DIAG, [&] { return launch_diag(M.prm, M.P, M.st); }));
    M.launches++;
    if (ocn_due) {
      static const int zero = 0;
      CU(launch_stress_ocn(M.prm, M.P, M.st));
      CU(cudaMemcpyAsync(&M.d_glob->save_src, &zero, sizeof(int), cudaMemcpyHostToDevice, M.st));
      M.launches++;
    }
    if (grid_write) write_output_file(M, now);
    if (spec_write && (rc = output_spectrum(M, now))) return rc;
    if (M.verbose) print_screen(M);
    // restart output, umwm_top.F90:183-190 (with the reference's test of
    // outspec == -1 for writing every step)
    {
      const HostModel& H0 = M.mem[0].H;
      const int64_t secs = now % 86400;
      const bool fullhour = secs % 3600 == 0;
      const int hour = (int)(secs / 3600);
      if ((H0.outrst > 0 && hour % H0.outrst == 0 && fullhour) || (H0.outrst <= 0 && H0.outspec == -1)) {
        // like the reference (which ignores the netCDF status here), a file
        // that cannot be written is reported and the run goes on
        const std::string key = time_to_string(now, '_');
        for (size_t m = 0; m < M.mem.size(); ++m) {
          const std::string path = restart_path(M, (int)m, key);
          if (restart_write(M, (int)m, path) != UMWM_OK) {
            std::fprintf(stderr, "umwm: restart_write: %s not written (%s)\n", path.c_str(), g_err.c_str());
            g_err.clear();
          } else if (M.verbose) {
            std::printf("umwm: restart_write: restart written to %s\n", path.c_str());
          }
        }
      }
    }
    if (M.check_finite) {
      // a NaN/Inf bin makes its point's significant wave height non-finite
      CU(cudaMemsetAsync(&M.d_glob->nonfinite, 0, sizeof(int), M.st));
      CU(launch_count_nonfinite(M.P.ht, (size_t)M.prm.ldN, &M.d_glob->nonfinite, M.st));
      CU(launch_count_nonfinite(M.P.ustar, (size_t)M.prm.ldN, &M.d_glob->nonfinite, M.st));
      M.launches += 2;
      CU(cudaMemcpyAsync(M.flag_h, M.d_glob, sizeof(Global), cudaMemcpyDeviceToHost, M.st));
      CU(cudaStreamSynchronize(M.st));
      if (M.flag_h->nonfinite)
        return fail(UMWM_ERR_NONFINITE, "umwm_run: non-finite significant wave height or friction velocity after "
                                        "the step to " + cur);
    }
  }
  return finish_run(M);
}

int init_common(std::vector<Pending>& members, bool device) {
  g_model.reset();
  std::unique_ptr<Model> M(new Model());
  M->mem.resize(members.size());
  for (size_t m = 0; m < members.size(); ++m) {
    MemberHost& mh = M->mem[m];
    mh.in = std::move(members[m].in);
    if (!mh.H.read_namelist(members[m].nml)) return fail(UMWM_ERR_NAMELIST, mh.H.err);
    // nothing staged: the reference's file input/umwm.gridtopo (umwm_init.F90:397-427, :541-546)
    const std::pair<bool, const char*> want[] = {
        {mh.H.gridfromfile, "lon"}, {mh.H.gridfromfile, "lat"}, {mh.H.topofromfile, "z"}};
    for (auto& w : want) {
      if (!w.first || mh.in.gridtopo.count(w.second)) continue;
      std::vector<size_t> sh;
      std::vector<float> v;
      std::string err;
      if (nc::read_float("input/umwm.gridtopo", w.second, sh, v, err)) mh.in.gridtopo[w.second] = std::move(v);
    }
    if (!mh.H.build(mh.in)) return fail(UMWM_ERR_INPUT, mh.H.err);
  }
  if (device) {
    int rc = init_device(*M);
    if (rc) return rc;
  }
  g_model = std::move(M);
  g_err.clear();
  return UMWM_OK;
}

int init_single(const std::string& text, bool device) {
  std::vector<Pending> one(1);
  one[0].nml = text;
  one[0].in = g_inputs;  // staged inputs are kept for later initializations
  return init_common(one, device);
}

Model* need_model(bool device) {
  if (!g_model) { fail(UMWM_ERR_STATE, "the model is not initialized"); return nullptr; }
  if (device && !g_model->on_device) { fail(UMWM_ERR_STATE, "the model has no device state (setup_host only)"); return nullptr; }
  return g_model.get();
}

// ---------------------------------------------------------------------------
// umwm_gpu_get_state_noalloc: the state read-back without device allocation.
//
// umwm_gpu_get_state transposes the spectrum into a temporary device buffer as
// large as the spectrum itself (om*pm*im floats, 4.2 GB on a 1000x1000 grid),
// allocated and freed on every call.  Some callers cannot do that: a job whose
// GPU memory is fully committed to an ensemble or to another model's pool
// allocator (the temporary would not fit, and a failed checkpoint loses the
// run), or a time-critical coupling loop that must not pay cudaFree's implicit
// device-wide synchronisation.  This variant streams the transpose through a
// fixed scratch area compiled into the library instead.
//
// The scratch is a file-scope __device__ array of NOALLOC_SCRATCH_FLOATS
// floats (16 MiB).  Every GPU that loads the library holds it until the
// process exits.  The spectrum goes through it in chunks of whole wet points
// (NOALLOC_SCRATCH_FLOATS / (om*pm) points per chunk, 3149 for om=37, pm=36),
// one transpose launch and one device-to-host copy per chunk, all on the
// model's stream.  A single point's spectrum larger than the scratch is
// rejected with UMWM_ERR_ARG.
//
// Every call shares the one array and leaves the last chunk in it.  Each chunk
// is written entirely before it is copied out, so nothing has to start at
// zero.  Calls that overlap on the GPU (two host threads, or a call racing a
// kernel launched by another thread on the same device) race on the scratch.
// ---------------------------------------------------------------------------
constexpr size_t NOALLOC_SCRATCH_FLOATS = (size_t)4 << 20;
static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_SCRATCH_FLOATS];

// per-device address of the scratch array, looked up once per device; the
// lock makes concurrent first calls from several host threads safe (the
// scratch itself is still shared, see above)
struct NoallocSlot {
  int device;
  float* ptr;
};
std::vector<NoallocSlot> g_noalloc_slots;
std::mutex g_noalloc_mu;

int noalloc_scratch(float** out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  for (const auto& s : g_noalloc_slots)
    if (s.device == dev) {
      *out = s.ptr;
      return UMWM_OK;
    }
  // first call on this device: resolve the array's device address with this
  // device current (the host-side symbol is only a stand-in, not a device
  // address)
  float* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
  if (e != cudaSuccess) return fail(UMWM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  g_noalloc_slots.push_back({dev, p});
  *out = p;
  return UMWM_OK;
}

}  // namespace

int set_error(int code, const std::string& msg) { return fail(code, msg); }

}  // namespace umwm

using namespace umwm;

extern "C" {

int umwm_gpu_put_gridtopo(const char* var, const float* field, int mm, int nm) {
  if (!var || !field || mm < 1 || nm < 1) return fail(UMWM_ERR_ARG, "put_gridtopo: bad arguments");
  std::string v(var);
  if (v != "lon" && v != "lat" && v != "z") return fail(UMWM_ERR_ARG, "put_gridtopo: variable must be lon, lat or z");
  g_inputs.gridtopo[v].assign(field, field + (size_t)mm * nm);
  return UMWM_OK;
}

int umwm_gpu_put_exclude(const int* mn, int npairs) {
  if (npairs < 0 || (npairs > 0 && !mn)) return fail(UMWM_ERR_ARG, "put_exclude: bad arguments");
  g_inputs.exclude.clear();
  for (int q = 0; q < npairs; ++q) g_inputs.exclude.push_back({mn[2 * q], mn[2 * q + 1]});
  return UMWM_OK;
}

int umwm_gpu_put_forcing(const char* time19, const char* var, const float* field, int mm, int nm) {
  if (!time19 || !var || !field || mm < 1 || nm < 1) return fail(UMWM_ERR_ARG, "put_forcing: bad arguments");
  std::string v(var);
  static const char* ok[] = {"uw", "vw", "uc", "vc", "rhoa", "rhow", "fice"};
  if (std::find_if(std::begin(ok), std::end(ok), [&](const char* s) { return v == s; }) == std::end(ok))
    return fail(UMWM_ERR_ARG, "put_forcing: unknown variable " + v);
  int64_t t;
  if (!time_from_string(time19, t)) return fail(UMWM_ERR_ARG, "put_forcing: bad time string");
  g_inputs.forcing[time_key(time19)][v].assign(field, field + (size_t)mm * nm);
  return UMWM_OK;
}

int umwm_gpu_put_restart(const char* time19, const float* F, long nF, const float* ust, long nust) {
  if (!time19 || !F || !ust || nF < 0 || nust < 0) return fail(UMWM_ERR_ARG, "put_restart: bad arguments");
  g_inputs.restarts[time_key(time19)] = {std::vector<float>(F, F + nF), std::vector<float>(ust, ust + nust)};
  return UMWM_OK;
}

int umwm_gpu_clear_inputs(void) {
  g_inputs = Inputs();
  return UMWM_OK;
}

int umwm_gpu_initialize_text(const char* text) {
  if (!text) return fail(UMWM_ERR_ARG, "initialize: null namelist");
  return init_single(text, true);
}

int umwm_gpu_initialize(const char* path) {
  std::string p = path ? path : "namelists/main.nml";
  std::ifstream f(p);
  if (!f) return fail(UMWM_ERR_NAMELIST, "cannot open namelist " + p);
  std::stringstream ss;
  ss << f.rdbuf();
  return init_single(ss.str(), true);
}

int umwm_gpu_setup_host(const char* text) {
  if (!text) return fail(UMWM_ERR_ARG, "setup_host: null namelist");
  return init_single(text, false);
}

int umwm_gpu_ensemble_add(const char* nml_text) {
  if (!nml_text) return fail(UMWM_ERR_ARG, "ensemble_add: null namelist");
  Pending pm;
  pm.nml = nml_text;
  pm.in = std::move(g_inputs);
  g_inputs = Inputs();
  g_pending.push_back(std::move(pm));
  return UMWM_OK;
}

int umwm_gpu_ensemble_initialize(void) {
  if (g_pending.empty()) return fail(UMWM_ERR_STATE, "ensemble_initialize: no member added");
  std::vector<Pending> members = std::move(g_pending);
  g_pending.clear();
  return init_common(members, true);
}

int umwm_gpu_select_member(int m) {
  Model* M = need_model(false);
  if (!M) return UMWM_ERR_STATE;
  if (m < 0 || m >= (int)M->mem.size()) return fail(UMWM_ERR_ARG, "select_member: no such member");
  M->sel = m;
  return UMWM_OK;
}

int umwm_gpu_run(const char* start, const char* stop) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  if (!start || !stop) return fail(UMWM_ERR_ARG, "run: null time");
  return run_impl(*M, start, stop);
}

int umwm_gpu_finalize(void) {
  g_model.reset();
  sur::release_model_buffers();
  return UMWM_OK;
}

int umwm_gpu_get_dims(int* dims) {
  Model* M = need_model(false);
  if (!M) return UMWM_ERR_STATE;
  if (!dims) return fail(UMWM_ERR_ARG, "get_dims: null");
  const HostModel& H = M->mem[M->sel].H;
  int v[8] = {H.mm, H.nm, H.om, H.pm, H.im, H.imm, H.lm, (int)M->substeps};
  std::memcpy(dims, v, sizeof v);
  return UMWM_OK;
}

int umwm_gpu_set_state(const float* F, const float* ust) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  return set_state_member(*M, M->sel, F, ust);
}

int umwm_gpu_get_state(float* F, float* ust) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  const Params& p = M->prm;
  const MemberHost& mh = M->mem[M->sel];
  CU(cudaStreamSynchronize(M->st));
  if (F) {
    const size_t n = (size_t)p.O * p.P * mh.N;
    float* tmp = nullptr;
    CU(cudaMalloc(&tmp, n * 4));
    cudaError_t e = launch_to_ref(p, M->E, tmp, mh.off, mh.N, M->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
    if (e == cudaSuccess) e = cudaMemcpy(F, tmp, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    CU(e);
  }
  if (ust) CU(cudaMemcpy(ust, M->P.ustar + mh.off, (size_t)mh.N * 4, cudaMemcpyDeviceToHost));
  return UMWM_OK;
}

int umwm_gpu_write_output(const char* path) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  if (!path) return fail(UMWM_ERR_ARG, "write_output: null path");
  if (M->mem.size() != 1) return fail(UMWM_ERR_UNSUPPORTED, "write_output: one-member models only");
  if (!M->P.ocn) return fail(UMWM_ERR_STATE, "write_output: stress('ocn') has not run (option stress_ocn)");
  return output_grid(*M, path);
}

int umwm_gpu_write_restart(const char* path) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  if (!path) return fail(UMWM_ERR_ARG, "write_restart: null path");
  return restart_write(*M, M->sel, path);
}

// Surrogate input rows of the selected member's wet points for the current
// state (the dts of the last substep), as f32 (n x 1344).
int umwm_gpu_surrogate_features(float* X, long n) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  const Params& p = M->prm;
  const MemberHost& mh = M->mem[M->sel];
  if (!X || n != (long)mh.N * sur::FPAD) return fail(UMWM_ERR_ARG, "surrogate_features: n must be im * 1344");
  if (p.O * p.P + sur::NEXTRA > sur::FPAD) return fail(UMWM_ERR_UNSUPPORTED, "surrogate: om*pm + 9 > 1344");
  __nv_bfloat16* d = nullptr;
  const size_t rows = (size_t)mh.padded;
  CU(cudaMalloc(&d, rows * sur::FPAD * 2));
  std::vector<int> pts(rows);
  for (size_t r = 0; r < rows; ++r) pts[r] = mh.off + (int)r;
  int* dp = nullptr;
  cudaError_t e = cudaMalloc(&dp, rows * 4);
  if (e == cudaSuccess) e = cudaMemcpy(dp, pts.data(), rows * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = sur::launch_features(p, M->P, dp, (int)rows, d, nullptr, nullptr, M->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
  std::vector<uint16_t> h((size_t)mh.N * sur::FPAD);
  if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, h.size() * 2, cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(dp);
  CU(e);
  for (size_t i = 0; i < h.size(); ++i) {
    const uint32_t u = (uint32_t)h[i] << 16;
    std::memcpy(&X[i], &u, 4);
  }
  return UMWM_OK;
}

// See the note at g_noalloc_scratch: the state read-back without any device
// allocation, through the library's fixed scratch area.  The first call on a
// device looks up the scratch address on that device (cudaGetSymbolAddress),
// so make the first call before any stream capture begins.
int umwm_gpu_get_state_noalloc(float* F, float* ust) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  const Params& p = M->prm;
  const MemberHost& mh = M->mem[M->sel];
  const size_t R = (size_t)p.O * p.P;
  if (R > NOALLOC_SCRATCH_FLOATS)
    return fail(UMWM_ERR_ARG, "get_state_noalloc: one point's spectrum (om*pm floats) exceeds the 16 MiB scratch");
  float* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  if (F) {
    const int chunk = (int)(NOALLOC_SCRATCH_FLOATS / R);
    for (int j0 = 0; j0 < mh.N; j0 += chunk) {
      const int nj = std::min(chunk, mh.N - j0);
      CU(launch_to_ref(p, M->E, scratch, mh.off + j0, nj, M->st));
      CU(cudaMemcpyAsync(F + (size_t)j0 * R, scratch, (size_t)nj * R * sizeof(float), cudaMemcpyDeviceToHost, M->st));
      // the next chunk overwrites the scratch: wait for this copy
      CU(cudaStreamSynchronize(M->st));
    }
  }
  if (ust) {
    CU(cudaMemcpyAsync(ust, M->P.ustar + mh.off, (size_t)mh.N * 4, cudaMemcpyDeviceToHost, M->st));
    CU(cudaStreamSynchronize(M->st));
  }
  return UMWM_OK;
}

int umwm_gpu_get_field(const char* name, float* out, long n) {
  Model* M = need_model(false);
  if (!M) return UMWM_ERR_STATE;
  if (!name || !out) return fail(UMWM_ERR_ARG, "get_field: null argument");
  const MemberHost& mh = M->mem[M->sel];
  const HostModel& H = mh.H;
  const std::string s(name);
  const int N = H.im, NM = H.imm, O = H.om;
  auto need = [&](long k) { return n >= k ? UMWM_OK : fail(UMWM_ERR_ARG, "get_field: buffer too small for " + s); };
  // host-side setup fields
  auto wet_host = [&](const std::vector<float>& v) {
    if (need(N)) return UMWM_ERR_ARG;
    for (int i = 1; i <= N; ++i) out[i - 1] = v[i];
    return UMWM_OK;
  };
  auto imm_host = [&](const std::vector<float>& v) {
    if (need(NM)) return UMWM_ERR_ARG;
    for (int i = 1; i <= NM; ++i) out[i - 1] = v[i];
    return UMWM_OK;
  };
  auto scalar = [&](float v) {
    if (need(1)) return UMWM_ERR_ARG;
    out[0] = v;
    return UMWM_OK;
  };
  // source terms the last stress('ocn') step kept (its last substep's Sin,
  // Sds after cothkd and Snl), in the reference's (i, th, f) layout
  if (s == "ssin" || s == "sds" || s == "snl") {
    if (!M->P.src_sin) return fail(UMWM_ERR_STATE, "get_field: " + s + " is kept by stress('ocn') steps only");
    const size_t cnt = (size_t)M->prm.O * M->prm.P * mh.N;
    if (need((long)cnt)) return UMWM_ERR_ARG;
    const float* src = s == "ssin" ? M->P.src_sin : s == "sds" ? M->P.src_sds : M->P.src_snl;
    float* tmp = nullptr;
    CU(cudaMalloc(&tmp, cnt * 4));
    cudaError_t e = launch_to_ref(M->prm, src, tmp, mh.off, mh.N, M->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, tmp, cnt * 4, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    CU(e);
    return UMWM_OK;
  }
  if (s == "ar") return wet_host(H.ar);
  if (s == "oneovar") return wet_host(H.oneovar);
  if (s == "oneovdx") return wet_host(H.oneovdx);
  if (s == "oneovdy") return wet_host(H.oneovdy);
  if (s == "dxn") return wet_host(H.dxn);
  if (s == "dxs") return wet_host(H.dxs);
  if (s == "dye") return wet_host(H.dye);
  if (s == "dyw") return wet_host(H.dyw);
  if (s == "d") return imm_host(H.d);
  if (s == "dx") return imm_host(H.dx);
  if (s == "dy") return imm_host(H.dy);
  if (s == "f" || s == "th" || s == "depth") {
    const std::vector<float>& v = s == "f" ? H.f : (s == "th" ? H.th : H.depth);
    if (need((long)v.size())) return UMWM_ERR_ARG;
    std::copy(v.begin(), v.end(), out);
    return UMWM_OK;
  }
  if (s == "dtamin") return scalar(H.dtamin);
  if (s == "cgmax") return scalar(H.cgmax);
  if (s == "dth") return scalar(H.dth);
  if (s == "d_2d" || s == "dx_2d" || s == "dy_2d" || s == "curv" || s == "lon" || s == "lat") {
    const std::vector<float>& v = s == "d_2d"    ? H.d_2d
                                  : s == "dx_2d" ? H.dx_2d
                                  : s == "dy_2d" ? H.dy_2d
                                  : s == "lon"   ? H.lon
                                  : s == "lat"   ? H.lat
                                                 : H.curv;
    if (need((long)v.size())) return UMWM_ERR_ARG;
    std::copy(v.begin(), v.end(), out);
    return UMWM_OK;
  }
  // tables (om, im) with o fastest; cp0/cg0 (om, 0:im)
  static const std::pair<const char*, int> tabs[] = {
      {"k", T_K}, {"cp0", T_CP0}, {"cg0", T_CG0}, {"logl2overz", T_LOGL2Z}, {"fkovg", T_FKOVG}, {"k4", T_K4},
      {"k3dk", T_K3DK}, {"kdk", T_KDK}, {"cothkd", T_COTHKD}, {"sbf", T_SBF}, {"sdv", T_SDV},
      {"bf1_renorm", T_BF1R}, {"bf2_renorm", T_BF2R}};
  for (auto& t : tabs)
    if (s == t.first) {
      const bool ghost = (t.second == T_CP0 || t.second == T_CG0);
      const std::vector<float>& src = t.second == T_K ? H.k : t.second == T_CP0 ? H.cp0 : t.second == T_CG0 ? H.cg0
          : t.second == T_LOGL2Z ? H.logl2overz : t.second == T_FKOVG ? H.fkovg : t.second == T_K4 ? H.k4
          : t.second == T_K3DK ? H.k3dk : t.second == T_KDK ? H.kdk : t.second == T_COTHKD ? H.cothkd
          : t.second == T_SBF ? H.sbf : t.second == T_SDV ? H.sdv : t.second == T_BF1R ? H.bf1r : H.bf2r;
      const int lo = ghost ? 0 : 1;
      if (need((long)O * (N - lo + 1))) return UMWM_ERR_ARG;
      for (int i = lo; i <= N; ++i)
        for (int o = 1; o <= O; ++o) out[(size_t)(i - lo) * O + (o - 1)] = src[H.oi(o, i)];
      return UMWM_OK;
    }
  if (!M->on_device) return fail(UMWM_ERR_STATE, "get_field: " + s + " needs the device model");
  const Ptrs& P = M->P;
  CU(cudaStreamSynchronize(M->st));
  static const char* wetnames[] = {"ustar", "cd", "taux", "tauy", "taux_form", "tauy_form", "taux_skin",
                                   "tauy_skin", "taux_diag", "tauy_diag", "tailatmx", "tailatmy", "shelt",
                                   "fcutoff", "physics_time_step", "ds", "ht", "mwp", "mwd", "mss", "mwl", "dwd",
                                   "dwl", "dwp", "dcp0", "dcp", "dcg0", "dcg", "momx", "momy", "cgmxx", "cgmxy",
                                   "cgmyy"};
  float* const wetptrs[] = {P.ustar, P.cd, P.taux, P.tauy, P.taux_form, P.tauy_form, P.taux_skin, P.tauy_skin,
                            P.taux_diag, P.tauy_diag, P.tailatmx, P.tailatmy, P.shelt, P.fcutoff, P.phys, P.ds,
                            P.ht, P.mwp, P.mwd, P.mss, P.mwl, P.dwd, P.dwl, P.dwp, P.dcp0, P.dcp, P.dcg0, P.dcg,
                            P.momx, P.momy, P.cgmxx, P.cgmxy, P.cgmyy};
  for (size_t q = 0; q < sizeof(wetnames) / sizeof(wetnames[0]); ++q)
    if (s == wetnames[q]) {
      if (need(N)) return UMWM_ERR_ARG;
      CU(cudaMemcpy(out, wetptrs[q] + mh.off, (size_t)N * 4, cudaMemcpyDeviceToHost));
      return UMWM_OK;
    }
  static const char* ocnnames[OCN_COUNT] = {"taux_ocntop", "tauy_ocntop", "taux_ocnbot", "tauy_ocnbot", "taux_snl",
                                            "tauy_snl", "epsx_ocn", "epsy_ocn", "epsx_atm", "epsy_atm", "tailocnx",
                                            "tailocny", "taux1", "tauy1", "taux2", "tauy2", "taux3", "tauy3"};
  for (int q = 0; q < OCN_COUNT; ++q)
    if (s == ocnnames[q]) {
      if (!P.ocn) return fail(UMWM_ERR_STATE, "get_field: " + s + " needs stress('ocn') (option stress_ocn or outgrid)");
      if (need(N)) return UMWM_ERR_ARG;
      CU(cudaMemcpy(out, P.ocn + (size_t)q * M->prm.ldN + mh.off, (size_t)N * 4, cudaMemcpyDeviceToHost));
      return UMWM_OK;
    }
  static const char* allnames[] = {"wspd", "wdir", "uc", "vc", "rhoa", "rhow", "rhorat", "fice"};
  float* const allptrs[] = {P.wspd, P.wdir, P.uc, P.vc, P.rhoa, P.rhow, P.rhorat, P.fice};
  for (size_t q = 0; q < 8; ++q)
    if (s == allnames[q]) {
      if (need(NM)) return UMWM_ERR_ARG;
      CU(cudaMemcpy(out, allptrs[q] + mh.nmoff, (size_t)NM * 4, cudaMemcpyDeviceToHost));
      return UMWM_OK;
    }
  if (s == "us" || s == "vs") {
    if (need((long)H.lm * N)) return UMWM_ERR_ARG;
    const float* src = s == "us" ? P.us : P.vs;
    for (int l = 0; l < H.lm; ++l)
      CU(cudaMemcpy(out + (size_t)l * N, src + (size_t)l * M->prm.ldN + mh.off, (size_t)N * 4,
                    cudaMemcpyDeviceToHost));
    return UMWM_OK;
  }
  Ctl c;
  CU(cudaMemcpy(&c, mh.ctl, sizeof c, cudaMemcpyDeviceToHost));
  if (s == "dts") return scalar(c.dts);
  if (s == "dta") return scalar(c.dta);
  if (s == "dtr") return scalar(c.dtr);
  if (s == "dtr_temp") return scalar(c.dtr_temp);
  if (s == "sumt") return scalar(c.sumt);
  return fail(UMWM_ERR_ARG, "get_field: unknown field " + s);
}

int umwm_gpu_get_field_i(const char* name, int* out, long n) {
  Model* M = need_model(false);
  if (!M) return UMWM_ERR_STATE;
  if (!name || !out) return fail(UMWM_ERR_ARG, "get_field_i: null argument");
  const MemberHost& mh = M->mem[M->sel];
  const HostModel& H = mh.H;
  const std::string s(name);
  auto vec = [&](const std::vector<int>& v, int lo, int hi) {
    if (n < hi - lo + 1) return fail(UMWM_ERR_ARG, "get_field_i: buffer too small for " + s);
    for (int i = lo; i <= hi; ++i) out[i - lo] = v[i];
    return UMWM_OK;
  };
  if (s == "mask" || s == "ii") {
    const std::vector<int>& v = s == "mask" ? H.mask : H.ii;
    if (n < (long)v.size()) return fail(UMWM_ERR_ARG, "get_field_i: buffer too small");
    std::copy(v.begin(), v.end(), out);
    return UMWM_OK;
  }
  if (s == "mi") return vec(H.mi, 1, H.imm);
  if (s == "ni") return vec(H.ni, 1, H.imm);
  if (s == "iw") return vec(H.iw, 1, H.imm);
  if (s == "ie") return vec(H.ie, 1, H.imm);
  if (s == "is") return vec(H.is, 1, H.imm);
  if (s == "in") return vec(H.in, 1, H.imm);
  if (s == "iiw") return vec(H.iiw, 1, H.imm);
  if (s == "iie") return vec(H.iie, 1, H.imm);
  if (s == "iis") return vec(H.iis, 1, H.imm);
  if (s == "iin") return vec(H.iin, 1, H.imm);
  if (s == "im" || s == "imm" || s == "iip" || s == "members") {
    if (n < 1) return fail(UMWM_ERR_ARG, "get_field_i: buffer too small");
    out[0] = s == "im" ? H.im : s == "imm" ? H.imm : s == "iip" ? H.iip : (int)M->mem.size();
    return UMWM_OK;
  }
  if (s == "oc") {
    if (!M->on_device) return fail(UMWM_ERR_STATE, "get_field_i: oc needs the device model");
    if (n < H.im) return fail(UMWM_ERR_ARG, "get_field_i: buffer too small");
    CU(cudaMemcpy(out, M->P.oc + mh.off, (size_t)H.im * 4, cudaMemcpyDeviceToHost));
    return UMWM_OK;
  }
  if (s == "substeps") {
    if (!M->on_device || n < 1) return fail(UMWM_ERR_STATE, "get_field_i: substeps needs the device model");
    Ctl c;
    CU(cudaMemcpy(&c, mh.ctl, sizeof c, cudaMemcpyDeviceToHost));
    out[0] = c.substep;
    return UMWM_OK;
  }
  return fail(UMWM_ERR_ARG, "get_field_i: unknown field " + s);
}

int umwm_gpu_get_screen(double* out, long n, long* rows) {
  Model* M = need_model(true);
  if (!M) return UMWM_ERR_STATE;
  const MemberHost& mh = M->mem[M->sel];
  int cnt = 0;
  CU(cudaMemcpy(&cnt, &mh.ctl->log_count, 4, cudaMemcpyDeviceToHost));
  if (rows) *rows = cnt;
  if (out && n > 0) {
    long k = std::min<long>(n / 8, cnt);
    CU(cudaMemcpy(out, mh.log, (size_t)k * 8 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return UMWM_OK;
}

int umwm_gpu_set_option(const char* name, double value) {
  if (!name) return fail(UMWM_ERR_ARG, "set_option: null name");
  std::string s(name);
  if (s == "device") { g_device = (int)value; return UMWM_OK; }
  if (s.compare(0, 9, "surrogate") == 0) return sur::set_option(s, value);
  Model* M = g_model.get();
  if (!M) return fail(UMWM_ERR_STATE, "set_option: initialize first");
  if (s == "kernel_timing") {
    M->ktime = value != 0;
    for (int k = 0; k < K_NK; ++k) { M->kms[k] = 0; M->kcnt[k] = 0; }
    return UMWM_OK;
  }
  if (s == "verbose") { M->verbose = value != 0; return UMWM_OK; }
  if (s == "max_substeps") { M->max_substeps = (long long)value; return UMWM_OK; }
  if (s == "check_finite") { M->check_finite = value != 0; return UMWM_OK; }
  if (s == "gust_seed") {
    if (value < 0 || value > 4294967295.0 || value != std::floor(value))
      return fail(UMWM_ERR_ARG, "gust_seed must be an integer in [0, 2^32)");
    M->gust_seed = (unsigned)value;
    M->prm.gust_seed = M->gust_seed;
    // the captured inner loop holds the old parameters
    if (M->graph_exec) { cudaGraphExecDestroy(M->graph_exec); M->graph_exec = nullptr; }
    if (M->graph) { cudaGraphDestroy(M->graph); M->graph = nullptr; }
    return UMWM_OK;
  }
  if (s == "use_graph") { M->use_graph = value != 0; return UMWM_OK; }
  if (s == "persistent") {
    if (value != 0 && !persist_supported(M->prm))
      return fail(UMWM_ERR_UNSUPPORTED, "persistent needs pm = 36 and one direction mapping for all three kernels");
    M->persistent = value != 0;
    return UMWM_OK;
  }
  if (s == "persistent_stall_test") { M->stall_test = value != 0 ? 1 : 0; return UMWM_OK; }
  if (s == "stress_ocn") {
    M->ocn_every = value != 0;
    return M->ocn_every ? ensure_ocn(*M) : UMWM_OK;
  }
  if (s == "direction_groups" || s == "advect_groups" || s == "phys_groups" || s == "integ_groups") {
    if (value != 2 && value != 4) return fail(UMWM_ERR_ARG, s + " must be 2 or 4");
    if (value == 4 && !quarter_groups(M->prm.P))
      return fail(UMWM_ERR_UNSUPPORTED, s + " 4 needs pm % 4 == 0 and pm/4 in {4, 6, 8, 9, 12}");
    const int g4 = value == 4 ? 1 : 0;
    if (s == "direction_groups" || s == "integ_groups") M->prm.groups4 = g4;
    if (s == "direction_groups" || s == "phys_groups") M->prm.groups4_phys = g4;
    if (s == "direction_groups" || s == "advect_groups") M->prm.adv_groups4 = g4;
    drop_graph(*M);
    return UMWM_OK;
  }
  // launch configuration of the spectral kernels (what the autotuner sets):
  // resident CTAs per SM of the register budget (0: the default instance; a
  // budget without an instance also runs the default) and prefetch distance
  {
    int* f = s == "minb_phys" ? &M->prm.minb_phys : s == "minb_integ" ? &M->prm.minb_integ
           : s == "minb_advect" ? &M->prm.minb_adv : s == "pf_phys" ? &M->prm.pf_phys
           : s == "pf_integ" ? &M->prm.pf_integ : s == "pf_advect" ? &M->prm.pf_adv : nullptr;
    if (f) {
      if (value != std::floor(value) || value < 0 || value > 8)
        return fail(UMWM_ERR_ARG, s + " must be an integer in [0, 8]");
      *f = (int)value;
      drop_graph(*M);
      return UMWM_OK;
    }
  }
  if (s == "advect_tma" || s == "phys_tma") {  // own rows staged by bulk copies (two groups, pm 36)
    // advect_tma 1: E* and e rows, 2: E* rows only; phys_tma 1: e rows
    (s == "advect_tma" ? M->prm.adv_tma : M->prm.phys_tma) =
        s == "advect_tma" ? std::max(0, std::min(2, (int)value)) : (value != 0 ? 1 : 0);
    drop_graph(*M);
    return UMWM_OK;
  }
  if (s == "count_cut") {
    if (value != 0 && M->prm.P != 36)
      return fail(UMWM_ERR_UNSUPPORTED, "count_cut needs pm = 36 (the counting kernel instances)");
    M->prm.count_cut = value != 0 ? 1 : 0;
    static const unsigned long long zero = 0;
    CU(cudaMemcpy(&M->d_glob->cut_count, &zero, sizeof zero, cudaMemcpyHostToDevice));
    drop_graph(*M);
    return UMWM_OK;
  }
  if (s == "autotune") {
    if (value != 0 && value != 1 && value != 2) return fail(UMWM_ERR_ARG, "autotune must be 0, 1 or 2");
    tune_start(*M, (int)value);
    return UMWM_OK;
  }
  return fail(UMWM_ERR_ARG, "set_option: unknown option " + s);
}

double umwm_gpu_get_stat(const char* name) {
  if (name && std::strncmp(name, "surrogate", 9) == 0) return sur::get_stat(name);
  Model* M = g_model.get();
  if (!M || !name) return -1.0;
  std::string s(name);
  if (s == "substeps") return (double)M->substeps;
  if (s == "gpu_ms") return M->last_gpu_ms;
  if (s == "bin_updates") return M->last_bins;
  if (s == "launches") return (double)M->launches;
  if (s == "persistent_graph") return (double)M->pgraph_state;  // 1 captured, -1 direct launches, 0 not run
  if (s.compare(0, 17, "persistent_stage:") == 0) {  // ms block 0 spent in stage n of the persistent kernel
    const int n = std::atoi(s.c_str() + 17);
    if (n < 0 || n >= 8) return -1.0;
    unsigned long long v = 0;
    if (cudaMemcpy(&v, &M->d_glob->stage_ns[n], sizeof v, cudaMemcpyDeviceToHost) != cudaSuccess) return -1.0;
    return (double)v * 1e-6;
  }
  if (s == "cut_count") {  // bins the non-negativity cut changed since count_cut was set
    unsigned long long c = 0;
    if (cudaMemcpy(&c, &M->d_glob->cut_count, sizeof c, cudaMemcpyDeviceToHost) != cudaSuccess) return -1.0;
    return (double)c;
  }
  // the tuner's measurements: "tune_n:<kernel>" candidates, "tune_cfg:<kernel>:<i>"
  // candidate i's configuration (encoded as config:*), "tune_ms:<kernel>:<i>"
  // its median time in ms (-1 before it was measured)
  if (s.compare(0, 5, "tune_") == 0) {
    const size_t c1 = s.find(':');
    if (c1 == std::string::npos) return -1.0;
    const size_t c2 = s.find(':', c1 + 1);
    const std::string what = s.substr(0, c1), kn = s.substr(c1 + 1, c2 == std::string::npos ? std::string::npos : c2 - c1 - 1);
    const int k = kn == "phys" ? TK_PHYS : kn == "integ" ? TK_INTEG : kn == "advect" ? TK_ADVECT : -1;
    if (k < 0) return -1.0;
    const KernelTune& K = M->tune.k[k];
    if (what == "tune_n") return (double)K.cands.size();
    const int i = c2 == std::string::npos ? -1 : std::atoi(s.c_str() + c2 + 1);
    if (i < 0 || i >= (int)K.cands.size()) return -1.0;
    if (what == "tune_cfg")
      return K.cands[i].tma * 1000.0 + (K.cands[i].g4 ? 4 : 2) * 100.0 + K.cands[i].minb * 10.0 + K.cands[i].pf;
    if (what == "tune_ms") {
      std::vector<float> v = K.ms[i];
      if (v.empty()) return -1.0;
      std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
      return v[v.size() / 2];
    }
    return -1.0;
  }
  if (s == "autotune_active") return M->tune.active ? 1.0 : 0.0;
  if (s == "autotune_done") return M->tune.done ? 1.0 : 0.0;
  if (s == "autotune_substeps") return (double)M->tune.step;
  // launch configuration in use, encoded as direction groups (2 or 4) * 100
  // + CTAs per SM * 10 + prefetch levels (CTAs 0: the default instance)
  if (s == "config:phys" || s == "config:integ" || s == "config:advect") {
    const int k = s == "config:phys" ? TK_PHYS : s == "config:integ" ? TK_INTEG : TK_ADVECT;
    const TuneCand c = tune_get(M->prm, k);
    return c.tma * 1000.0 + (c.g4 ? 4 : 2) * 100.0 + c.minb * 10.0 + c.pf;
  }
  if (s == "device_free_bytes") {  // cudaMemGetInfo of the current device
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return -1.0;
    return (double)fr;
  }
  for (int k = 0; k < K_NK; ++k) {
    if (s == std::string("ms:") + KNAMES[k]) return M->kms[k];
    if (s == std::string("count:") + KNAMES[k]) return (double)M->kcnt[k];
  }
  return -1.0;
}

const char* umwm_gpu_last_error(void) { return g_err.c_str(); }

}  // extern "C"
