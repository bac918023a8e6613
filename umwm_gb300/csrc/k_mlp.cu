// Tensor-core GEMM (tcgen05, TMA, TMEM) of the source-term surrogate and its
// host launcher.  See tc_gemm.cuh for the pipeline.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "mlp.hpp"
#include "tc_gemm.cuh"

namespace umwm {
namespace tc {

template <int EPI>
__device__ __forceinline__ void epilogue(const EpiArgs& ep, int row, int col, const float* v) {
  if (EPI == EPI_F32 || EPI == EPI_F32_ACC) {
    float* o = static_cast<float*>(ep.out) + (size_t)row * ep.ldo + col;
#pragma unroll
    for (int i = 0; i < 32; i += 4) {
      float4 w = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      if (EPI == EPI_F32 && ep.bias) {
        w.x += ep.bias[col + i];
        w.y += ep.bias[col + i + 1];
        w.z += ep.bias[col + i + 2];
        w.w += ep.bias[col + i + 3];
      }
      if (EPI == EPI_F32_ACC) {
        const float4 p = *reinterpret_cast<const float4*>(o + i);
        w.x += p.x;
        w.y += p.y;
        w.z += p.z;
        w.w += p.w;
      }
      *reinterpret_cast<float4*>(o + i) = w;
    }
  } else {
    __nv_bfloat16* o = static_cast<__nv_bfloat16*>(ep.out) + (size_t)row * ep.ldo + col;
    float z[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) z[i] = v[i] + ((EPI != EPI_BF16_DGELU && ep.bias) ? ep.bias[col + i] : 0.f);
    if (EPI == EPI_BF16_DGELU) {
      const __nv_bfloat16* zi = ep.zin + (size_t)row * ep.ldz + col;
#pragma unroll
      for (int i = 0; i < 32; i += 8) {
        const uint4 raw = *reinterpret_cast<const uint4*>(zi + i);
        const __nv_bfloat16* zz = reinterpret_cast<const __nv_bfloat16*>(&raw);
#pragma unroll
        for (int t = 0; t < 8; ++t) z[i + t] *= gelu_grad(__bfloat162float(zz[t]));
      }
    }
    if (EPI == EPI_BF16_GELU && ep.zout) {
      __nv_bfloat16* zo = ep.zout + (size_t)row * ep.ldz + col;
#pragma unroll
      for (int i = 0; i < 32; i += 8) {
        uint4 raw;
        __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&raw);
#pragma unroll
        for (int t = 0; t < 4; ++t) h[t] = __floats2bfloat162_rn(z[i + 2 * t], z[i + 2 * t + 1]);
        *reinterpret_cast<uint4*>(zo + i) = raw;
      }
    }
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
      uint4 raw;
      __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&raw);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        float a = z[i + 2 * t], b = z[i + 2 * t + 1];
        if (EPI == EPI_BF16_GELU) {
          a = gelu(a);
          b = gelu(b);
        }
        h[t] = __floats2bfloat162_rn(a, b);
      }
      *reinterpret_cast<uint4*>(o + i) = raw;
    }
  }
}

template <int EPI, int BN_>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int M, int N, int K,
           EpiArgs ep, int* err) {
  using C = Cfg<BN_>;
  constexpr int BN = C::BN, STAGES = C::STAGES, STAGE_BYTES = C::STAGE_BYTES, TMEM_COLS = C::TMEM_COLS;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], acc_full[2], acc_empty[2], mma_done;
  __shared__ uint32_t tmem_slot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int KB = K / BK;
  const int ntn = (N + BN - 1) / BN, ntiles = ntn * ((M + BM - 1) / BM);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), 32 * EPI_WARPS);
    }
    mbar_init(smem_u32(&mma_done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(&tmem_slot), TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      // producer: TMA loads of A and B k-blocks into the stage ring, tile after tile
      int it = 0;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int m0 = (t / ntn) * BM, n0 = (t % ntn) * BN;
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int s = it % STAGES;
          if (it >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ((it / STAGES) & 1) ^ 1)) {
            ok = false;
            break;
          }
          const uint32_t a = base + s * STAGE_BYTES, b = a + A_TILE_BYTES;
          mbar_expect_tx(smem_u32(&full_bar[s]), STAGE_BYTES);
          tma_load_2d(a, &ta, kb * BK, m0, smem_u32(&full_bar[s]));
          tma_load_2d(b, &tb, kb * BK, n0, smem_u32(&full_bar[s]));
        }
      }
      // drain: the last load of each stage has landed (bounded)
      for (int i = (it > STAGES ? it - STAGES : 0); i < it; ++i)
        if (!mbar_wait(smem_u32(&full_bar[i % STAGES]), (i / STAGES) & 1)) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: 4 x (M=128, N=BN, K=16) per k-block into accumulator tl & 1
      // (N = the valid columns, a multiple of 32, for the last column tile)
      int it = 0, tl = 0;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tl) {
        const int buf = tl & 1, use = tl >> 1;
        const uint32_t idesc = idesc_bf16(BM, min(BN, N - (t % ntn) * BN));
        // the epilogue has read this accumulator's previous tile
        if (use > 0 && !mbar_wait(smem_u32(&acc_empty[buf]), (use - 1) & 1)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(buf * BN);
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int s = it % STAGES;
          if (!mbar_wait(smem_u32(&full_bar[s]), (it / STAGES) & 1)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a = base + s * STAGE_BYTES, b = a + A_TILE_BYTES;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k)
            umma_bf16(d, sw128_desc(a + k * 32), sw128_desc(b + k * 32), idesc, (kb | k) ? 1u : 0u);
          umma_commit(smem_u32(&empty_bar[s]));
        }
        if (ok) umma_commit(smem_u32(&acc_full[buf]));  // arrives once the tile's MMAs have completed
      }
      // every MMA issued has completed before the TMEM is freed (bounded)
      umma_commit(smem_u32(&mma_done));
      if (!mbar_wait(smem_u32(&mma_done), 0)) ok = false;
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (one C row per
    // thread) and half the accumulator's columns
    const int q = warp & 3, h = (warp - 2) >> 2;
    int tl = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tl) {
      const int buf = tl & 1, use = tl >> 1;
      ok = mbar_wait(smem_u32(&acc_full[buf]), use & 1);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      tc_fence_after();
      const int m0 = (t / ntn) * BM, n0 = (t % ntn) * BN;
      const int row = m0 + q * 32 + lane;
      for (int c = h * (BN / 2); c < (h + 1) * (BN / 2); c += 32) {
        float v[32];
        tmem_ld32(tmem + (static_cast<uint32_t>(q * 32) << 16) + (uint32_t)(buf * BN + c), v);
        if (row < M && n0 + c < N) epilogue<EPI>(ep, row, n0 + c, v);
      }
      tc_fence_before();
      mbar_arrive(smem_u32(&acc_empty[buf]));
    }
  }
  if (!ok) atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---- host side --------------------------------------------------------------

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

cudaError_t get_encoder() {
  static std::once_flag once;
  static cudaError_t status = cudaSuccess;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    status = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (status == cudaSuccess && (q != cudaDriverEntryPointSuccess || !fn)) status = cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  return status;
}

// rows x cols bf16, row-major (cols contiguous), boxes of box_rows x 64.
cudaError_t make_map(CUtensorMap* m, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box_rows) {
  cudaError_t e = get_encoder();
  if (e != cudaSuccess) return e;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(BK), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int EPI, int BN>
cudaError_t launch_bn(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const EpiArgs& ep,
                      int* err, int nsm, cudaStream_t st) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_gemm<EPI, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<BN>::SMEM_BYTES);
  });
  if (attr != cudaSuccess) return attr;
  CUtensorMap ta, tb;
  cudaError_t e = make_map(&ta, A, M, K, BM);
  if (e == cudaSuccess) e = make_map(&tb, B, N, K, BN);
  if (e != cudaSuccess) return e;
  const long tiles = (long)((N + BN - 1) / BN) * ((M + BM - 1) / BM);
  const int grid = (int)std::min<long>(tiles, nsm);  // persistent: one CTA per SM
  k_gemm<EPI, BN><<<grid, THREADS, Cfg<BN>::SMEM_BYTES, st>>>(ta, tb, M, N, K, ep, err);
  return cudaGetLastError();
}

// 256-wide tiles when they fill the SMs, else 128-wide ones
template <int EPI>
cudaError_t launch(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const EpiArgs& ep, int* err,
                   cudaStream_t st) {
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0, n = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    nsm = n;
  }
  const long tiles256 = (long)((N + 255) / 256) * ((M + BM - 1) / BM);
  return tiles256 >= nsm ? launch_bn<EPI, 256>(A, B, M, N, K, ep, err, nsm, st)
                         : launch_bn<EPI, 128>(A, B, M, N, K, ep, err, nsm, st);
}

}  // namespace

}  // namespace tc

cudaError_t gemm_bf16(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, int epi,
                      const tc::EpiArgs& ep, int* err, cudaStream_t st) {
  using namespace tc;
  if (M <= 0 || N <= 0 || K <= 0 || K % BK || N % 32 || ep.ldo % 8 || (ep.ldz && ep.ldz % 8) ||
      (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15))
    return cudaErrorInvalidValue;
  switch (epi) {
    case EPI_F32: return launch<EPI_F32>(A, B, M, N, K, ep, err, st);
    case EPI_BF16: return launch<EPI_BF16>(A, B, M, N, K, ep, err, st);
    case EPI_BF16_GELU: return launch<EPI_BF16_GELU>(A, B, M, N, K, ep, err, st);
    case EPI_BF16_DGELU: return launch<EPI_BF16_DGELU>(A, B, M, N, K, ep, err, st);
    case EPI_F32_ACC: return launch<EPI_F32_ACC>(A, B, M, N, K, ep, err, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace umwm
