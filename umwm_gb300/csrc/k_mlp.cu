// Tensor-core GEMM (tcgen05, TMA, TMEM) of the source-term surrogate and its
// host launcher.  See tc_gemm.cuh for the pipeline.
#include <cudaTypedefs.h>

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

template <int EPI>
__global__ void __launch_bounds__(THREADS, 2)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int M, int N, int K,
           EpiArgs ep, int* err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accum_bar;
  __shared__ uint32_t tmem_slot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
  const int KB = K / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&accum_bar), 1);
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
      // producer: TMA loads of A and B k-blocks into the stage ring
      int issued = 0;
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (kb >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1)) {
          ok = false;
          break;
        }
        const uint32_t a = base + s * STAGE_BYTES, b = a + A_TILE_BYTES;
        mbar_expect_tx(smem_u32(&full_bar[s]), STAGE_BYTES);
        tma_load_2d(a, &ta, kb * BK, m0, smem_u32(&full_bar[s]));
        tma_load_2d(b, &tb, kb * BK, n0, smem_u32(&full_bar[s]));
        issued = kb + 1;
      }
      // drain: the last load of each stage has landed (bounded)
      for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; ++kb)
        if (!mbar_wait(smem_u32(&full_bar[kb % STAGES]), (kb / STAGES) & 1)) ok = false;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: 4 x (M=128, N=128, K=16) per k-block, accumulate in TMEM
      const uint32_t idesc = idesc_bf16(BM, BN);
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % STAGES;
        if (!mbar_wait(smem_u32(&full_bar[s]), (kb / STAGES) & 1)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a = base + s * STAGE_BYTES, b = a + A_TILE_BYTES;
#pragma unroll
        for (int k = 0; k < BK / 16; ++k)
          umma_bf16(tmem, sw128_desc(a + k * 32), sw128_desc(b + k * 32), idesc, (kb | k) ? 1u : 0u);
        umma_commit(smem_u32(&empty_bar[s]));
      }
      umma_commit(smem_u32(&accum_bar));  // arrives once every issued MMA has completed
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31, one C row per thread
    ok = mbar_wait(smem_u32(&accum_bar), 0);
    ok = __all_sync(0xffffffffu, ok);
    tc_fence_after();
    if (ok) {
      const int q = warp & 3;
      const int row = m0 + q * 32 + lane;
      for (int c = 0; c < BN; c += 32) {
        float v[32];
        tmem_ld32(tmem + (static_cast<uint32_t>(q * 32) << 16) + c, v);
        if (row < M && n0 + c < N) epilogue<EPI>(ep, row, n0 + c, v);
      }
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

template <int EPI>
cudaError_t launch(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, const EpiArgs& ep, int* err,
                   cudaStream_t st) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_gemm<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  });
  if (attr != cudaSuccess) return attr;
  CUtensorMap ta, tb;
  cudaError_t e = make_map(&ta, A, M, K, BM);
  if (e == cudaSuccess) e = make_map(&tb, B, N, K, BN);
  if (e != cudaSuccess) return e;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  k_gemm<EPI><<<grid, THREADS, SMEM_BYTES, st>>>(ta, tb, M, N, K, ep, err);
  return cudaGetLastError();
}

}  // namespace

}  // namespace tc

cudaError_t gemm_bf16(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, int epi,
                      const tc::EpiArgs& ep, int* err, cudaStream_t st) {
  using namespace tc;
  if (M <= 0 || N <= 0 || K <= 0 || K % BK || N % 32 || ep.ldo % 8 || (ep.ldz && ep.ldz % 8) ||
      (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15) || M > 65535 * BM)
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
