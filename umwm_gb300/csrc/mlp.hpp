// Launchers of the source-term surrogate: the tensor-core GEMM and the
// feature / apply / training kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "tc_gemm.cuh"

namespace umwm {

// C = A * B^T with the given epilogue (tc::Epi).  A: M x K, B: N x K, bf16,
// rows dense (leading dimension K).  K % 64 == 0, N % 32 == 0, A and B
// 16-byte aligned.  *err is set (device side) if a bounded wait gave up.
cudaError_t gemm_bf16(const __nv_bfloat16* A, const __nv_bfloat16* B, int M, int N, int K, int epi,
                      const tc::EpiArgs& ep, int* err, cudaStream_t st);

}  // namespace umwm
