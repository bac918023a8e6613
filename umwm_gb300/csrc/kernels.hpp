// Launchers of the GB300 UMWM kernels (all on one stream).
#pragma once
#include <cuda_runtime.h>

#include "dev.cuh"

namespace umwm {

bool supported_pm(int pm);
cudaError_t launch_prep(const Params& prm, const Ptrs& P, int compute_rot, int max_nm, cudaStream_t st);
cudaError_t launch_sice(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_source_phys(const Params& prm, const Ptrs& P, int compute_rot, cudaStream_t st);
cudaError_t launch_dts(const Params& prm, const Ptrs& P, int compute_rot, int first, cudaStream_t st);
cudaError_t launch_source_integ(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_advect(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_diag(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_stokes(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_screen(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_to_ref(const Params& prm, const float* E, float* F, int off, int n, cudaStream_t st);
cudaError_t launch_from_ref(const Params& prm, const float* F, float* E, int off, int n, cudaStream_t st);
cudaError_t launch_begin_dtg(const Params& prm, cudaStream_t st);
cudaError_t launch_stress_ocn(const Params& prm, const Ptrs& P, cudaStream_t st);
cudaError_t launch_loop_arm(Global* g, int budget, cudaStream_t st);
cudaError_t launch_loop_cond(Global* g, cudaGraphConditionalHandle h, cudaStream_t st);
cudaError_t launch_count_nonfinite(const float* a, size_t n, int* count, cudaStream_t st);
cudaError_t launch_fill(float* a, size_t n, float v, cudaStream_t st);
// persistent substep kernel (k_persist.cu): up to Global::budget substeps
// (armed by launch_loop_arm) of every member in one cooperative launch;
// Global::iters counts them, bar_err marks a barrier wait that ran out
// (stall_test: one CTA more is expected than launched, so every wait runs
// out after 20 ms)
bool persist_supported(const Params& prm);
cudaError_t launch_persist(const Params& prm, const Ptrs& P, int stall_test, cudaStream_t st);

}  // namespace umwm
