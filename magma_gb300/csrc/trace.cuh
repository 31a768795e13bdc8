// trace.cuh -- launch accounting and opt-in per-kernel timing.
//
// Every kernel launch of the library goes through MLU_LAUNCH, which counts it
// and, while timing is enabled for the launch's kernel class, brackets it with
// CUDA events recorded on the launching stream (never while that stream is
// being captured into a graph).  Host-side only; the cost when timing is off
// is one relaxed atomic increment per launch.
#pragma once
#include <cuda_runtime.h>

namespace mlu {

// Kernel classes (values are part of the C ABI: magma_lu_timing_start).
enum KernelClass {
    KC_OTHER = 0,
    KC_SMALL_GESV = 1,    // fused n <= 32 factor+solve (lu_small.cu)
    KC_PANEL = 2,         // panel factorisation of the blocked LU
    KC_SWAP_TRSM = 3,     // row interchanges + L11^{-1} A12 of the blocked LU
    KC_GEMM = 4,          // SIMT trailing update of the blocked LU
    KC_TC_UPDATE = 5,     // tensor-core trailing update (lu_tc.cu)
    KC_GETRS = 6,         // triangular solves (blocked and small getrs)
    KC_IR_RESIDUAL = 7,   // FP64 residual of the refinement
    KC_IR_SOLVE = 8,      // low-precision correction solve + FP64 update
    KC_IR_INIT = 9,       // FP64 -> low-precision conversion, norms
    KC_VB_LU = 10,        // persistent variable-size factor+solve
    KC_ADJ_GER = 11,      // adjoint outer product
    KC_OUTER = 12,        // rank-128 update right of a block of the FP32 LU (lu_outer.cu)
    KC_COUNT = 13
};

void trace_before(int cls, cudaStream_t s);
void trace_after(int cls, cudaStream_t s);

}  // namespace mlu

// MLU_LAUNCH(class, stream, kernel<<<grid, block, smem, stream>>>(args...))
#define MLU_LAUNCH(cls, stream, ...)            \
    do {                                        \
        mlu::trace_before((cls), (stream));     \
        __VA_ARGS__;                            \
        mlu::trace_after((cls), (stream));      \
    } while (0)
