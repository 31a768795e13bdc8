// common.cuh -- shared definitions for the GB300 batched LU kernels.
//
// Arithmetic contract shared by every kernel in this library: each update of
// a matrix or right-hand-side element is one fused multiply-add
// a = fma(-l, u, a), applied in increasing elimination order with a single
// accumulator per element, the column below a pivot is scaled by the
// reciprocal of the pivot (or divided by it when |pivot| < sfmin, as LAPACK
// dgetf2 does), and the U solve multiplies by the same reciprocal.  Any
// schedule that honours this contract returns bit-identical factors, pivots
// and solutions, which is what the parity tests check.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include "../../include/magma_lu.h"

struct magma_queue {
    int device;
    cudaStream_t stream;
    bool own_stream;
    // Queue-owned device workspace, grown on demand by routines that need
    // scratch space (never by the factor/solve routines themselves).
    void *work;
    size_t work_bytes;
};

namespace mlu {

constexpr unsigned FULL = 0xffffffffu;

// ---------------------------------------------------------------------------
// Precision traits.
template <typename T> struct Prec;
template <> struct Prec<double> {
    // bit pattern helpers: exponent field non-zero <=> |x| >= DBL_MIN or x is
    // inf/NaN, i.e. the reciprocal of x does not overflow.
    __device__ static inline bool normal_or_special(double x) {
        return (__double2hiint(x) & 0x7ff00000) != 0;
    }
    __device__ static inline bool nonzero(double x) {
        return ((__double_as_longlong(x) << 1) != 0);
    }
    __device__ static inline bool isnan_(double x) {
        return (((unsigned long long)__double_as_longlong(x)) << 1) > (0x7ff0000000000000ull << 1);
    }
    // |x| as a 63-bit unsigned key (monotone in |x| for non-NaN x).
    __device__ static inline unsigned long long absbits(double x) {
        return ((unsigned long long)__double_as_longlong(x)) & 0x7fffffffffffffffull;
    }
    __device__ static inline double fma_(double a, double b, double c) { return fma(a, b, c); }
};
template <> struct Prec<float> {
    __device__ static inline bool normal_or_special(float x) {
        return (__float_as_uint(x) & 0x7f800000u) != 0;
    }
    __device__ static inline bool nonzero(float x) { return (__float_as_uint(x) << 1) != 0; }
    __device__ static inline bool isnan_(float x) {
        return (__float_as_uint(x) << 1) > (0x7f800000u << 1);
    }
    __device__ static inline unsigned long long absbits(float x) {
        return (unsigned long long)(__float_as_uint(x) & 0x7fffffffu);
    }
    __device__ static inline float fma_(float a, float b, float c) { return fmaf(a, b, c); }
};

// x scaled by the reciprocal r of d, or divided by d when d is subnormal
// (LAPACK dgetf2's sfmin rule).
template <typename T>
__device__ __forceinline__ T rscale(T x, T d, T r) {
    return Prec<T>::normal_or_special(d) ? x * r : x / d;
}

// ---------------------------------------------------------------------------
// Warp arg-max of a 64-bit key with ties resolved to the smallest `pos`.
// Returns the winning pos (all lanes agree).  Uses redux.sync on 32-bit
// halves so that the search never touches the floating-point pipes.
__device__ __forceinline__ unsigned warp_argmax_key(unsigned long long key, unsigned pos) {
    unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    unsigned mhi = __reduce_max_sync(FULL, hi);
    unsigned mlo = __reduce_max_sync(FULL, hi == mhi ? lo : 0u);
    bool cand = (hi == mhi) && (lo == mlo);
    return __reduce_min_sync(FULL, cand ? pos : 0xffffffffu);
}

template <typename T>
__device__ __forceinline__ T shfl(T v, int src) { return __shfl_sync(FULL, v, src); }

// ---------------------------------------------------------------------------
// Bounds-check build (-DMLU_BOUNDS_CHECK, the library's stand-in for a memory
// sanitizer): MLU_BC2(r, c, m, n, site) is true when element (r, c) lies inside
// the logical m x n operand; otherwise it records the first violation (site,
// r, c) in a device word, counts it, and is false, so that the caller skips the
// access.  In the normal build it is the constant true and costs nothing.
#ifdef MLU_BOUNDS_CHECK
__device__ void bc_fail(int site, long long r, long long c);
#define MLU_BC2(r, c, m, n, site)                                                         \
    (((unsigned long long)(long long)(r) < (unsigned long long)(long long)(m) &&         \
      (unsigned long long)(long long)(c) < (unsigned long long)(long long)(n))            \
         ? true                                                                           \
         : (mlu::bc_fail((site), (long long)(r), (long long)(c)), false))
#else
#define MLU_BC2(r, c, m, n, site) true
#endif

// cp.async of one element (4 or 8 bytes) to shared memory; `valid` false
// writes zeros and reads nothing (src must still be a valid address).
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void *dst, const void *src, bool valid)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(src), "n"(BYTES),
                 "r"(valid ? BYTES : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

}  // namespace mlu

#define MLU_CHECK_LAUNCH()                                                              \
    do {                                                                                \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess) {                                                        \
            fprintf(stderr, "magma_lu: launch failed in %s: %s\n", __func__,            \
                    cudaGetErrorString(e_));                                            \
            return MAGMA_ERR_UNKNOWN;                                                   \
        }                                                                               \
    } while (0)

// Lets `kernel` use as much dynamic shared memory as the device allows next to
// its static shared memory.  Returns that amount in bytes.  Any error of the
// attribute calls is consumed here so that it cannot surface as a launch error.
template <typename K>
static inline size_t mlu_allow_dynamic_smem(K kernel)
{
    cudaFuncAttributes fa;
    int dev = 0, optin = 0;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return 48 * 1024;
    }
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) {
        cudaGetLastError();
        return 48 * 1024 - fa.sharedSizeBytes;
    }
    return (size_t)dyn;
}

// Per-device cache of a value computed once per device by f(), such as the
// dynamic shared memory a kernel may use after cudaFuncSetAttribute (which
// applies to the current device only).  `cache` has MLU_MAX_DEVICES entries, all
// zero at first; f() must return a non-zero value.  Two threads that race on
// the first call both run f(), which is harmless for the attribute calls.
constexpr int MLU_MAX_DEVICES = 64;
template <typename F>
static inline size_t mlu_device_cached(size_t *cache, F f)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MLU_MAX_DEVICES) {
        cudaGetLastError();
        return f();
    }
    size_t v = __atomic_load_n(&cache[dev], __ATOMIC_ACQUIRE);
    if (v == 0) {
        v = f();
        __atomic_store_n(&cache[dev], v, __ATOMIC_RELEASE);
    }
    return v;
}

namespace mlu {
// Tuning of the fixed-size factorisation (tuning.cu): per precision and size bin
// of max(m, n) (<= 64, 128, 256, 512, 1024, larger).
constexpr int FIXED_TUNE_BINS = 6;
struct FixedTune {
    unsigned char two_level[FIXED_TUNE_BINS];   // FP32: 128-column blocks (lu_outer.cu)
    unsigned char band_ctas[FIXED_TUNE_BINS];   // FP32: fused band kernel from this many CTAs per SM
    unsigned char tile64[FIXED_TUNE_BINS];      // FP64: 64 x 64 update tiles (else 32 x 32)
};
struct FixedChoice {
    bool two_level;
    int band_ctas;
    bool tile64;
};
FixedChoice fixed_choice(bool fp64, int m, int n);
int fixed_tune_bin(int m, int n);
// loads the tuning file named by MAGMA_LU_TUNING_FILE, once per process
void tuning_load_env_once();

// Every device allocation the library makes for itself (queue workspaces, the
// autotuner's trial batches) goes through this wrapper, so that a test can make
// the next allocations fail (magma_lu_fail_allocations) and check the
// MAGMA_ERR_DEVICE_ALLOC path without exhausting a shared GPU.
cudaError_t device_malloc(void **ptr, size_t bytes);
}  // namespace mlu

static inline magma_int_t mlu_max(magma_int_t a, magma_int_t b) { return a > b ? a : b; }
static inline magma_int_t mlu_min(magma_int_t a, magma_int_t b) { return a < b ? a : b; }
static inline magma_int_t mlu_ceildiv(magma_int_t a, magma_int_t b) { return (a + b - 1) / b; }

// Batches are launched in chunks of at most this many matrices per grid
// dimension (gridDim.y/z limit), like MAGMA's max_batchCount.
constexpr magma_int_t MLU_MAX_GRID_Y = 65535;
