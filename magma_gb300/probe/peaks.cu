// peaks.cu -- measured arithmetic peaks used as roofline denominators.
//
// The FP64 factor/solve kernels are bound by the FP64 FMA pipe, whose rate on
// GB300 is a small fraction of the FP32 rate; this probe measures it (and the
// FP32 FMA rate) on the device the benchmark runs on, with the same launch
// conditions as a long kernel: every SM busy, independent FMA chains so that
// latency is hidden.  Not part of the MAGMA ABI; the benchmark loads it.
#include <cuda_runtime.h>

template <typename T>
__global__ void fma_chain_kernel(T *out, int iters, T a, T b) {
    T x0 = threadIdx.x * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == T(12345.678)) out[0] = s;   // keeps the chains live
}

template <typename T>
static double run(int iters, int blocks_per_sm, int threads, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    T *out = nullptr;
    cudaMalloc(&out, sizeof(T));
    dim3 grid(sms * blocks_per_sm);
    fma_chain_kernel<T><<<grid, threads, 0, s>>>(out, iters / 8, T(0.999999), T(1e-7));  // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    fma_chain_kernel<T><<<grid, threads, 0, s>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    double flops = 2.0 * 32.0 * (double)iters * threads * (double)grid.x;
    return flops / (ms * 1e-3) / 1e12;
}

// Returns TFLOP/s of dependent-chain-free FMA throughput over all SMs.
extern "C" double mlu_probe_fp64_tflops(void *stream) {
    return run<double>(2048, 4, 256, (cudaStream_t)stream);
}

extern "C" double mlu_probe_fp32_tflops(void *stream) {
    return run<float>(16384, 4, 256, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Check of the integer-pipe double -> float conversion used by the refinement
// (csrc/convert.cuh) against CUDA's __double2float_rn: random 64-bit patterns
// and doubles built around float rounding boundaries (random low bits, exact
// ties, ties +- 1 ulp of double).  Returns the number of mismatching results
// (NaN matches any NaN).
#include "../csrc/convert.cuh"

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

__global__ void d2f_check_kernel(unsigned long long seed, long long n, unsigned long long *bad)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r = splitmix64(seed ^ (unsigned long long)i);
        unsigned long long bits;
        const int mode = (int)(i & 3);
        if (mode == 0) {
            bits = r;
        } else {
            // a double whose top part is a random float, exponent biased to the
            // float range (including its subnormals), with chosen low bits
            const unsigned long long r2 = splitmix64(r);
            const int e = 1023 - 160 + (int)(r2 % 300);      // 2^-160 .. 2^139
            const unsigned long long top = (r >> 11) & 0xfffffffffffffull;
            unsigned long long low;
            if (mode == 1) low = (r2 >> 20) & ((1ull << 29) - 1);
            else if (mode == 2) low = 1ull << 28;                       // exact tie
            else low = (1ull << 28) + ((r2 & 1) ? 1 : (1ull << 29) - 1) - ((r2 & 1) ? 0 : (1ull << 28));
            bits = ((r >> 63) << 63) | ((unsigned long long)e << 52) | ((top & ~((1ull << 29) - 1)) | low);
        }
        const double x = __longlong_as_double((long long)bits);
        const float a = __double2float_rn(x);
        const float b = mlu::d2f_rn_int(x);
        const bool both_nan = (a != a) && (b != b);
        if (!both_nan && __float_as_uint(a) != __float_as_uint(b)) atomicAdd(bad, 1ull);
    }
}

extern "C" long long mlu_check_d2f(long long n, unsigned long long seed)
{
    unsigned long long *bad = nullptr;
    if (cudaMalloc(&bad, sizeof(unsigned long long)) != cudaSuccess) return -1;
    cudaMemset(bad, 0, sizeof(unsigned long long));
    d2f_check_kernel<<<1024, 256>>>(seed, n, bad);
    unsigned long long h = 0;
    cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    if (cudaGetLastError() != cudaSuccess) return -1;
    return (long long)h;
}
