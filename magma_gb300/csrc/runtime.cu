// runtime.cu -- the MAGMA runtime subset the batched LU path needs: init,
// queues over CUDA streams, device/pinned allocation, vector copies,
// pointer-array helpers and argument-error reporting.
//
// Follows interface_cuda/interface.cpp (magma_init :164, magma_finalize :237,
// queue creation :931-1034), control/xerbla.cpp:51 and
// magmablas/zset_pointer.cu:20-25 in behaviour; the queue here is a plain
// struct around one cudaStream_t and carries no cuBLAS/cuSPARSE handles.
#include "common.cuh"
#include "trace.cuh"
#include <atomic>
#include <stdlib.h>

namespace {
std::atomic<int> g_fail_allocs{0};   // allocations still to fail (fault injection for tests)
}

cudaError_t mlu::device_malloc(void **ptr, size_t bytes)
{
    int left = g_fail_allocs.load();
    while (left > 0 && !g_fail_allocs.compare_exchange_weak(left, left - 1)) {
    }
    if (left > 0) {
        *ptr = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(ptr, bytes);
}

// Fault injection for tests: the next `count` device allocations the library
// makes for itself fail as if the device were out of memory (the calls that
// make them return MAGMA_ERR_DEVICE_ALLOC, as the reference does when its
// pivot workspace cannot be allocated, src/zgetrf_batched.cpp:137-142).
// count = 0 turns it off.  Returns the number that was still pending.
extern "C" magma_int_t magma_lu_fail_allocations(magma_int_t count)
{
    return g_fail_allocs.exchange(count < 0 ? 0 : count);
}

extern "C" magma_int_t magma_init(void) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return MAGMA_ERR_UNKNOWN;
    return MAGMA_SUCCESS;
}

extern "C" magma_int_t magma_finalize(void) { return MAGMA_SUCCESS; }

extern "C" void magma_xerbla(const char *name, magma_int_t info) {
    if (info < 0)
        fprintf(stderr, "Error in %s, function-specific error (info = %d)\n", name, (int)info);
    else
        fprintf(stderr, "Error in %s, argument %d had an illegal value\n", name, (int)info);
}

extern "C" void magma_queue_create_internal(magma_device_t device, magma_queue_t *queue_ptr,
                                            const char *, const char *, int) {
    mlu::tuning_load_env_once();
    magma_queue_t q = (magma_queue_t)calloc(1, sizeof(struct magma_queue));
    if (!q) { *queue_ptr = nullptr; return; }
    q->device = device;
    cudaSetDevice(device);
    if (cudaStreamCreateWithFlags(&q->stream, cudaStreamNonBlocking) != cudaSuccess) {
        free(q);
        *queue_ptr = nullptr;
        return;
    }
    q->own_stream = true;
    *queue_ptr = q;
}

extern "C" void magma_queue_create_from_cuda_internal(magma_device_t device, void *cuda_stream,
                                                      void *, void *, magma_queue_t *queue_ptr,
                                                      const char *, const char *, int) {
    mlu::tuning_load_env_once();
    magma_queue_t q = (magma_queue_t)calloc(1, sizeof(struct magma_queue));
    if (!q) { *queue_ptr = nullptr; return; }
    q->device = device;
    q->stream = (cudaStream_t)cuda_stream;
    q->own_stream = false;
    *queue_ptr = q;
}

extern "C" void magma_queue_destroy_internal(magma_queue_t queue, const char *, const char *, int) {
    if (!queue) return;
    if (queue->stream) cudaStreamSynchronize(queue->stream);
    if (queue->work) cudaFree(queue->work);
    if (queue->own_stream) cudaStreamDestroy(queue->stream);
    free(queue);
}

extern "C" void magma_queue_sync_internal(magma_queue_t queue, const char *, const char *, int) {
    if (queue) cudaStreamSynchronize(queue->stream);
}

extern "C" magma_int_t magma_queue_get_device(magma_queue_t queue) { return queue->device; }

extern "C" void *magma_queue_get_cuda_stream(magma_queue_t queue) { return (void *)queue->stream; }

extern "C" magma_int_t magma_malloc(magma_ptr *ptr_ptr, size_t bytes) {
    if (bytes == 0) bytes = 16;   // MAGMA allocates a minimal buffer for size 0
    if (cudaMalloc(ptr_ptr, bytes) != cudaSuccess) {
        *ptr_ptr = nullptr;
        return MAGMA_ERR_DEVICE_ALLOC;
    }
    return MAGMA_SUCCESS;
}

extern "C" magma_int_t magma_malloc_pinned(void **ptr_ptr, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (cudaMallocHost(ptr_ptr, bytes) != cudaSuccess) {
        *ptr_ptr = nullptr;
        return MAGMA_ERR_HOST_ALLOC;
    }
    return MAGMA_SUCCESS;
}

extern "C" magma_int_t magma_free_internal(magma_ptr ptr, const char *func, const char *file,
                                           int line) {
    if (cudaFree(ptr) != cudaSuccess) {
        fprintf(stderr, "magma_free: invalid pointer at %s (%s:%d)\n", func, file, line);
        return MAGMA_ERR_INVALID_PTR;
    }
    return MAGMA_SUCCESS;
}

extern "C" magma_int_t magma_free_pinned_internal(void *ptr, const char *func, const char *file,
                                                  int line) {
    if (cudaFreeHost(ptr) != cudaSuccess) {
        fprintf(stderr, "magma_free_pinned: invalid pointer at %s (%s:%d)\n", func, file, line);
        return MAGMA_ERR_INVALID_PTR;
    }
    return MAGMA_SUCCESS;
}

extern "C" void magma_setvector_internal(magma_int_t n, magma_int_t elemSize, const void *hx_src,
                                         magma_int_t incx, magma_ptr dy_dst, magma_int_t incy,
                                         magma_queue_t queue, const char *, const char *, int) {
    if (n <= 0) return;
    cudaMemcpy2DAsync(dy_dst, (size_t)incy * elemSize, hx_src, (size_t)incx * elemSize, elemSize,
                      n, cudaMemcpyHostToDevice, queue->stream);
    cudaStreamSynchronize(queue->stream);
}

extern "C" void magma_getvector_internal(magma_int_t n, magma_int_t elemSize, const void *dx_src,
                                         magma_int_t incx, void *hy_dst, magma_int_t incy,
                                         magma_queue_t queue, const char *, const char *, int) {
    if (n <= 0) return;
    cudaMemcpy2DAsync(hy_dst, (size_t)incy * elemSize, dx_src, (size_t)incx * elemSize, elemSize,
                      n, cudaMemcpyDeviceToHost, queue->stream);
    cudaStreamSynchronize(queue->stream);
}

template <typename T>
__global__ void set_pointer_kernel(T **out, T *in, magma_int_t lda, magma_int_t row,
                                   magma_int_t column, long long batch_offset, int batch) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < batch) out[k] = in + (long long)k * batch_offset + row + (long long)column * lda;
}

template <typename T>
static void set_pointer(T **out, T *in, magma_int_t lda, magma_int_t row, magma_int_t column,
                        magma_int_t batch_offset, magma_int_t batch, magma_queue_t queue) {
    if (batch <= 0) return;
    MLU_LAUNCH(mlu::KC_OTHER, queue->stream, set_pointer_kernel<T><<<mlu_ceildiv(batch, 256), 256, 0, queue->stream>>>(
        out, in, lda, row, column, (long long)batch_offset, batch));
}

extern "C" void magma_dset_pointer(double **output_array, double *input, magma_int_t lda,
                                   magma_int_t row, magma_int_t column, magma_int_t batch_offset,
                                   magma_int_t batchCount, magma_queue_t queue) {
    set_pointer(output_array, input, lda, row, column, batch_offset, batchCount, queue);
}

extern "C" void magma_sset_pointer(float **output_array, float *input, magma_int_t lda,
                                   magma_int_t row, magma_int_t column, magma_int_t batch_offset,
                                   magma_int_t batchCount, magma_queue_t queue) {
    set_pointer(output_array, input, lda, row, column, batch_offset, batchCount, queue);
}

extern "C" void magma_iset_pointer(magma_int_t **output_array, magma_int_t *input,
                                   magma_int_t lda, magma_int_t row, magma_int_t column,
                                   magma_int_t batch_offset, magma_int_t batchCount,
                                   magma_queue_t queue) {
    set_pointer(output_array, input, lda, row, column, batch_offset, batchCount, queue);
}

#ifdef MLU_BOUNDS_CHECK
// The bounds-check build's record: the first violation (site << 48 | row << 24
// | column, each clipped to 24 bits) and the number of violations.
namespace mlu {
__device__ unsigned long long g_bc_first;
__device__ unsigned long long g_bc_count;
__device__ void bc_fail(int site, long long r, long long c)
{
    const unsigned long long rec = ((unsigned long long)(site & 0xffff) << 48) |
                                   (((unsigned long long)r & 0xffffffull) << 24) |
                                   ((unsigned long long)c & 0xffffffull);
    atomicCAS(&g_bc_first, 0ull, rec);
    atomicAdd(&g_bc_count, 1ull);
}
}  // namespace mlu

// Reads the record (first violation, count) and, with reset != 0, clears it.
// Exported by the bounds-check build only.
extern "C" int mlu_bounds_check_read(unsigned long long *first, unsigned long long *count, int reset)
{
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    if (cudaMemcpyFromSymbol(first, mlu::g_bc_first, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemcpyFromSymbol(count, mlu::g_bc_count, sizeof(unsigned long long)) != cudaSuccess)
        return -1;
    if (reset) {
        const unsigned long long z = 0;
        if (cudaMemcpyToSymbol(mlu::g_bc_first, &z, sizeof z) != cudaSuccess ||
            cudaMemcpyToSymbol(mlu::g_bc_count, &z, sizeof z) != cudaSuccess)
            return -1;
    }
    return 0;
}
#endif
