// strided.cu -- strided-batch entry points for the batched LU: one base
// pointer and a stride per operand instead of arrays of device pointers.
//
// MAGMA offers this calling form for its banded and SVD routines
// (magma_zgbtrf_batched_strided, include/magma_zbatched.h:613;
// magmablas_zgemm_batched_strided, :135) but not for getrf/getrs/gesv.  The
// entry points below follow the same convention: matrix k of the batch is at
// dA + k * strideA, its pivots at dipiv + k * strideP.  They build the pointer
// arrays on the device (one small kernel, queue-owned scratch grown on demand,
// as MAGMA's own strided routines do) and call the pointer-array routines, so
// results are identical to those.
#include "common.cuh"
#include "trace.cuh"

extern "C" {
magma_int_t magma_dgetrf_batched(magma_int_t, magma_int_t, double **, magma_int_t, magma_int_t **,
                                 magma_int_t *, magma_int_t, magma_queue_t);
magma_int_t magma_sgetrf_batched(magma_int_t, magma_int_t, float **, magma_int_t, magma_int_t **,
                                 magma_int_t *, magma_int_t, magma_queue_t);
magma_int_t magma_dgetrs_batched(magma_trans_t, magma_int_t, magma_int_t, double **, magma_int_t,
                                 magma_int_t **, double **, magma_int_t, magma_int_t,
                                 magma_queue_t);
magma_int_t magma_sgetrs_batched(magma_trans_t, magma_int_t, magma_int_t, float **, magma_int_t,
                                 magma_int_t **, float **, magma_int_t, magma_int_t, magma_queue_t);
magma_int_t magma_dgesv_batched(magma_int_t, magma_int_t, double **, magma_int_t, magma_int_t **,
                                double **, magma_int_t, magma_int_t *, magma_int_t, magma_queue_t);
magma_int_t magma_sgesv_batched(magma_int_t, magma_int_t, float **, magma_int_t, magma_int_t **,
                                float **, magma_int_t, magma_int_t *, magma_int_t, magma_queue_t);
}

namespace mlu {

// ptrs[k] = base + k * stride for up to three operands (null bases skipped)
__global__ void strided_pointers_kernel(int batch, char *a, size_t sa, char **pa, char *b,
                                        size_t sb, char **pb, char *c, size_t sc, char **pc)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= batch) return;
    if (a) pa[k] = a + (size_t)k * sa;
    if (b) pb[k] = b + (size_t)k * sb;
    if (c) pc[k] = c + (size_t)k * sc;
}

// Three pointer arrays of `batch` entries in the queue's scratch (grown, after
// a synchronisation, when too small).
static void **strided_scratch(magma_queue_t q, int batch)
{
    const size_t need = 3 * (((size_t)batch * sizeof(void *) + 255) & ~(size_t)255) + 256;
    if (q->work_bytes < need) {
        if (q->work) { cudaStreamSynchronize(q->stream); cudaFree(q->work); }
        q->work = nullptr;
        q->work_bytes = 0;
        if (mlu::device_malloc(&q->work, need) != cudaSuccess) return nullptr;
        q->work_bytes = need;
    }
    return (void **)q->work;
}

struct StridedPtrs {
    void **a, **b, **c;
};

static magma_int_t make_pointers(magma_queue_t q, int batch, void *a, size_t sa, void *b,
                                 size_t sb, void *c, size_t sc, StridedPtrs &out)
{
    void **base = strided_scratch(q, batch);
    if (!base) return MAGMA_ERR_DEVICE_ALLOC;
    const size_t slot = (((size_t)batch * sizeof(void *) + 255) & ~(size_t)255) / sizeof(void *);
    out = {base, base + slot, base + 2 * slot};
    MLU_LAUNCH(mlu::KC_OTHER, q->stream,
               strided_pointers_kernel<<<mlu_ceildiv(batch, 256), 256, 0, q->stream>>>(
                   batch, (char *)a, sa, (char **)out.a, (char *)b, sb, (char **)out.b, (char *)c,
                   sc, (char **)out.c));
    MLU_CHECK_LAUNCH();
    return 0;
}

}  // namespace mlu

using namespace mlu;

#define MLU_STRIDED_GETRF(P, T)                                                                 \
    extern "C" magma_int_t magma_##P##getrf_batched_strided(                                    \
        magma_int_t m, magma_int_t n, T *dA, magma_int_t ldda, magma_int_t strideA,             \
        magma_int_t *dipiv, magma_int_t strideP, magma_int_t *info_array,                       \
        magma_int_t batchCount, magma_queue_t queue)                                            \
    {                                                                                           \
        if (batchCount <= 0 || m <= 0 || n <= 0)                                                \
            return magma_##P##getrf_batched(m, n, nullptr, ldda, nullptr, info_array,           \
                                            batchCount, queue);                                 \
        if (strideA < ldda * n) return -5;                                                      \
        if (strideP < mlu_min(m, n)) return -7;                                                 \
        StridedPtrs p;                                                                          \
        magma_int_t rc = make_pointers(queue, batchCount, dA, (size_t)strideA * sizeof(T),      \
                                       dipiv, (size_t)strideP * sizeof(int), nullptr, 0, p);    \
        if (rc != 0) return rc;                                                                 \
        return magma_##P##getrf_batched(m, n, (T **)p.a, ldda, (magma_int_t **)p.b,             \
                                        info_array, batchCount, queue);                         \
    }

#define MLU_STRIDED_GETRS(P, T)                                                                 \
    extern "C" magma_int_t magma_##P##getrs_batched_strided(                                    \
        magma_trans_t trans, magma_int_t n, magma_int_t nrhs, T *dA, magma_int_t ldda,          \
        magma_int_t strideA, magma_int_t *dipiv, magma_int_t strideP, T *dB, magma_int_t lddb,  \
        magma_int_t strideB, magma_int_t batchCount, magma_queue_t queue)                       \
    {                                                                                           \
        if (batchCount <= 0 || n <= 0 || nrhs <= 0)                                             \
            return magma_##P##getrs_batched(trans, n, nrhs, nullptr, ldda, nullptr, nullptr,    \
                                            lddb, batchCount, queue);                           \
        if (strideA < ldda * n) return -6;                                                      \
        if (strideP < n) return -8;                                                             \
        if (strideB < lddb * nrhs) return -11;                                                  \
        StridedPtrs p;                                                                          \
        magma_int_t rc = make_pointers(queue, batchCount, dA, (size_t)strideA * sizeof(T),      \
                                       dipiv, (size_t)strideP * sizeof(int), dB,                \
                                       (size_t)strideB * sizeof(T), p);                         \
        if (rc != 0) return rc;                                                                 \
        return magma_##P##getrs_batched(trans, n, nrhs, (T **)p.a, ldda, (magma_int_t **)p.b,   \
                                        (T **)p.c, lddb, batchCount, queue);                    \
    }

#define MLU_STRIDED_GESV(P, T)                                                                  \
    extern "C" magma_int_t magma_##P##gesv_batched_strided(                                     \
        magma_int_t n, magma_int_t nrhs, T *dA, magma_int_t ldda, magma_int_t strideA,          \
        magma_int_t *dipiv, magma_int_t strideP, T *dB, magma_int_t lddb, magma_int_t strideB,  \
        magma_int_t *dinfo_array, magma_int_t batchCount, magma_queue_t queue)                  \
    {                                                                                           \
        if (batchCount <= 0 || n <= 0 || nrhs <= 0)                                             \
            return magma_##P##gesv_batched(n, nrhs, nullptr, ldda, nullptr, nullptr, lddb,      \
                                           dinfo_array, batchCount, queue);                     \
        if (strideA < ldda * n) return -5;                                                      \
        if (strideP < n) return -7;                                                             \
        if (strideB < lddb * nrhs) return -10;                                                  \
        StridedPtrs p;                                                                          \
        magma_int_t rc = make_pointers(queue, batchCount, dA, (size_t)strideA * sizeof(T),      \
                                       dipiv, (size_t)strideP * sizeof(int), dB,                \
                                       (size_t)strideB * sizeof(T), p);                         \
        if (rc != 0) return rc;                                                                 \
        return magma_##P##gesv_batched(n, nrhs, (T **)p.a, ldda, (magma_int_t **)p.b,           \
                                       (T **)p.c, lddb, dinfo_array, batchCount, queue);        \
    }

MLU_STRIDED_GETRF(d, double)
MLU_STRIDED_GETRF(s, float)
MLU_STRIDED_GETRS(d, double)
MLU_STRIDED_GETRS(s, float)
MLU_STRIDED_GESV(d, double)
MLU_STRIDED_GESV(s, float)
