// nopiv.cu -- batched LU without pivoting and its solves.
//
// Replaces magma_?getrf_nopiv_batched, magma_?getrs_nopiv_batched and
// magma_?gesv_nopiv_batched (include/magma_zbatched.h:977-999,
// src/zgetrf_nopiv_batched.cpp): the pivot of column k is the diagonal
// entry.  They run the kernels of the pivoting path with no pivot array: the
// panels take the diagonal as pivot (NOPIV instantiations), the interchange
// step moves nothing, the solves apply no interchanges.  A zero diagonal sets
// info to its 1-based column and leaves that column unscaled (the rule the
// pivoting path applies to a zero pivot).  No allocation, no synchronisation.
#include "common.cuh"

namespace mlu {
template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q);
template <typename T>
magma_int_t blocked_getrs(bool trans, int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB,
                          int lddb, int batch, magma_queue_t q);
}  // namespace mlu

template <typename T>
static magma_int_t getrf_nopiv(const char *name, magma_int_t m, magma_int_t n, T **dA_array,
                               magma_int_t ldda, magma_int_t *info_array, magma_int_t batchCount,
                               magma_queue_t queue)
{
    magma_int_t info = 0;
    if (m < 0) info = -1;
    else if (n < 0) info = -2;
    else if (ldda < mlu_max(1, m)) info = -4;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (batchCount <= 0) return 0;
    if (m == 0 || n == 0)
        return cudaMemsetAsync(info_array, 0, batchCount * sizeof(magma_int_t), queue->stream) ==
                       cudaSuccess ? 0 : MAGMA_ERR_UNKNOWN;
    return mlu::blocked_getrf<T>(m, n, dA_array, ldda, nullptr, info_array, batchCount, queue);
}

template <typename T>
static magma_int_t getrs_nopiv(const char *name, magma_trans_t trans, magma_int_t n,
                               magma_int_t nrhs, T **dA_array, magma_int_t ldda, T **dB_array,
                               magma_int_t lddb, magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    const bool notran = trans == MagmaNoTrans;
    if (!notran && trans != MagmaTrans && trans != MagmaConjTrans) info = -1;
    else if (n < 0) info = -2;
    else if (nrhs < 0) info = -3;
    else if (ldda < mlu_max(1, n)) info = -5;
    else if (lddb < mlu_max(1, n)) info = -7;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    return mlu::blocked_getrs<T>(!notran, n, nrhs, dA_array, ldda, nullptr, dB_array, lddb,
                                 batchCount, queue);
}

template <typename T>
static magma_int_t gesv_nopiv(const char *name, magma_int_t n, magma_int_t nrhs, T **dA_array,
                              magma_int_t ldda, T **dB_array, magma_int_t lddb,
                              magma_int_t *info_array, magma_int_t batchCount,
                              magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (lddb < mlu_max(1, n)) info = -6;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (batchCount <= 0) return 0;
    magma_int_t rc = getrf_nopiv<T>(name, n, n, dA_array, ldda, info_array, batchCount, queue);
    if (rc != 0) return rc;
    return getrs_nopiv<T>(name, MagmaNoTrans, n, nrhs, dA_array, ldda, dB_array, lddb,
                          batchCount, queue);
}

#define MLU_NOPIV(P, T)                                                                        \
    extern "C" magma_int_t magma_##P##getrf_nopiv_batched(                                     \
        magma_int_t m, magma_int_t n, T **dA_array, magma_int_t ldda, magma_int_t *info_array, \
        magma_int_t batchCount, magma_queue_t queue)                                           \
    {                                                                                          \
        return getrf_nopiv<T>(__func__, m, n, dA_array, ldda, info_array, batchCount, queue);  \
    }                                                                                          \
    extern "C" magma_int_t magma_##P##getrs_nopiv_batched(                                     \
        magma_trans_t trans, magma_int_t n, magma_int_t nrhs, T **dA_array, magma_int_t ldda,  \
        T **dB_array, magma_int_t lddb, magma_int_t *info_array, magma_int_t batchCount,       \
        magma_queue_t queue)                                                                   \
    {                                                                                          \
        (void)info_array;                                                                      \
        return getrs_nopiv<T>(__func__, trans, n, nrhs, dA_array, ldda, dB_array, lddb,        \
                              batchCount, queue);                                              \
    }                                                                                          \
    extern "C" magma_int_t magma_##P##gesv_nopiv_batched(                                      \
        magma_int_t n, magma_int_t nrhs, T **dA_array, magma_int_t ldda, T **dB_array,         \
        magma_int_t lddb, magma_int_t *info_array, magma_int_t batchCount,                     \
        magma_queue_t queue)                                                                   \
    {                                                                                          \
        return gesv_nopiv<T>(__func__, n, nrhs, dA_array, ldda, dB_array, lddb, info_array,    \
                             batchCount, queue);                                               \
    }

MLU_NOPIV(d, double)
MLU_NOPIV(s, float)
