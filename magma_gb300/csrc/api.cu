// api.cu -- the MAGMA batched LU entry points (argument checks, dispatch).
//
// Argument checking and return codes follow src/zgetrf_batched.cpp:93-112,
// src/zgetrs_batched.cpp:100-124 and src/zgesv_batched.cpp:102-124; the
// dispatch replaces MAGMA's (small fused kernel for n <= 32, blocked
// right-looking LU otherwise) with this library's kernels.
#include "common.cuh"

namespace mlu {
template <typename T>
magma_int_t small_gesv(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb, int *info,
                       int batch, magma_queue_t q);
template <typename T>
magma_int_t small_getrs(bool trans, int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB,
                        int lddb, int batch, magma_queue_t q);
template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q);
template <typename T>
magma_int_t blocked_getrs(bool trans, int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB,
                          int lddb, int batch, magma_queue_t q);
}  // namespace mlu

template <typename T>
static magma_int_t getrf_batched(const char *name, magma_int_t m, magma_int_t n, T **dA_array,
                                 magma_int_t ldda, magma_int_t **ipiv_array,
                                 magma_int_t *info_array, magma_int_t batchCount,
                                 magma_queue_t queue)
{
    magma_int_t arginfo = 0;
    if (m < 0) arginfo = -1;
    else if (n < 0) arginfo = -2;
    else if (ldda < mlu_max(1, m)) arginfo = -4;
    if (arginfo != 0) {
        magma_xerbla(name, -arginfo);
        return arginfo;
    }
    if (m == 0 || n == 0 || batchCount <= 0) return 0;
    if (m == n && m <= 32)
        return mlu::small_gesv<T>(n, 0, dA_array, ldda, ipiv_array, nullptr, 1, info_array,
                                  batchCount, queue);
    return mlu::blocked_getrf<T>(m, n, dA_array, ldda, ipiv_array, info_array, batchCount, queue);
}

template <typename T>
static magma_int_t getrs_batched(const char *name, magma_trans_t trans, magma_int_t n,
                                 magma_int_t nrhs, T **dA_array, magma_int_t ldda,
                                 magma_int_t **dipiv_array, T **dB_array, magma_int_t lddb,
                                 magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    const bool notran = (trans == MagmaNoTrans);
    if (!notran && trans != MagmaTrans && trans != MagmaConjTrans) info = -1;
    else if (n < 0) info = -2;
    else if (nrhs < 0) info = -3;
    else if (ldda < mlu_max(1, n)) info = -5;
    else if (lddb < mlu_max(1, n)) info = -8;
    if (info != 0) {
        magma_xerbla(name, -info);
        return info;
    }
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    if (n <= 32)
        return mlu::small_getrs<T>(!notran, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                   batchCount, queue);
    return mlu::blocked_getrs<T>(!notran, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                 batchCount, queue);
}

template <typename T>
static magma_int_t gesv_batched(const char *name, magma_int_t n, magma_int_t nrhs, T **dA_array,
                                magma_int_t ldda, magma_int_t **dipiv_array, T **dB_array,
                                magma_int_t lddb, magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue)
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
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    info = mlu::small_gesv<T>(n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb, dinfo_array,
                              batchCount, queue);
    if (info == 0) return 0;
    info = getrf_batched<T>(name, n, n, dA_array, ldda, dipiv_array, dinfo_array, batchCount,
                            queue);
    if (info != 0) return info;
    return getrs_batched<T>(name, MagmaNoTrans, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                            lddb, batchCount, queue);
}

template <typename T>
static magma_int_t gesv_small_entry(const char *name, magma_int_t n, magma_int_t nrhs,
                                    T **dA_array, magma_int_t ldda, magma_int_t **dipiv_array,
                                    T **dB_array, magma_int_t lddb, magma_int_t *dinfo_array,
                                    magma_int_t batchCount, magma_queue_t queue)
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
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    return mlu::small_gesv<T>(n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb, dinfo_array,
                              batchCount, queue);
}

extern "C" {

magma_int_t magma_dgetrf_batched(magma_int_t m, magma_int_t n, double **dA_array, magma_int_t ldda,
                                 magma_int_t **ipiv_array, magma_int_t *info_array,
                                 magma_int_t batchCount, magma_queue_t queue)
{
    return getrf_batched<double>(__func__, m, n, dA_array, ldda, ipiv_array, info_array,
                                 batchCount, queue);
}

magma_int_t magma_sgetrf_batched(magma_int_t m, magma_int_t n, float **dA_array, magma_int_t ldda,
                                 magma_int_t **ipiv_array, magma_int_t *info_array,
                                 magma_int_t batchCount, magma_queue_t queue)
{
    return getrf_batched<float>(__func__, m, n, dA_array, ldda, ipiv_array, info_array,
                                batchCount, queue);
}

magma_int_t magma_dgetrf_batched_smallsq_noshfl(magma_int_t n, double **dA_array,
                                                magma_int_t ldda, magma_int_t **ipiv_array,
                                                magma_int_t *info_array, magma_int_t batchCount,
                                                magma_queue_t queue)
{
    if (n < 0 || ldda < mlu_max(1, n)) return MAGMA_ERR;
    if (n == 0 || batchCount <= 0) return 0;
    return mlu::small_gesv<double>(n, 0, dA_array, ldda, ipiv_array, nullptr, 1, info_array,
                                   batchCount, queue);
}

magma_int_t magma_sgetrf_batched_smallsq_noshfl(magma_int_t n, float **dA_array,
                                                magma_int_t ldda, magma_int_t **ipiv_array,
                                                magma_int_t *info_array, magma_int_t batchCount,
                                                magma_queue_t queue)
{
    if (n < 0 || ldda < mlu_max(1, n)) return MAGMA_ERR;
    if (n == 0 || batchCount <= 0) return 0;
    return mlu::small_gesv<float>(n, 0, dA_array, ldda, ipiv_array, nullptr, 1, info_array,
                                  batchCount, queue);
}

magma_int_t magma_dgetrs_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                 double **dA_array, magma_int_t ldda, magma_int_t **dipiv_array,
                                 double **dB_array, magma_int_t lddb, magma_int_t batchCount,
                                 magma_queue_t queue)
{
    return getrs_batched<double>(__func__, trans, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                 lddb, batchCount, queue);
}

magma_int_t magma_sgetrs_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                 float **dA_array, magma_int_t ldda, magma_int_t **dipiv_array,
                                 float **dB_array, magma_int_t lddb, magma_int_t batchCount,
                                 magma_queue_t queue)
{
    return getrs_batched<float>(__func__, trans, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                lddb, batchCount, queue);
}

magma_int_t magma_dgesv_batched(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                magma_int_t ldda, magma_int_t **dipiv_array, double **dB_array,
                                magma_int_t lddb, magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue)
{
    return gesv_batched<double>(__func__, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                dinfo_array, batchCount, queue);
}

magma_int_t magma_sgesv_batched(magma_int_t n, magma_int_t nrhs, float **dA_array,
                                magma_int_t ldda, magma_int_t **dipiv_array, float **dB_array,
                                magma_int_t lddb, magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue)
{
    return gesv_batched<float>(__func__, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                               dinfo_array, batchCount, queue);
}

magma_int_t magma_dgesv_batched_small(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                      magma_int_t ldda, magma_int_t **dipiv_array,
                                      double **dB_array, magma_int_t lddb,
                                      magma_int_t *dinfo_array, magma_int_t batchCount,
                                      magma_queue_t queue)
{
    return gesv_small_entry<double>(__func__, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                    lddb, dinfo_array, batchCount, queue);
}

magma_int_t magma_sgesv_batched_small(magma_int_t n, magma_int_t nrhs, float **dA_array,
                                      magma_int_t ldda, magma_int_t **dipiv_array,
                                      float **dB_array, magma_int_t lddb,
                                      magma_int_t *dinfo_array, magma_int_t batchCount,
                                      magma_queue_t queue)
{
    return gesv_small_entry<float>(__func__, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                   lddb, dinfo_array, batchCount, queue);
}

}  // extern "C"
