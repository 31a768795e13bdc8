/*
 * magma_lu.h -- C ABI of the GB300-native batched LU factor-and-solve library
 * (libmagma_lu.so).
 *
 * The names, argument order, argument meaning, return codes and pivot/info
 * conventions are those of MAGMA 2.x, so that code written against MAGMA's
 * batched LU entry points links against this library unchanged.  Every
 * declaration below cites the MAGMA interface it replaces, by the path of the
 * file inside the MAGMA source tree.  MAGMA writes its batched routines once
 * in double-complex ("z") and generates the d/s files at build time; the
 * citations point to the z templates (read z -> d, magmaDoubleComplex ->
 * double).
 *
 * Conventions (identical to MAGMA):
 *   - magma_int_t is a 32-bit int (LP64 build; include/magma_types.h:68-71).
 *   - Matrices are column-major, element (i,j) of matrix k at
 *     dA_array[k][i + j*ldda].
 *   - All arrays passed to batched routines -- the pointer arrays themselves,
 *     the matrices, the pivot vectors and the info vector -- live in device
 *     memory and are owned by the caller.
 *   - Pivots are 1-based, LAPACK sequential-interchange order: row i of the
 *     matrix was interchanged with row ipiv[i].
 *   - info[k] = 0 on success, or j > 0 when U(j,j) of matrix k is exactly
 *     zero (the factorisation still completes).
 *   - A negative return value -i means argument i was illegal; the routine
 *     then prints a message through magma_xerbla and does nothing else.
 *   - Every routine only enqueues work on the queue's CUDA stream; none
 *     synchronises the host unless its description says so.
 */
#ifndef MAGMA_LU_H
#define MAGMA_LU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Types and constants -- include/magma_types.h:68-100, 549-634            */

typedef int magma_int_t;              /* include/magma_types.h:71 (LP64) */
typedef int magma_device_t;           /* include/magma_types.h:101 */
typedef void *magma_ptr;
typedef struct magma_queue *magma_queue_t;   /* include/magma_types.h:99-100 */

#define MAGMA_SUCCESS               0
#define MAGMA_ERR                  -100
#define MAGMA_ERR_NOT_INITIALIZED  -101
#define MAGMA_ERR_NOT_SUPPORTED    -103
#define MAGMA_ERR_HOST_ALLOC       -112
#define MAGMA_ERR_DEVICE_ALLOC     -113
#define MAGMA_ERR_INVALID_PTR      -115
#define MAGMA_ERR_UNKNOWN          -116
#define MAGMA_ERR_NOT_IMPLEMENTED  -117

typedef enum {
    MagmaNoTrans   = 111,
    MagmaTrans     = 112,
    MagmaConjTrans = 113
} magma_trans_t;                      /* include/magma_types.h:613-618 */

typedef enum {
    MagmaFalse = 0,
    MagmaTrue  = 1
} magma_bool_t;                       /* include/magma_types.h:600-603 */

typedef enum {
    MagmaUpper = 121,
    MagmaLower = 122
} magma_uplo_t;                       /* include/magma_types.h:619-623 (MagmaFull omitted) */

/* ------------------------------------------------------------------------ */
/* Runtime subset -- include/magma_auxiliary.h:24-25, 82-105, 258-330, 357 */

magma_int_t magma_init(void);         /* interface_cuda/interface.cpp:164 */
magma_int_t magma_finalize(void);     /* interface_cuda/interface.cpp:237 */

/* Prints "Error in <name>, function-specific error (info = <info>)" to
 * stderr, like control/xerbla.cpp:51. */
void magma_xerbla(const char *name, magma_int_t info);

/* MAGMA's magma_queue_create(device, &queue) macro expands to this call
 * (include/magma_auxiliary.h:258-260).  The queue owns a new non-blocking
 * CUDA stream. */
void magma_queue_create_internal(magma_device_t device, magma_queue_t *queue_ptr,
                                 const char *func, const char *file, int line);

/* include/magma_auxiliary.h:284-292.  Wraps an existing cudaStream_t (passed
 * as void* so that this header needs no CUDA include).  The cuBLAS and
 * cuSPARSE handles are accepted for ABI compatibility and ignored: no routine
 * here calls either library. */
void magma_queue_create_from_cuda_internal(magma_device_t device, void *cuda_stream,
                                           void *cublas_handle, void *cusparse_handle,
                                           magma_queue_t *queue_ptr,
                                           const char *func, const char *file, int line);

void magma_queue_destroy_internal(magma_queue_t queue,
                                  const char *func, const char *file, int line);
void magma_queue_sync_internal(magma_queue_t queue,
                               const char *func, const char *file, int line);
magma_int_t magma_queue_get_device(magma_queue_t queue);
/* Returns the queue's cudaStream_t (as void*). */
void *magma_queue_get_cuda_stream(magma_queue_t queue);

#define magma_queue_create(device, queue_ptr) \
    magma_queue_create_internal(device, queue_ptr, __func__, __FILE__, __LINE__)
#define magma_queue_create_from_cuda(device, stream, cublas, cusparse, queue_ptr) \
    magma_queue_create_from_cuda_internal(device, stream, cublas, cusparse, queue_ptr, \
                                          __func__, __FILE__, __LINE__)
#define magma_queue_destroy(queue) \
    magma_queue_destroy_internal(queue, __func__, __FILE__, __LINE__)
#define magma_queue_sync(queue) \
    magma_queue_sync_internal(queue, __func__, __FILE__, __LINE__)

/* Device and pinned-host memory (include/magma_auxiliary.h:82-105). */
magma_int_t magma_malloc(magma_ptr *ptr_ptr, size_t bytes);
magma_int_t magma_malloc_pinned(void **ptr_ptr, size_t bytes);
magma_int_t magma_free_internal(magma_ptr ptr, const char *func, const char *file, int line);
magma_int_t magma_free_pinned_internal(void *ptr, const char *func, const char *file, int line);
#define magma_free(ptr)        magma_free_internal(ptr, __func__, __FILE__, __LINE__)
#define magma_free_pinned(ptr) magma_free_pinned_internal(ptr, __func__, __FILE__, __LINE__)

/* Host <-> device vector copies, asynchronous on the queue's stream followed
 * by a stream synchronisation, like include/magma_copy.h:27-30. */
void magma_setvector_internal(magma_int_t n, magma_int_t elemSize,
                              const void *hx_src, magma_int_t incx,
                              magma_ptr dy_dst, magma_int_t incy, magma_queue_t queue,
                              const char *func, const char *file, int line);
void magma_getvector_internal(magma_int_t n, magma_int_t elemSize,
                              const void *dx_src, magma_int_t incx,
                              void *hy_dst, magma_int_t incy, magma_queue_t queue,
                              const char *func, const char *file, int line);
#define magma_setvector(n, elemSize, hx, incx, dy, incy, queue) \
    magma_setvector_internal(n, elemSize, hx, incx, dy, incy, queue, __func__, __FILE__, __LINE__)
#define magma_getvector(n, elemSize, dx, incx, hy, incy, queue) \
    magma_getvector_internal(n, elemSize, dx, incx, hy, incy, queue, __func__, __FILE__, __LINE__)

/* Pointer-array helpers: output_array[k] = input + k*batch_offset + row +
 * column*lda (magmablas/zset_pointer.cu:20-25, include/magma_zbatched.h:28,
 * include/magma_batched.h:63). */
void magma_dset_pointer(double **output_array, double *input, magma_int_t lda,
                        magma_int_t row, magma_int_t column, magma_int_t batch_offset,
                        magma_int_t batchCount, magma_queue_t queue);
void magma_sset_pointer(float **output_array, float *input, magma_int_t lda,
                        magma_int_t row, magma_int_t column, magma_int_t batch_offset,
                        magma_int_t batchCount, magma_queue_t queue);
void magma_iset_pointer(magma_int_t **output_array, magma_int_t *input, magma_int_t lda,
                        magma_int_t row, magma_int_t column, magma_int_t batch_offset,
                        magma_int_t batchCount, magma_queue_t queue);

/* ------------------------------------------------------------------------ */
/* Batched LU, fixed size -- include/magma_zbatched.h                       */

/* A = P*L*U for batchCount m-by-n matrices (include/magma_zbatched.h:848,
 * src/zgetrf_batched.cpp:82-213).  Returns 0 or -1 (m<0), -2 (n<0),
 * -4 (ldda<max(1,m)).  Workspace comes from the queue; the call neither
 * allocates per call nor synchronises the host. */
magma_int_t magma_dgetrf_batched(magma_int_t m, magma_int_t n,
                                 double **dA_array, magma_int_t ldda,
                                 magma_int_t **ipiv_array, magma_int_t *info_array,
                                 magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrf_batched(magma_int_t m, magma_int_t n,
                                 float **dA_array, magma_int_t ldda,
                                 magma_int_t **ipiv_array, magma_int_t *info_array,
                                 magma_int_t batchCount, magma_queue_t queue);

/* Square n <= 32 factorisation in registers (include/magma_zbatched.h:865,
 * magmablas/zgetrf_batched_smallsq_noshfl.cu:193-285).  Returns -100 when
 * n > 32. */
magma_int_t magma_dgetrf_batched_smallsq_noshfl(magma_int_t n,
                                                double **dA_array, magma_int_t ldda,
                                                magma_int_t **ipiv_array, magma_int_t *info_array,
                                                magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrf_batched_smallsq_noshfl(magma_int_t n,
                                                float **dA_array, magma_int_t ldda,
                                                magma_int_t **ipiv_array, magma_int_t *info_array,
                                                magma_int_t batchCount, magma_queue_t queue);

/* Solve op(A)*X = B with the factors of magma_?getrf_batched
 * (include/magma_zbatched.h:464, src/zgetrs_batched.cpp:86-181).
 * trans is MagmaNoTrans, MagmaTrans or MagmaConjTrans (= MagmaTrans for real
 * data).  Returns 0 or -1 (trans), -2 (n<0), -3 (nrhs<0), -5 (ldda<max(1,n)),
 * -8 (lddb<max(1,n)). */
magma_int_t magma_dgetrs_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                 double **dA_array, magma_int_t ldda,
                                 magma_int_t **dipiv_array,
                                 double **dB_array, magma_int_t lddb,
                                 magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrs_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                 float **dA_array, magma_int_t ldda,
                                 magma_int_t **dipiv_array,
                                 float **dB_array, magma_int_t lddb,
                                 magma_int_t batchCount, magma_queue_t queue);

/* Factor and solve A*X = B (include/magma_zbatched.h:1009,
 * src/zgesv_batched.cpp:93-154).  Returns 0 or -1 (n<0), -2 (nrhs<0),
 * -4 (ldda<max(1,n)), -6 (lddb<max(1,n)).  As in MAGMA, the solve runs even
 * for matrices whose info is positive. */
magma_int_t magma_dgesv_batched(magma_int_t n, magma_int_t nrhs,
                                double **dA_array, magma_int_t ldda,
                                magma_int_t **dipiv_array,
                                double **dB_array, magma_int_t lddb,
                                magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgesv_batched(magma_int_t n, magma_int_t nrhs,
                                float **dA_array, magma_int_t ldda,
                                magma_int_t **dipiv_array,
                                float **dB_array, magma_int_t lddb,
                                magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue);

/* Fused factor + solve for n <= 32 in one kernel (include/magma_zbatched.h:713,
 * magmablas/zgesv_batched_small.cu:376-493).  MAGMA's version handles
 * nrhs == 1 only; this one handles 1 <= nrhs <= 16.  Returns -100 (not
 * applicable) for n > 32 or nrhs > 16, like MAGMA. */
magma_int_t magma_dgesv_batched_small(magma_int_t n, magma_int_t nrhs,
                                      double **dA_array, magma_int_t ldda,
                                      magma_int_t **dipiv_array,
                                      double **dB_array, magma_int_t lddb,
                                      magma_int_t *dinfo_array,
                                      magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgesv_batched_small(magma_int_t n, magma_int_t nrhs,
                                      float **dA_array, magma_int_t ldda,
                                      magma_int_t **dipiv_array,
                                      float **dB_array, magma_int_t lddb,
                                      magma_int_t *dinfo_array,
                                      magma_int_t batchCount, magma_queue_t queue);

/* ------------------------------------------------------------------------ */
/* Batched LU, variable size -- include/magma_zvbatched.h                   */
/* m, n, nrhs, ldda, lddb are device arrays of batchCount ints.             */

/* include/magma_zvbatched.h:57, src/zgetrf_vbatched.cpp:341-398.  Checks the
 * sizes on the device and reads back their maxima (one synchronisation of the
 * queue's stream, as MAGMA does); returns 0 or -1 (some m<0), -2 (some n<0),
 * -4 (some ldda<max(1,m)).  Grows the queue's workspace when needed. */
magma_int_t magma_dgetrf_vbatched(magma_int_t *m, magma_int_t *n,
                                  double **dA_array, magma_int_t *ldda,
                                  magma_int_t **ipiv_array, magma_int_t *info_array,
                                  magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrf_vbatched(magma_int_t *m, magma_int_t *n,
                                  float **dA_array, magma_int_t *ldda,
                                  magma_int_t **ipiv_array, magma_int_t *info_array,
                                  magma_int_t batchCount, magma_queue_t queue);

/* include/magma_zvbatched.h:73, src/zgetrf_vbatched.cpp:224-282.  The caller
 * provides the maxima and a workspace (*lwork < 0: *lwork receives the bytes
 * needed and nothing else happens); no checks, no allocation, no host
 * synchronisation -- capturable in a CUDA graph.  max_minmn and max_mxn are
 * accepted for ABI compatibility and unused.  Returns -12 if *lwork is too
 * small. */
magma_int_t magma_dgetrf_vbatched_max_nocheck_work(magma_int_t *m, magma_int_t *n,
                                                   magma_int_t max_m, magma_int_t max_n,
                                                   magma_int_t max_minmn, magma_int_t max_mxn,
                                                   double **dA_array, magma_int_t *ldda,
                                                   magma_int_t **dipiv_array,
                                                   magma_int_t *info_array,
                                                   void *work, magma_int_t *lwork,
                                                   magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference (MAGMA has no variable-size solve).
 * Arguments as magma_dgetrs_batched with per-matrix n, nrhs, ldda, lddb.
 * Returns 0 or -1 (trans), -2 (some n<0), -3 (some nrhs<0), -5 (ldda), -8 (lddb).
 * One synchronisation to read the maxima. */
magma_int_t magma_dgetrs_vbatched(magma_trans_t trans, magma_int_t *n, magma_int_t *nrhs,
                                  double **dA_array, magma_int_t *ldda,
                                  magma_int_t **dipiv_array,
                                  double **dB_array, magma_int_t *lddb,
                                  magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrs_vbatched(magma_trans_t trans, magma_int_t *n, magma_int_t *nrhs,
                                  float **dA_array, magma_int_t *ldda,
                                  magma_int_t **dipiv_array,
                                  float **dB_array, magma_int_t *lddb,
                                  magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference.  Factor and solve, variable sizes, in one
 * persistent launch.  Returns 0 or -1 (some n<0), -2 (some nrhs<0), -4 (ldda),
 * -7 (lddb).  One synchronisation to check and read the maxima. */
magma_int_t magma_dgesv_vbatched(magma_int_t *n, magma_int_t *nrhs,
                                 double **dA_array, magma_int_t *ldda,
                                 magma_int_t **dipiv_array,
                                 double **dB_array, magma_int_t *lddb,
                                 magma_int_t *dinfo_array,
                                 magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgesv_vbatched(magma_int_t *n, magma_int_t *nrhs,
                                 float **dA_array, magma_int_t *ldda,
                                 magma_int_t **dipiv_array,
                                 float **dB_array, magma_int_t *lddb,
                                 magma_int_t *dinfo_array,
                                 magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference: magma_dgesv_vbatched with caller-provided
 * maxima and workspace, in the style of magma_dgetrf_vbatched_max_nocheck_work;
 * no checks, allocation or synchronisation -- capturable in a CUDA graph. */
magma_int_t magma_dgesv_vbatched_max_nocheck_work(magma_int_t *n, magma_int_t *nrhs,
                                                  magma_int_t max_n, magma_int_t max_nrhs,
                                                  double **dA_array, magma_int_t *ldda,
                                                  magma_int_t **dipiv_array,
                                                  double **dB_array, magma_int_t *lddb,
                                                  magma_int_t *dinfo_array,
                                                  void *work, magma_int_t *lwork,
                                                  magma_int_t batchCount, magma_queue_t queue);

/* ------------------------------------------------------------------------ */
/* Adjoint of the batched solve.  No counterpart in the reference (MAGMA has
 * no autograd).  Given the forward factors (magma_?getrf_batched or
 * magma_?gesv_batched output: LU in dLU_array, pivots in dipiv_array), the
 * solutions X and the upstream gradients G = dL/dX (overwritten by
 * dL/dB = A^{-T} G), writes dL/dA = -(A^{-T} G) X^T to dGA_array.
 * Returns 0 or -i for an illegal argument i (n, nrhs, ldda = 4, lddx = 7,
 * lddg = 9, lddga = 11). */
magma_int_t magma_dgesv_adjoint_batched(magma_int_t n, magma_int_t nrhs,
                                        double **dLU_array, magma_int_t ldda,
                                        magma_int_t **dipiv_array,
                                        double **dX_array, magma_int_t lddx,
                                        double **dG_array, magma_int_t lddg,
                                        double **dGA_array, magma_int_t lddga,
                                        magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgesv_adjoint_batched(magma_int_t n, magma_int_t nrhs,
                                        float **dLU_array, magma_int_t ldda,
                                        magma_int_t **dipiv_array,
                                        float **dX_array, magma_int_t lddx,
                                        float **dG_array, magma_int_t lddg,
                                        float **dGA_array, magma_int_t lddga,
                                        magma_int_t batchCount, magma_queue_t queue);

/* GA_k = -G_k X_k^T (n x n, rank nrhs) for every k: the outer-product half of
 * the adjoint, in the naming style of magmablas_zger_batched
 * (include/magma_zbatched.h).  Returns 0 or -i (n, nrhs, lddg = 4, lddx = 6,
 * lddga = 8). */
magma_int_t magmablas_dger_neg_batched(magma_int_t n, magma_int_t nrhs,
                                       double **dG_array, magma_int_t lddg,
                                       double **dX_array, magma_int_t lddx,
                                       double **dGA_array, magma_int_t lddga,
                                       magma_int_t batchCount, magma_queue_t queue);
magma_int_t magmablas_sger_neg_batched(magma_int_t n, magma_int_t nrhs,
                                       float **dG_array, magma_int_t lddg,
                                       float **dX_array, magma_int_t lddx,
                                       float **dGA_array, magma_int_t lddga,
                                       magma_int_t batchCount, magma_queue_t queue);

/* ------------------------------------------------------------------------ */
/* FP32 factorisation with tensor-core trailing updates.  The batched form of
 * the reference's half-precision factorisation (magma_xhsgetrf_gpu,
 * src/xhsgetrf_gpu.cpp:212; Magma_PREC_SHT, include/magma_types.h:861): the
 * matrix stays FP32, panels, interchanges and TRSM run in FP32, and every
 * trailing update of at least 128 x 128 runs on the tensor cores with FP16
 * (precision = 905, Magma_PREC_SHT) or BF16 (precision = 930, no counterpart
 * in the reference) operands and FP32 accumulation.  work == NULL: *lwork
 * receives the workspace bytes.  Returns 0, -i for an illegal argument
 * (precision = 1, m = 2, n = 3, ldda = 5) or -9 if *lwork is too small. */
#define Magma_PREC_SHT 905
#define Magma_PREC_SBT 930
magma_int_t magma_sgetrf_batched_tc(magma_int_t precision, magma_int_t m, magma_int_t n,
                                    float **dA_array, magma_int_t ldda,
                                    magma_int_t **ipiv_array, magma_int_t *info_array,
                                    void *work, size_t *lwork,
                                    magma_int_t batchCount, magma_queue_t queue);
/* Error flag left by the last magma_sgetrf_batched_tc in `work` (0: no tensor
 * pipeline wait timed out); synchronises the queue. */
magma_int_t magma_sgetrf_batched_tc_status(magma_int_t m, magma_int_t n, void *work,
                                           magma_int_t batchCount, magma_queue_t queue);
/* No counterpart in the reference.  Self-test of the tensor-core kernels'
 * bounded waits: one CTA takes tensor memory and waits, for at most
 * limit_cycles SM clocks (1 .. 4e9), on an mbarrier that nothing arrives at
 * (nothing is in flight), then records error 3 in *flag (one int of device
 * memory), frees the tensor memory and returns.  Returns the recorded code (3
 * when the wait ran out, as it must) or -1 / -2 for a bad limit / flag, and
 * leaves the context usable.  Synchronises the queue. */
magma_int_t magma_sgetrf_batched_tc_wait_selftest(long long limit_cycles, magma_int_t *flag,
                                                  magma_queue_t queue);

/* ------------------------------------------------------------------------ */
/* Batched mixed-precision iterative refinement.  MAGMA refines one matrix
 * at a time (magma_dsgesv_gpu, src/zcgesv_gpu.cpp:144-366, declared in
 * include/magma_zc.h); these apply the same algorithm, arguments and ITER
 * codes to a batch:
 *   iter[k] >= 0   converged after iter[k] refinements (0: the FP32 solve was
 *                  already accurate), A_k unchanged, ipiv_k = FP32 pivots;
 *   iter[k] = -2   A_k overflows in FP32;  -3  the FP32 LU hit a zero pivot;
 *   iter[k] = -itermax-1  no convergence.
 * For iter[k] < 0 the matrix is re-solved in FP64 (A_k overwritten by its
 * FP64 LU, info[k] from that factorisation), like zcgesv_gpu.cpp:352-362.
 * Size limits (all of these routines and their adjoints): nrhs <= 16, and the
 * order n such that one matrix's right-hand sides fit in shared memory -- on
 * GB300 n <= 13999 for nrhs = 1, 12800 for 2, 6400 for 3..4, 3200 for 5..8,
 * 1600 for 9..16; larger orders return MAGMA_ERR_NOT_SUPPORTED with a message
 * naming the limit. */

/* FP32 factorisation, FP64 residual, ITERMAX = 30, dsgesv stopping rule
 * ||r_c||_inf <= ||x_c||_inf * ||A||_inf * eps * sqrt(n) for every column c.
 * Uses (and grows) the queue's workspace; synchronises the queue's stream
 * once at the end to decide whether any matrix needs the FP64 re-solve.
 * nrhs <= 16. */
magma_int_t magma_dsgesv_batched(magma_int_t n, magma_int_t nrhs,
                                 double **dA_array, magma_int_t ldda,
                                 magma_int_t **dipiv_array,
                                 double **dB_array, magma_int_t lddb,
                                 double **dX_array, magma_int_t lddx,
                                 magma_int_t *dinfo_array, magma_int_t *diter_array,
                                 magma_int_t batchCount, magma_queue_t queue);

/* Expert form with caller-provided workspace (work == NULL: *lwork receives
 * the byte count and nothing else happens; the query needs no queue).
 * tol > 0 replaces the dsgesv rule by the scaled-residual rule
 * ||B - A X||_inf / (||A||_inf ||X||_inf n eps) <= tol (the reference tester's
 * acceptance metric, testing/testing_zgesv_batched.cpp:131-152).
 * fallback = 0 skips the FP64 re-solve: the call then never synchronises and
 * is capturable in a CUDA graph; matrices with iter < 0 keep the last iterate.
 * Returns -15 when *lwork is too small. */
magma_int_t magma_dsgesv_batched_work(magma_int_t n, magma_int_t nrhs,
                                      double **dA_array, magma_int_t ldda,
                                      magma_int_t **dipiv_array,
                                      double **dB_array, magma_int_t lddb,
                                      double **dX_array, magma_int_t lddx,
                                      magma_int_t *dinfo_array, magma_int_t *diter_array,
                                      magma_int_t itermax, double tol, magma_int_t fallback,
                                      void *work, size_t *lwork,
                                      magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference.  The same solve as magma_dsgesv_batched
 * (same arguments, ITER codes and FP64 re-solve) for callers that cannot
 * allocate device memory -- a process whose device memory is reserved by
 * another allocator, code where allocation calls are not allowed, or a
 * foreign-language binding with no way to own a device buffer.  It allocates
 * nothing: its scratch is a 32 MiB array compiled into the library, present on
 * every GPU that loads it until the process exits.  Returns
 * MAGMA_ERR_NOT_SUPPORTED, with a message, when the batch needs more scratch
 * than that (workspace size: magma_dsgesv_batched_work with work == NULL).
 * The first call on each device looks up the array's address and should come
 * before any stream capture.  All calls share the array: calls that overlap on
 * the GPU race, so issue them in order on one stream. */
magma_int_t magma_dsgesv_batched_noalloc(magma_int_t n, magma_int_t nrhs,
                                         double **dA_array, magma_int_t ldda,
                                         magma_int_t **dipiv_array,
                                         double **dB_array, magma_int_t lddb,
                                         double **dX_array, magma_int_t lddx,
                                         magma_int_t *dinfo_array, magma_int_t *diter_array,
                                         magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference: magma_dsgesv_batched_work with the
 * factorisation precision as first argument -- 900 (Magma_PREC_SS: FP32
 * factorisation, identical to magma_dsgesv_batched_work), 905
 * (Magma_PREC_SHT: FP32 storage, trailing updates on the tensor cores with
 * FP16 operands, the matrix first scaled by powers of two per row and column so
 * that FP16 cannot overflow) or 930 (Magma_PREC_SBT: BF16 operands, no
 * scaling).  The half-precision forms converge for moderately conditioned
 * matrices (kappa * unit roundoff well below 1) and otherwise end with the
 * FP64 re-solve.  Error codes: -1 precision, then those of
 * magma_dsgesv_batched_work shifted by one. */
magma_int_t magma_dxgesv_batched_work(magma_int_t precision, magma_int_t n, magma_int_t nrhs,
                                      double **dA_array, magma_int_t ldda,
                                      magma_int_t **dipiv_array,
                                      double **dB_array, magma_int_t lddb,
                                      double **dX_array, magma_int_t lddx,
                                      magma_int_t *dinfo_array, magma_int_t *diter_array,
                                      magma_int_t itermax, double tol, magma_int_t fallback,
                                      void *work, size_t *lwork,
                                      magma_int_t batchCount, magma_queue_t queue);

/* Batched form of magma_dxgesv_gmres_gpu (src/dxgesv_gmres_gpu.cpp:160-170,
 * declared in include/magma_htc.h) for the two refinement solvers that use a
 * low-precision LU: solver_type 920 (Magma_REFINE_IRSTRS, include/
 * magma_types.h:873) is magma_dxgesv_batched_work; 922 (Magma_REFINE_IRGMSTRS)
 * solves each refinement iteration's correction equation A d = r with GMRES
 * right-preconditioned by the factors (at most min(n, 50) inner iterations,
 * stop at a 1e-4 relative reduction, as the reference's inner FGMRES) instead
 * of one solve.  The residual, update and stopping rule stay in FP64 (as
 * magma_dxgesv_batched_work); the inner GMRES runs in FP32 on an FP32 copy of
 * A.  diter_array reports, for a converged matrix, the total of its inner
 * iteration counts (the largest over its right-hand sides in each refinement
 * iteration), as the reference's iter for these solvers; the other codes are
 * those of magma_dxgesv_batched_work, itermax bounding the refinement
 * iterations (the reference uses max(10, min(n, 500) / 50) for this solver).
 * Unlike the reference, a refinement step after which the residual 2-norm of
 * some right-hand side has not at least halved ends that matrix's refinement
 * (iter -itermax-1, then the FP64 re-solve when fallback is set).  922 takes
 * nrhs <= 8 and uniform sizes.  Other arguments,
 * workspace query and errors as magma_dxgesv_batched_work, shifted by two;
 * -1 precision, -2 solver_type, -4 nrhs above 8 for 922. */
#define Magma_REFINE_IRSTRS 920
#define Magma_REFINE_IRGMSTRS 922
magma_int_t magma_dxgesv_gmres_batched_work(magma_int_t precision, magma_int_t solver_type,
                                            magma_int_t n, magma_int_t nrhs,
                                            double **dA_array, magma_int_t ldda,
                                            magma_int_t **dipiv_array,
                                            double **dB_array, magma_int_t lddb,
                                            double **dX_array, magma_int_t lddx,
                                            magma_int_t *dinfo_array, magma_int_t *diter_array,
                                            magma_int_t itermax, double tol, magma_int_t fallback,
                                            void *work, size_t *lwork,
                                            magma_int_t batchCount, magma_queue_t queue);

/* Batched form of magma_dsposv_gpu (src/zcposv_gpu.cpp:134, declared as
 * magma_zcposv_gpu in include/magma_zc.h:69): for symmetric positive definite
 * A (lower triangle referenced), FP32 Cholesky of float(A) and FP64 refinement
 * (FP64 residual, update and stopping rule, FP32 L L^T corrections); ITER
 * codes, tol, fallback and the workspace query as magma_dsgesv_batched_work
 * (-3: the FP32 Cholesky met a non-positive pivot).  With fallback, matrices
 * that did not converge are solved by magma_dposv_batched in FP64 (A then
 * holds their FP64 Cholesky factor, info its result).  MagmaUpper returns -1.
 * Errors: -1 uplo, -2 n, -3 nrhs (> 16), -5 ldda, -7 lddb, -9 lddx,
 * -12 itermax. */
magma_int_t magma_dsposv_batched_work(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                                      double **dA_array, magma_int_t ldda,
                                      double **dB_array, magma_int_t lddb,
                                      double **dX_array, magma_int_t lddx,
                                      magma_int_t *dinfo_array, magma_int_t *diter_array,
                                      magma_int_t itermax, double tol, magma_int_t fallback,
                                      void *work, size_t *lwork,
                                      magma_int_t batchCount, magma_queue_t queue);
/* magma_dsposv_batched_work with itermax 30, the default stopping rule, the
 * fallback, and workspace owned by the queue (allocated, after a
 * synchronisation, when too small). */
magma_int_t magma_dsposv_batched(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                                 double **dA_array, magma_int_t ldda,
                                 double **dB_array, magma_int_t lddb,
                                 double **dX_array, magma_int_t lddx,
                                 magma_int_t *dinfo_array, magma_int_t *diter_array,
                                 magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference: the batched refinement of
 * magma_dxgesv_batched_work for a variable-size batch.  n[k], nrhs[k], ldda[k],
 * lddb[k] and lddx[k] are device arrays; max_n and max_nrhs (<= 16) are their
 * maxima, taken from the caller unchecked as in the _max_nocheck routines.
 * precision 900 (Magma_PREC_SS): the FP32 factorisation runs in the persistent
 * variable-size kernel.  Workspace query with work == NULL (sized by
 * batchCount, max_n and max_nrhs).  No allocation; no synchronisation unless
 * fallback is set.  Errors: -1 precision, -4 max_n, -5 max_nrhs, -15 itermax,
 * -18 lwork too small, -19 lwork NULL, -20 batchCount. */
magma_int_t magma_dxgesv_vbatched_work(magma_int_t precision, magma_int_t *n, magma_int_t *nrhs,
                                       magma_int_t max_n, magma_int_t max_nrhs,
                                       double **dA_array, magma_int_t *ldda,
                                       magma_int_t **dipiv_array, double **dB_array,
                                       magma_int_t *lddb, double **dX_array, magma_int_t *lddx,
                                       magma_int_t *dinfo_array, magma_int_t *diter_array,
                                       magma_int_t itermax, double tol, magma_int_t fallback,
                                       void *work, size_t *lwork, magma_int_t batchCount,
                                       magma_queue_t queue);

/* No counterpart in the reference: the adjoint of a refinement solve.  Given
 * the forward call's inputs and outputs -- A and ipiv as magma_dxgesv_batched_work
 * (precision 900) or magma_dxgesv_vbatched_work left them, its solution X, its
 * iteration codes diter_fwd and its workspace `work` (same sizes, untouched
 * since, holding the FP32 factors) -- and an upstream gradient G of X, computes
 * GB = A^{-T} G (the gradient of B), refined to FP64 accuracy with the FP32
 * factors (residual G - A^T GB in FP64, the forward's stopping rule with
 * ||A^T||_inf), and, when dGA_array is not NULL, GA = -GB X^T (the gradient of
 * A).  Matrices whose forward solve fell back to FP64 use their FP64 factors
 * (a transposed FP64 solve); with `fallback`, matrices whose adjoint
 * refinement does not converge are factored in FP64 in place (A, ipiv and
 * info overwritten) and solved the same way.  diter_array receives the
 * adjoint's iteration codes (the forward's code for FP64 matrices).  G is not
 * modified.  With `fallback` the call synchronises once (to size the FP64
 * solves); without it, it never synchronises (capturable in a CUDA graph) and
 * matrices with a negative forward or adjoint code keep an unsolved GB.  Errors: negative
 * argument positions; MAGMA_ERR_NOT_SUPPORTED for orders whose solve or
 * residual does not fit in shared memory. */
magma_int_t magma_dxgesv_adjoint_batched_work(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                              magma_int_t ldda, magma_int_t **dipiv_array,
                                              double **dX_array, magma_int_t lddx,
                                              double **dG_array, magma_int_t lddg,
                                              double **dGB_array, magma_int_t lddgb,
                                              double **dGA_array, magma_int_t lddga,
                                              magma_int_t *diter_fwd, magma_int_t *dinfo_array,
                                              magma_int_t *diter_array, magma_int_t itermax,
                                              double tol, magma_int_t fallback, void *work,
                                              size_t lwork, magma_int_t batchCount,
                                              magma_queue_t queue);
magma_int_t magma_dxgesv_adjoint_vbatched_work(magma_int_t *n, magma_int_t *nrhs,
                                               magma_int_t max_n, magma_int_t max_nrhs,
                                               double **dA_array, magma_int_t *ldda,
                                               magma_int_t **dipiv_array, double **dX_array,
                                               magma_int_t *lddx, double **dG_array,
                                               magma_int_t *lddg, double **dGB_array,
                                               magma_int_t *lddgb, double **dGA_array,
                                               magma_int_t *lddga, magma_int_t *diter_fwd,
                                               magma_int_t *dinfo_array, magma_int_t *diter_array,
                                               magma_int_t itermax, double tol,
                                               magma_int_t fallback, void *work, size_t lwork,
                                               magma_int_t batchCount, magma_queue_t queue);

/* No counterpart in the reference: magmablas_dger_neg_batched for a
 * variable-size batch, GA_k = -G_k X_k^T (order n[k], nrhs[k] columns; max_n
 * the largest order).  Errors: -3 max_n, -10 batchCount. */
magma_int_t magmablas_dger_neg_vbatched(magma_int_t *n, magma_int_t *nrhs, magma_int_t max_n,
                                        double **dG_array, magma_int_t *lddg, double **dX_array,
                                        magma_int_t *lddx, double **dGA_array, magma_int_t *lddga,
                                        magma_int_t batchCount, magma_queue_t queue);

/* Inverse from the LU factors, out of place (include/magma_zbatched.h:872,
 * src/zgetri_outofplace_batched.cpp:82): invA = inv(A) = inv(U) inv(L) P^T
 * for factors and pivots from magma_?getrf_batched.  dA_array is read only;
 * info_array is not written (as in the reference).  Never synchronises.
 * Errors: -1 n, -3 ldda, -6 lddia, -8 batchCount; MAGMA_ERR_NOT_SUPPORTED when
 * 8 columns of order n do not fit in shared memory. */
magma_int_t magma_dgetri_outofplace_batched(magma_int_t n, double **dA_array, magma_int_t ldda,
                                            magma_int_t **dipiv_array, double **dinvA_array,
                                            magma_int_t lddia, magma_int_t *info_array,
                                            magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetri_outofplace_batched(magma_int_t n, float **dA_array, magma_int_t ldda,
                                            magma_int_t **dipiv_array, float **dinvA_array,
                                            magma_int_t lddia, magma_int_t *info_array,
                                            magma_int_t batchCount, magma_queue_t queue);

/* Strided batches (no counterpart for getrf/getrs/gesv in the reference,
 * which offers the form for banded LU, magma_zgbtrf_batched_strided,
 * include/magma_zbatched.h:613): matrix k at dA + k*strideA, its pivots at
 * dipiv + k*strideP, its right-hand sides at dB + k*strideB (strides in
 * elements).  The pointer arrays are built on the device in the queue's
 * scratch (allocated on first use, then reused), then the pointer-array
 * routine runs: identical results.  Errors: those of the pointer-array
 * routine, or the position of a stride that is too small. */
magma_int_t magma_dgetrf_batched_strided(magma_int_t m, magma_int_t n, double *dA,
                                         magma_int_t ldda, magma_int_t strideA,
                                         magma_int_t *dipiv, magma_int_t strideP,
                                         magma_int_t *info_array, magma_int_t batchCount,
                                         magma_queue_t queue);
magma_int_t magma_sgetrf_batched_strided(magma_int_t m, magma_int_t n, float *dA,
                                         magma_int_t ldda, magma_int_t strideA,
                                         magma_int_t *dipiv, magma_int_t strideP,
                                         magma_int_t *info_array, magma_int_t batchCount,
                                         magma_queue_t queue);
magma_int_t magma_dgetrs_batched_strided(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                         double *dA, magma_int_t ldda, magma_int_t strideA,
                                         magma_int_t *dipiv, magma_int_t strideP, double *dB,
                                         magma_int_t lddb, magma_int_t strideB,
                                         magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrs_batched_strided(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                         float *dA, magma_int_t ldda, magma_int_t strideA,
                                         magma_int_t *dipiv, magma_int_t strideP, float *dB,
                                         magma_int_t lddb, magma_int_t strideB,
                                         magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_dgesv_batched_strided(magma_int_t n, magma_int_t nrhs, double *dA,
                                        magma_int_t ldda, magma_int_t strideA, magma_int_t *dipiv,
                                        magma_int_t strideP, double *dB, magma_int_t lddb,
                                        magma_int_t strideB, magma_int_t *dinfo_array,
                                        magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgesv_batched_strided(magma_int_t n, magma_int_t nrhs, float *dA,
                                        magma_int_t ldda, magma_int_t strideA, magma_int_t *dipiv,
                                        magma_int_t strideP, float *dB, magma_int_t lddb,
                                        magma_int_t strideB, magma_int_t *dinfo_array,
                                        magma_int_t batchCount, magma_queue_t queue);

/* LU without pivoting (include/magma_zbatched.h:977-999,
 * src/zgetrf_nopiv_batched.cpp): the diagonal entry is the pivot.  info = the
 * first zero diagonal (1-based); its column is left unscaled.  getrs_nopiv's
 * info_array is unused, as in the reference.  No allocation or
 * synchronisation. */
magma_int_t magma_dgetrf_nopiv_batched(magma_int_t m, magma_int_t n, double **dA_array,
                                       magma_int_t ldda, magma_int_t *info_array,
                                       magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrf_nopiv_batched(magma_int_t m, magma_int_t n, float **dA_array,
                                       magma_int_t ldda, magma_int_t *info_array,
                                       magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_dgetrs_nopiv_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                       double **dA_array, magma_int_t ldda, double **dB_array,
                                       magma_int_t lddb, magma_int_t *info_array,
                                       magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sgetrs_nopiv_batched(magma_trans_t trans, magma_int_t n, magma_int_t nrhs,
                                       float **dA_array, magma_int_t ldda, float **dB_array,
                                       magma_int_t lddb, magma_int_t *info_array,
                                       magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_dgesv_nopiv_batched(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                      magma_int_t ldda, double **dB_array, magma_int_t lddb,
                                      magma_int_t *info_array, magma_int_t batchCount,
                                      magma_queue_t queue);
magma_int_t magma_sgesv_nopiv_batched(magma_int_t n, magma_int_t nrhs, float **dA_array,
                                      magma_int_t ldda, float **dB_array, magma_int_t lddb,
                                      magma_int_t *info_array, magma_int_t batchCount,
                                      magma_queue_t queue);

/* Random butterfly transformation and the solve built on it
 * (include/magma_zbatched.h:1001-1045, src/zgesv_rbt_batched.cpp,
 * src/zgerbt_batched.cpp).  Depth-2 recursive butterflies U, V (outer order n,
 * inner orders ceil(n/2) and n - ceil(n/2)) with random diagonals: U and V
 * are host arrays of 2n entries, du and dv their device copies.
 * magma_dgerbt_batched: A <- U^T A V and B <- U^T B for every matrix; with
 * gen == MagmaTrue it first fills U and V (exp(r/10), r uniform in [-1/2,1/2),
 * one process-wide stream); copies them to the device and synchronises.
 * magmablas_dprbt_batched: A <- U^T A V; _mtv: B <- U^T B; _mv: B <- V B.
 * magma_dgesv_rbt_batched: gerbt, LU without pivoting, solve, x = V y; the
 * matrix is overwritten by the factors of U^T A V.  No iterative refinement
 * (as in the reference). */
magma_int_t magma_dgerbt_batched(magma_bool_t gen, magma_int_t n, magma_int_t nrhs,
                                 double **dA_array, magma_int_t ldda, double **dB_array,
                                 magma_int_t lddb, double *U, double *V, magma_int_t *info,
                                 magma_int_t batchCount, magma_queue_t queue);
void magmablas_dprbt_batched(magma_int_t n, double **dA_array, magma_int_t ldda, double *du,
                             double *dv, magma_int_t batchCount, magma_queue_t queue);
void magmablas_dprbt_mtv_batched(magma_int_t n, magma_int_t nrhs, double *du, double **db_array,
                                 magma_int_t lddb, magma_int_t batchCount, magma_queue_t queue);
void magmablas_dprbt_mv_batched(magma_int_t n, magma_int_t nrhs, double *dv, double **db_array,
                                magma_int_t lddb, magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_dgesv_rbt_batched(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                    magma_int_t ldda, double **dB_array, magma_int_t lddb,
                                    magma_int_t *dinfo_array, magma_int_t batchCount,
                                    magma_queue_t queue);

/* Cholesky A = L L^T of symmetric positive definite matrices and the solve
 * (include/magma_zbatched.h: magma_zpotrf_batched, magma_zpotrs_batched,
 * magma_zposv_batched; src/zpotrf_batched.cpp:96-170).  Lower triangle only;
 * MagmaUpper returns -1 after magma_xerbla, as in the reference.  info = j
 * (1-based) for the first non-positive (or NaN) pivot; that matrix is left
 * as it was at that point.  The strictly upper triangle is never written.  No
 * allocation, no synchronisation. */
magma_int_t magma_dpotrf_batched(magma_uplo_t uplo, magma_int_t n, double **dA_array,
                                 magma_int_t ldda, magma_int_t *info_array,
                                 magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_spotrf_batched(magma_uplo_t uplo, magma_int_t n, float **dA_array,
                                 magma_int_t ldda, magma_int_t *info_array,
                                 magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_dpotrs_batched(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                                 double **dA_array, magma_int_t ldda, double **dB_array,
                                 magma_int_t lddb, magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_spotrs_batched(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                                 float **dA_array, magma_int_t ldda, float **dB_array,
                                 magma_int_t lddb, magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_dposv_batched(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                                double **dA_array, magma_int_t ldda, double **dB_array,
                                magma_int_t lddb, magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue);
magma_int_t magma_sposv_batched(magma_uplo_t uplo, magma_int_t n, magma_int_t nrhs,
                                float **dA_array, magma_int_t ldda, float **dB_array,
                                magma_int_t lddb, magma_int_t *dinfo_array,
                                magma_int_t batchCount, magma_queue_t queue);

/* ------------------------------------------------------------------------
 * Tuning of the variable-size kernel.  No counterpart in the reference, whose
 * batched routines read fixed crossover tables
 * (control/get_batched_crossover.cpp:300-342, 918-928).
 *
 * The persistent kernel of magma_?getrf_vbatched / magma_?gesv_vbatched picks,
 * per matrix, a panel width (nb: 8, 16 or 32) and a trailing-update tile
 * (tile: 0 = 64x64, 1 = 32x64, 2 = 32x32) from a table indexed by the size bin
 * of max(m, n): <= 16, 32, 64, 128, 256, 512, 1024, larger (8 entries).  No
 * choice changes a result bit: every element receives the same updates in the
 * same order.
 *
 * Batches whose largest matrix exceeds 256 do not use the table: they run the
 * per-step kernels of the fixed-size path with per-matrix sizes (several CTAs
 * per matrix and step).
 *
 * magma_?getrf_vbatched_autotune: times every (nb in {16, 32}) x (tile)
 * candidate on `queue`'s device for each bin up to max_n (bins above 256 are
 * not timed), installs the fastest in the table of that precision and returns
 * the table in nb[8], tile[8] (either may be NULL).  Allocates its trial
 * batches and synchronises the queue.  max_n = 0 only returns the table.
 * Errors: -1 max_n < 0, -4 no queue, MAGMA_ERR_DEVICE_ALLOC.
 *
 * magma_?vbatched_tuning_get / _set: read or replace the table (8 entries
 * each); _set returns -1 for a bad nb, -2 for a bad tile. */
magma_int_t magma_dgetrf_vbatched_autotune(magma_int_t max_n, magma_int_t *nb, magma_int_t *tile,
                                           magma_queue_t queue);
magma_int_t magma_sgetrf_vbatched_autotune(magma_int_t max_n, magma_int_t *nb, magma_int_t *tile,
                                           magma_queue_t queue);
magma_int_t magma_dvbatched_tuning_get(magma_int_t *nb, magma_int_t *tile);
magma_int_t magma_svbatched_tuning_get(magma_int_t *nb, magma_int_t *tile);
magma_int_t magma_dvbatched_tuning_set(const magma_int_t *nb, const magma_int_t *tile);
magma_int_t magma_svbatched_tuning_set(const magma_int_t *nb, const magma_int_t *tile);

/* ------------------------------------------------------------------------
 * Tuning of the fixed-size factorisation and the tuning file.  No counterpart
 * in the reference, whose batched LU reads fixed crossover tables
 * (control/get_batched_crossover.cpp:300-342, 918-928;
 * control/get_batched_gemm_decision.cpp:233-253).  One table per precision,
 * six size bins of max(m, n): <= 64, 128, 256, 512, 1024, larger.  Entries:
 *   two_level[b]  FP32: 1 = 128-column blocks with one rank-128 update right of
 *                 each, 0 = a rank-32 update after every 32-column panel;
 *   band_ctas[b]  FP32: the fused band kernel when a step gives at least this
 *                 many CTAs per SM (1, 2 or 4);
 *   tile64[b]     FP64: 1 = 64 x 64 update tiles, 0 = 32 x 32.
 * Every setting gives bit-identical results; only the time changes.
 *
 * magma_?getrf_batched_autotune: times the candidates of every bin up to max_n
 * on `batch` trial matrices on `queue`'s device (allocates them, synchronises)
 * and installs the fastest.  Must not run beside other calls of this library.
 * Errors: -1 max_n < 0, -2 batch < 1, -3 no queue, MAGMA_ERR_DEVICE_ALLOC.
 * magma_?getrf_batched_tuning_get / _set: read or replace the table (six
 * entries per array); _set returns -1 / -2 / -3 for a bad entry.
 *
 * magma_lu_tuning_save / _load: write or read this table and the
 * variable-size one (magma_?vbatched_tuning_*) as a JSON file; _load checks
 * the whole file before installing anything.  A queue created while the
 * environment variable MAGMA_LU_TUNING_FILE names a file loads it, once per
 * process.  Return 0, -1 for a NULL path, MAGMA_ERR_UNKNOWN for an unreadable
 * or malformed file. */
magma_int_t magma_dgetrf_batched_autotune(magma_int_t max_n, magma_int_t batch, magma_queue_t queue);
magma_int_t magma_sgetrf_batched_autotune(magma_int_t max_n, magma_int_t batch, magma_queue_t queue);
magma_int_t magma_dgetrf_batched_tuning_get(magma_int_t *two_level, magma_int_t *band_ctas,
                                            magma_int_t *tile64);
magma_int_t magma_sgetrf_batched_tuning_get(magma_int_t *two_level, magma_int_t *band_ctas,
                                            magma_int_t *tile64);
magma_int_t magma_dgetrf_batched_tuning_set(const magma_int_t *two_level, const magma_int_t *band_ctas,
                                            const magma_int_t *tile64);
magma_int_t magma_sgetrf_batched_tuning_set(const magma_int_t *two_level, const magma_int_t *band_ctas,
                                            const magma_int_t *tile64);
magma_int_t magma_lu_tuning_save(const char *path);
magma_int_t magma_lu_tuning_load(const char *path);

/* ------------------------------------------------------------------------
 * Launch accounting and kernel timing.  No counterpart in the reference,
 * whose testers time whole calls on the host
 * (testing/testing_zgesv_batched.cpp:158-166).
 *
 * magma_lu_launch_count: number of kernels this library has launched in the
 * process (graph capture counts the captured launches once).
 *
 * magma_lu_timing_start: from now on every launch of one kernel class, on any
 * queue and outside stream capture, is bracketed by CUDA events on its stream,
 * for up to `capacity` launches (later ones are counted as dropped).  Classes:
 * 1 fused n<=32 factor+solve, 2 panel, 3 interchanges + L11^{-1}A12, 4 SIMT
 * trailing update, 5 tensor-core trailing update, 6 triangular solves,
 * 7 refinement FP64 residual, 8 refinement correction solve, 9 refinement
 * conversion, 10 variable-size persistent factor+solve, 11 adjoint outer
 * product, 12 rank-128 update right of a 128-column block (FP32 LU: the
 * block's interchanges, its U12 solve and its trailing update).  Returns -1 for a bad class, -2 for a bad capacity.
 *
 * magma_lu_timing_stop: waits for the recorded events, returns the number of
 * timed launches, the number dropped and their summed device time, and turns
 * timing off.  Use from one host thread. */
long long magma_lu_launch_count(void);
/* No counterpart in the reference.  Fault injection for tests: the next
 * `count` device allocations the library makes for itself (queue workspaces,
 * the autotuner's trial batches, the RBT butterflies) fail as if the device
 * were out of memory, so the calls return MAGMA_ERR_DEVICE_ALLOC as the
 * reference does when its workspace cannot be allocated
 * (src/zgetrf_batched.cpp:137-142).  0 turns it off; returns the count that was
 * still pending. */
magma_int_t magma_lu_fail_allocations(magma_int_t count);
magma_int_t magma_lu_timing_start(magma_int_t kernel_class, magma_int_t capacity);
magma_int_t magma_lu_timing_stop(magma_int_t *launches, magma_int_t *dropped, double *total_ms);

#ifdef __cplusplus
}
#endif

#endif /* MAGMA_LU_H */
