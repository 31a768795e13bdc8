// lu_vbatched.cu -- variable-size batched LU factorisation and solve.
//
// Replaces magma_dgetrf_vbatched and its _max_nocheck_work variant
// (src/zgetrf_vbatched.cpp:20-398: host-side checker and max reductions with
// two device-to-host copies, cudaMalloc'ed workspace, and a host loop of
// panel / swap / trsm / gemm launches whose grids are sized for the largest
// matrix) and adds the solve, which MAGMA does not have for variable sizes:
// magma_dgetrs_vbatched and magma_dgesv_vbatched.
//
// Design: one persistent launch does the whole factorisation (and solve).
//   1. vb_sort_kernel (one CTA): counting sort of the matrices by size,
//      largest first, into a work list -- no host round trip;
//   2. vb_lu_kernel: every CTA repeatedly takes the next matrix of the list
//      (atomic counter) and runs its complete blocked LU -- panel in shared
//      memory, interchanges applied to the other columns and to the
//      right-hand sides, TRSM, 64x64 trailing-update tiles -- then the
//      triangular solves.  Largest-first order keeps the SMs evenly loaded to
//      the end (longest-processing-time scheduling).
// The steps are the device functions of lu_core.cuh, so factors, pivots and
// solutions are bit-identical to the fixed-size path and to the CPU oracle.
// The _max_nocheck_work entry points never allocate or synchronise and can
// be captured in a CUDA graph.
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"
#include "solve_core.cuh"

#include <mutex>
#include <vector>

namespace mlu {

constexpr int VB_THREADS = PANEL_REGS_THREADS;   // the register panel runs on all threads
constexpr int VB_BINS = 1024;
constexpr int VB_NR = 16;                  // right-hand sides per solve pass
constexpr size_t VB_SMEM_CAP = 220 * 1024;

// Per-size-bin tuning of the persistent kernel: panel width and trailing-update
// tile shape for matrices whose max(m, n) falls in bin b (<= 16, 32, 64, 128,
// 256, 512, 1024, larger).  Every choice applies the same updates to every
// element in the same order, so the tuning never changes a result.
constexpr int VB_TUNE_BINS = 8;
// Batches whose largest matrix is at most this run in the persistent kernel
// (one CTA per matrix); larger ones in the per-step kernels of the fixed-size
// path with per-matrix sizes, where every step of a large matrix spreads over
// many CTAs.
constexpr int VB_PERSISTENT_MAX = 256;
enum VbTile { VB_TILE_64x64 = 0, VB_TILE_32x64 = 1, VB_TILE_32x32 = 2, VB_TILE_COUNT = 3 };
struct VbTune {
    unsigned char nb[VB_TUNE_BINS];     // panel width: 8, 16 or 32
    unsigned char tile[VB_TUNE_BINS];   // VbTile
};

__host__ __device__ inline int vb_tune_bin(int mx)
{
    int b = 0;
    for (int ub = 16; b < VB_TUNE_BINS - 1 && mx > ub; ub <<= 1) b++;
    return b;
}

// all tiles of the trailing update of one step, BM x BN tiles
template <typename T, int BM, int BN, int TM, int TN>
__device__ __forceinline__ void vb_update(T *A, int lda, int m, int n, int j0, int ib, T *sL, T *sU)
{
    const int rm = m - j0 - ib, rn = n - j0 - ib;
    for (int tn = 0; tn < rn; tn += BN)
        for (int tm = 0; tm < rm; tm += BM)
            gemm_tile<T, BM, BN, TM, TN>(A, lda, m, n, j0, ib, j0 + ib + tm, j0 + ib + tn, sL, sU);
}

__device__ __forceinline__ int vb_key(int m, int n) { return min(max(max(m, n), 0), VB_BINS - 1); }

// order[] = matrix indices sorted by decreasing max(m,n); counter = 0.
__global__ void __launch_bounds__(1024)
vb_sort_kernel(const int *m_arr, const int *n_arr, int batch, int *order, int *counter)
{
    __shared__ int hist[VB_BINS];
    __shared__ int warp_tot[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < VB_BINS; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (int k = tid; k < batch; k += blockDim.x) atomicAdd(&hist[vb_key(m_arr[k], n_arr[k])], 1);
    __syncthreads();
    // exclusive scan over bins in descending key order (thread t <-> bin VB_BINS-1-t)
    const int bin = VB_BINS - 1 - tid;
    const int v = hist[bin];
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(FULL, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = warp_tot[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(FULL, w, d);
            if (lane >= d) w += y;
        }
        warp_tot[lane] = w - warp_tot[lane];   // exclusive warp offsets
    }
    __syncthreads();
    hist[bin] = warp_tot[warp] + x - v;        // exclusive offset of this bin
    __syncthreads();
    for (int k = tid; k < batch; k += blockDim.x) {
        const int pos = atomicAdd(&hist[vb_key(m_arr[k], n_arr[k])], 1);
        order[pos] = k;
    }
    if (tid == 0) *counter = 0;
}

template <typename T>
__global__ void __launch_bounds__(VB_THREADS, 2)
vb_lu_kernel(const int *m_arr, const int *n_arr, const int *nrhs_arr, T **dA_array,
             const int *ldda_arr, int **ipiv_array, T **dB_array, const int *lddb_arr,
             int *info_array, const int *order, int *counter, int batch, int smem_bytes,
             VbTune tune)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_item, s_ipiv[PANEL_NB], s_row[2 * PANEL_NB], s_src[2 * PANEL_NB], s_cnt;
    const int tid = threadIdx.x, warp = tid >> 5;
    T *sT = reinterpret_cast<T *>(smem);
    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int idx = s_item;
        if (idx >= batch) break;
        const int k = order[idx];
        const int m = m_arr[k], n = n_arr[k], lda = ldda_arr[k];
        const int nrhs = nrhs_arr ? nrhs_arr[k] : 0;
        T *A = dA_array[k];
        int *ipiv = ipiv_array[k];
        T *B = nrhs > 0 ? dB_array[k] : nullptr;
        const int ldb = nrhs > 0 ? lddb_arr[k] : 1;
        const int mn = min(m, n);
        const int bin = vb_tune_bin(max(m, n));
        const int nbw = tune.nb[bin], tile = tune.tile[bin];
        int info = 0;
        for (int j0 = 0; j0 < mn;) {
            const int pm = m - j0;
            // register-resident panel (one row per thread) when pm <= 256, else
            // the shared-memory panel
            const int ib = pm <= VB_THREADS ? min(nbw, mn - j0)
                                            : panel_width<T>(pm, min(nbw, mn - j0),
                                                             (size_t)smem_bytes);
            T *Ap = A + j0 + (size_t)j0 * lda;
            const int il = pm <= VB_THREADS ? panel_factor_regs<T, 1>(pm, ib, Ap, lda, s_ipiv, j0,
                                                                      smem)
                                            : panel_factor<T>(pm, ib, Ap, lda, smem, s_ipiv, j0);
            if (info == 0) info = il;
            if (tid < ib) ipiv[j0 + tid] = j0 + s_ipiv[tid] + 1;
            __syncthreads();
            if (warp == 0) build_permutation(ipiv, j0, ib, s_row, s_src, &s_cnt);
            __syncthreads();
            const int cnt = s_cnt;
            if (cnt > 0) {
                apply_permutation<T>(A, lda, 0, j0, s_row, s_src, cnt, sT);
                apply_permutation<T>(A, lda, j0 + ib, n, s_row, s_src, cnt, sT);
                if (nrhs > 0) apply_permutation<T>(B, ldb, 0, nrhs, s_row, s_src, cnt, sT);
            }
            if (j0 + ib < n) {
                trsm_l11_smem<T>(A, lda, j0, ib, j0 + ib, n, sT, 64);
                T *sL = sT, *sU = sT + PANEL_NB * 64;
                if (tile == VB_TILE_32x32)
                    vb_update<T, 32, 32, 2, 2>(A, lda, m, n, j0, ib, sL, sU);
                else if (tile == VB_TILE_32x64)
                    vb_update<T, 32, 64, 2, 4>(A, lda, m, n, j0, ib, sL, sU);
                else
                    vb_update<T, 64, 64, 4, 4>(A, lda, m, n, j0, ib, sL, sU);
                __syncthreads();
            }
            j0 += ib;
        }
        if (tid == 0) info_array[k] = info;
        if (nrhs > 0 && m == n && n > 0) {
            for (int c0 = 0; c0 < nrhs; c0 += VB_NR) {
                const int nr = min(VB_NR, nrhs - c0);
                T *Bc = B + (size_t)c0 * ldb;
                __syncthreads();
                for (int e = tid; e < VB_NR * n; e += VB_THREADS) {
                    const int c = e / n, i = e % n;
                    sT[c * n + i] = c < nr ? Bc[i + (size_t)c * ldb] : T(0);
                }
                __syncthreads();
                solve_smem<T, false, VB_NR>(n, A, lda, nullptr, sT, nr);
                for (int e = tid; e < nr * n; e += VB_THREADS) {
                    const int c = e / n, i = e % n;
                    Bc[i + (size_t)c * ldb] = sT[c * n + i];
                }
            }
        }
    }
}

// Solve with existing factors, one CTA per (matrix, group of VB_NR columns).
template <typename T, bool TRANS>
__global__ void __launch_bounds__(VB_THREADS)
vb_getrs_kernel(const int *n_arr, const int *nrhs_arr, T **dA_array, const int *ldda_arr,
                int **ipiv_array, T **dB_array, const int *lddb_arr)
{
    extern __shared__ __align__(16) unsigned char smem[];
    T *sB = reinterpret_cast<T *>(smem);
    const int k = blockIdx.y, tid = threadIdx.x;
    const int n = n_arr[k], nrhs = nrhs_arr[k];
    const int c0 = blockIdx.x * VB_NR;
    if (n <= 0 || c0 >= nrhs) return;
    const int nr = min(VB_NR, nrhs - c0);
    const int ldb = lddb_arr[k];
    T *B = dB_array[k] + (size_t)c0 * ldb;
    for (int e = tid; e < VB_NR * n; e += VB_THREADS) {
        const int c = e / n, i = e % n;
        sB[c * n + i] = c < nr ? B[i + (size_t)c * ldb] : T(0);
    }
    __syncthreads();
    solve_smem<T, TRANS, VB_NR>(n, dA_array[k], ldda_arr[k], ipiv_array[k], sB, nr);
    for (int e = tid; e < nr * n; e += VB_THREADS) {
        const int c = e / n, i = e % n;
        B[i + (size_t)c * ldb] = sB[c * n + i];
    }
}

// argument check + maxima, one small kernel: stats = {err_m, err_n, err_ldda, err_lddb,
// max_m, max_n, max_nrhs, err_nrhs}
__global__ void vb_check_kernel(const int *m, const int *n, const int *nrhs, const int *ldda,
                                const int *lddb, int batch, int *stats)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= batch) return;
    const int mk = m[k], nk = n[k], rk = nrhs ? nrhs[k] : 0;
    if (mk < 0) stats[0] = 1;
    if (nk < 0) stats[1] = 1;
    if (rk < 0) stats[7] = 1;
    if (ldda[k] < max(1, mk)) stats[2] = 1;
    if (lddb && lddb[k] < max(1, nk)) stats[3] = 1;
    atomicMax(&stats[4], mk);
    atomicMax(&stats[5], nk);
    atomicMax(&stats[6], rk);
}

template <typename T>
size_t vb_smem_bytes(int max_m, int max_n, int max_nrhs)
{
    size_t need = 0;
    const int pm = max(max_m, 1);
    if (pm > VB_THREADS)   // shorter panels live in registers
        need = max(need, panel_smem_bytes<T>(pm, min(PANEL_NB, max(min(max_m, max_n), 1))));
    if (max_m > 0 && max_n > 0) need = max(need, panel_regs_smem_bytes<T, 1>());
    need = max(need, (size_t)2 * PANEL_NB * (SWAP_W + 1) * sizeof(T));
    need = max(need, (size_t)(PANEL_NB + GEMM_LDU) * 64 * sizeof(T));
    if (max_nrhs > 0) need = max(need, (size_t)VB_NR * max_n * sizeof(T));
    return min(need, VB_SMEM_CAP);
}

size_t vb_work_bytes(int batch) { return ((size_t)batch * sizeof(int) + 16 + 255) & ~(size_t)255; }

template <typename T>
magma_int_t blocked_getrf_vbatched(const int *m, const int *n, const int *ld, int max_m,
                                   int max_n, T **dA, int **ipiv, int *info, int batch,
                                   magma_queue_t q);
template <typename T>
magma_int_t vb_getrs_run(bool trans, const int *n, const int *nrhs, int max_n, int max_nrhs, T **dA,
                         const int *ldda, int **ipiv, T **dB, const int *lddb, int batch,
                         magma_queue_t q);

// Tuning tables in use (one per precision), set by magma_?vbatched_tuning_set
// or the autotuner.  Defaults: the autotuner's choices on GB300.
static std::mutex g_tune_mu;
static VbTune g_tune[2] = {
    {{32, 32, 32, 32, 32, 32, 32, 32}, {0, 0, 0, 0, 0, 0, 0, 0}},   // double
    {{32, 32, 32, 32, 32, 32, 32, 32}, {0, 0, 0, 0, 0, 0, 0, 0}},   // float
};
template <typename T> inline int tune_index() { return sizeof(T) == 8 ? 0 : 1; }
template <typename T> static VbTune current_tune()
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune[tune_index<T>()];
}

template <typename T>
magma_int_t vb_run(const int *m, const int *n, const int *nrhs, int max_m, int max_n, int max_nrhs,
                   T **dA, const int *ldda, int **ipiv, T **dB, const int *lddb, int *info,
                   void *work, int batch, magma_queue_t q, const VbTune *tune_override = nullptr)
{
    const VbTune tune = tune_override ? *tune_override : current_tune<T>();
    if (batch <= 0) return 0;
    if (max(max_m, max_n) > VB_PERSISTENT_MAX) {
        // large matrices: the per-step kernels, several CTAs per matrix
        magma_int_t rc = blocked_getrf_vbatched<T>(m, n, ldda, max_m, max_n, dA, ipiv, info,
                                                   batch, q);
        if (rc == 0 && max_nrhs > 0)
            rc = vb_getrs_run<T>(false, n, nrhs, max_n, max_nrhs, dA, ldda, ipiv, dB, lddb, batch, q);
        return rc;
    }
    static size_t dyn_cache[MLU_MAX_DEVICES];
    const size_t dyn_max = mlu_device_cached(dyn_cache, [] { return mlu_allow_dynamic_smem(vb_lu_kernel<T>); });
    const size_t smem = min(vb_smem_bytes<T>(max_m, max_n, max_nrhs), dyn_max);
    // the panel of the largest matrix must fit with at least width 1
    if (max_m > VB_THREADS && panel_smem_bytes<T>(max_m, 1) > smem)
        return MAGMA_ERR_NOT_SUPPORTED;
    if ((size_t)(PANEL_NB + GEMM_LDU) * 64 * sizeof(T) > smem) return MAGMA_ERR_NOT_SUPPORTED;
    if (max_m > 0 && max_n > 0 && panel_regs_smem_bytes<T, 1>() > smem) return MAGMA_ERR_NOT_SUPPORTED;
    if (max_nrhs > 0 && (size_t)VB_NR * max_n * sizeof(T) > smem) return MAGMA_ERR_NOT_SUPPORTED;
    int *order = (int *)work;
    int *counter = (int *)((char *)work + vb_work_bytes(batch) - 16);
    MLU_LAUNCH(mlu::KC_OTHER, q->stream, vb_sort_kernel<<<1, 1024, 0, q->stream>>>(m, n, batch, order, counter));
    int dev = q->device, sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vb_lu_kernel<T>, VB_THREADS, smem);
    const int grid = max(1, min(batch, sms * max(per_sm, 1)));
    MLU_LAUNCH(mlu::KC_VB_LU, q->stream, vb_lu_kernel<T><<<grid, VB_THREADS, smem, q->stream>>>(m, n, nrhs, dA, ldda, ipiv, dB, lddb, info,
                                                          order, counter, batch, (int)smem, tune));
    MLU_CHECK_LAUNCH();
    return 0;
}

template magma_int_t vb_run<double>(const int *, const int *, const int *, int, int, int, double **,
                                    const int *, int **, double **, const int *, int *, void *,
                                    int, magma_queue_t, const VbTune *);
template magma_int_t vb_run<float>(const int *, const int *, const int *, int, int, int, float **,
                                   const int *, int **, float **, const int *, int *, void *, int,
                                   magma_queue_t, const VbTune *);

template <typename T>
magma_int_t vb_getrs_run(bool trans, const int *n, const int *nrhs, int max_n, int max_nrhs, T **dA,
                         const int *ldda, int **ipiv, T **dB, const int *lddb, int batch,
                         magma_queue_t q)
{
    if (batch <= 0 || max_n <= 0 || max_nrhs <= 0) return 0;
    const size_t smem = (size_t)VB_NR * max_n * sizeof(T);
    if (smem > VB_SMEM_CAP) return MAGMA_ERR_NOT_SUPPORTED;
    static size_t dyn_cache[2][MLU_MAX_DEVICES];
    const size_t dyn_max = trans ? mlu_device_cached(dyn_cache[1], [] { return mlu_allow_dynamic_smem(vb_getrs_kernel<T, true>); })
                                 : mlu_device_cached(dyn_cache[0], [] { return mlu_allow_dynamic_smem(vb_getrs_kernel<T, false>); });
    if (smem > dyn_max) return MAGMA_ERR_NOT_SUPPORTED;
    for (int b0 = 0; b0 < batch; b0 += MLU_MAX_GRID_Y) {
        const int nb = min(batch - b0, (int)MLU_MAX_GRID_Y);
        dim3 grid((max_nrhs + VB_NR - 1) / VB_NR, nb);
        if (trans)
            MLU_LAUNCH(mlu::KC_GETRS, q->stream, vb_getrs_kernel<T, true><<<grid, VB_THREADS, smem, q->stream>>>(
                n + b0, nrhs + b0, dA + b0, ldda + b0, ipiv + b0, dB + b0, lddb + b0));
        else
            MLU_LAUNCH(mlu::KC_GETRS, q->stream, vb_getrs_kernel<T, false><<<grid, VB_THREADS, smem, q->stream>>>(
                n + b0, nrhs + b0, dA + b0, ldda + b0, ipiv + b0, dB + b0, lddb + b0));
    }
    MLU_CHECK_LAUNCH();
    return 0;
}

template magma_int_t vb_getrs_run<double>(bool, const int *, const int *, int, int, double **,
                                          const int *, int **, double **, const int *, int,
                                          magma_queue_t);

// Synchronous argument check and maxima (the reference's checker + setup,
// magmablas/vbatched_check.cu:39-58, magmablas/vbatched_aux.cu:27-87).
static magma_int_t vb_check(const int *m, const int *n, const int *nrhs, const int *ldda,
                            const int *lddb, int batch, magma_queue_t q, int out[8])
{
    for (int i = 0; i < 8; i++) out[i] = 0;
    if (batch <= 0) return 0;
    int *stats = nullptr;
    if (q->work_bytes < 64) {
        if (q->work) { cudaStreamSynchronize(q->stream); cudaFree(q->work); }
        q->work = nullptr;
        q->work_bytes = 0;
        if (mlu::device_malloc(&q->work, 64) != cudaSuccess) return MAGMA_ERR_DEVICE_ALLOC;
        q->work_bytes = 64;
    }
    stats = (int *)q->work;
    cudaMemsetAsync(stats, 0, 8 * sizeof(int), q->stream);
    MLU_LAUNCH(mlu::KC_OTHER, q->stream, vb_check_kernel<<<(batch + 255) / 256, 256, 0, q->stream>>>(m, n, nrhs, ldda, lddb, batch, stats));
    cudaMemcpyAsync(out, stats, 8 * sizeof(int), cudaMemcpyDeviceToHost, q->stream);
    if (cudaStreamSynchronize(q->stream) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    return 0;
}

// Workspace for vb_run owned by the queue (placed after the 64-byte stats area).
static void *vb_queue_work(magma_queue_t q, int batch)
{
    const size_t need = 256 + vb_work_bytes(batch);
    if (q->work_bytes < need) {
        if (q->work) { cudaStreamSynchronize(q->stream); cudaFree(q->work); }
        q->work = nullptr;
        q->work_bytes = 0;
        if (mlu::device_malloc(&q->work, need) != cudaSuccess) return nullptr;
        q->work_bytes = need;
    }
    return (char *)q->work + 256;
}

}  // namespace mlu

using namespace mlu;

// ---------------------------------------------------------------------------
// getrf

template <typename T>
static magma_int_t getrf_vbatched(const char *name, magma_int_t *m, magma_int_t *n, T **dA_array,
                                  magma_int_t *ldda, magma_int_t **ipiv_array,
                                  magma_int_t *info_array, magma_int_t batchCount,
                                  magma_queue_t queue)
{
    int st[8];
    magma_int_t rc = vb_check(m, n, nullptr, ldda, nullptr, batchCount, queue, st);
    if (rc != 0) return rc;
    magma_int_t arginfo = st[0] ? -1 : st[1] ? -2 : st[2] ? -4 : 0;
    if (arginfo != 0) {
        magma_xerbla(name, -arginfo);
        return arginfo;
    }
    if (batchCount <= 0) return 0;
    void *work = vb_queue_work(queue, batchCount);
    if (!work) return MAGMA_ERR_DEVICE_ALLOC;
    return vb_run<T>(m, n, nullptr, st[4], st[5], 0, dA_array, ldda, ipiv_array, nullptr, nullptr,
                     info_array, work, batchCount, queue);
}

extern "C" magma_int_t magma_dgetrf_vbatched(magma_int_t *m, magma_int_t *n, double **dA_array,
                                             magma_int_t *ldda, magma_int_t **ipiv_array,
                                             magma_int_t *info_array, magma_int_t batchCount,
                                             magma_queue_t queue)
{
    return getrf_vbatched<double>(__func__, m, n, dA_array, ldda, ipiv_array, info_array,
                                  batchCount, queue);
}

extern "C" magma_int_t magma_sgetrf_vbatched(magma_int_t *m, magma_int_t *n, float **dA_array,
                                             magma_int_t *ldda, magma_int_t **ipiv_array,
                                             magma_int_t *info_array, magma_int_t batchCount,
                                             magma_queue_t queue)
{
    return getrf_vbatched<float>(__func__, m, n, dA_array, ldda, ipiv_array, info_array,
                                 batchCount, queue);
}

extern "C" magma_int_t
magma_dgetrf_vbatched_max_nocheck_work(magma_int_t *m, magma_int_t *n, magma_int_t max_m,
                                       magma_int_t max_n, magma_int_t max_minmn,
                                       magma_int_t max_mxn, double **dA_array, magma_int_t *ldda,
                                       magma_int_t **dipiv_array, magma_int_t *info_array,
                                       void *work, magma_int_t *lwork, magma_int_t batchCount,
                                       magma_queue_t queue)
{
    (void)max_minmn;
    (void)max_mxn;
    const size_t need = vb_work_bytes(mlu_max(batchCount, 0));
    if (*lwork < 0) {
        *lwork = (magma_int_t)need;
        return 0;
    }
    if ((size_t)*lwork < need) return -12;
    return vb_run<double>(m, n, nullptr, max_m, max_n, 0, dA_array, ldda, dipiv_array, nullptr,
                          nullptr, info_array, work, batchCount, queue);
}

// ---------------------------------------------------------------------------
// gesv / getrs (no counterpart in the reference)

template <typename T>
static magma_int_t gesv_vbatched(const char *name, magma_int_t *n, magma_int_t *nrhs, T **dA_array,
                                 magma_int_t *ldda, magma_int_t **dipiv_array, T **dB_array,
                                 magma_int_t *lddb, magma_int_t *dinfo_array,
                                 magma_int_t batchCount, magma_queue_t queue)
{
    int st[8];
    magma_int_t rc = vb_check(n, n, nrhs, ldda, lddb, batchCount, queue, st);
    if (rc != 0) return rc;
    magma_int_t arginfo = st[1] ? -1 : st[7] ? -2 : st[2] ? -4 : st[3] ? -7 : 0;
    if (arginfo != 0) {
        magma_xerbla(name, -arginfo);
        return arginfo;
    }
    if (batchCount <= 0) return 0;
    void *work = vb_queue_work(queue, batchCount);
    if (!work) return MAGMA_ERR_DEVICE_ALLOC;
    return vb_run<T>(n, n, nrhs, st[5], st[5], st[6], dA_array, ldda, dipiv_array, dB_array, lddb,
                     dinfo_array, work, batchCount, queue);
}

extern "C" magma_int_t magma_dgesv_vbatched(magma_int_t *n, magma_int_t *nrhs, double **dA_array,
                                            magma_int_t *ldda, magma_int_t **dipiv_array,
                                            double **dB_array, magma_int_t *lddb,
                                            magma_int_t *dinfo_array, magma_int_t batchCount,
                                            magma_queue_t queue)
{
    return gesv_vbatched<double>(__func__, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                 dinfo_array, batchCount, queue);
}

extern "C" magma_int_t magma_sgesv_vbatched(magma_int_t *n, magma_int_t *nrhs, float **dA_array,
                                            magma_int_t *ldda, magma_int_t **dipiv_array,
                                            float **dB_array, magma_int_t *lddb,
                                            magma_int_t *dinfo_array, magma_int_t batchCount,
                                            magma_queue_t queue)
{
    return gesv_vbatched<float>(__func__, n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                dinfo_array, batchCount, queue);
}

extern "C" magma_int_t
magma_dgesv_vbatched_max_nocheck_work(magma_int_t *n, magma_int_t *nrhs, magma_int_t max_n,
                                      magma_int_t max_nrhs, double **dA_array, magma_int_t *ldda,
                                      magma_int_t **dipiv_array, double **dB_array,
                                      magma_int_t *lddb, magma_int_t *dinfo_array, void *work,
                                      magma_int_t *lwork, magma_int_t batchCount,
                                      magma_queue_t queue)
{
    const size_t need = vb_work_bytes(mlu_max(batchCount, 0));
    if (*lwork < 0) {
        *lwork = (magma_int_t)need;
        return 0;
    }
    if ((size_t)*lwork < need) return -12;
    return vb_run<double>(n, n, nrhs, max_n, max_n, max_nrhs, dA_array, ldda, dipiv_array,
                          dB_array, lddb, dinfo_array, work, batchCount, queue);
}

template <typename T>
static magma_int_t getrs_vbatched(const char *name, magma_trans_t trans, magma_int_t *n,
                                  magma_int_t *nrhs, T **dA_array, magma_int_t *ldda,
                                  magma_int_t **dipiv_array, T **dB_array, magma_int_t *lddb,
                                  magma_int_t batchCount, magma_queue_t queue)
{
    if (trans != MagmaNoTrans && trans != MagmaTrans && trans != MagmaConjTrans) {
        magma_xerbla(name, 1);
        return -1;
    }
    int st[8];
    magma_int_t rc = vb_check(n, n, nrhs, ldda, lddb, batchCount, queue, st);
    if (rc != 0) return rc;
    magma_int_t arginfo = st[1] ? -2 : st[7] ? -3 : st[2] ? -5 : st[3] ? -8 : 0;
    if (arginfo != 0) {
        magma_xerbla(name, -arginfo);
        return arginfo;
    }
    return vb_getrs_run<T>(trans != MagmaNoTrans, n, nrhs, st[5], st[6], dA_array, ldda, dipiv_array,
                           dB_array, lddb, batchCount, queue);
}

extern "C" magma_int_t magma_dgetrs_vbatched(magma_trans_t trans, magma_int_t *n,
                                             magma_int_t *nrhs, double **dA_array,
                                             magma_int_t *ldda, magma_int_t **dipiv_array,
                                             double **dB_array, magma_int_t *lddb,
                                             magma_int_t batchCount, magma_queue_t queue)
{
    return getrs_vbatched<double>(__func__, trans, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                  lddb, batchCount, queue);
}

extern "C" magma_int_t magma_sgetrs_vbatched(magma_trans_t trans, magma_int_t *n,
                                             magma_int_t *nrhs, float **dA_array,
                                             magma_int_t *ldda, magma_int_t **dipiv_array,
                                             float **dB_array, magma_int_t *lddb,
                                             magma_int_t batchCount, magma_queue_t queue)
{
    return getrs_vbatched<float>(__func__, trans, n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                 lddb, batchCount, queue);
}

// ---------------------------------------------------------------------------
// Tuning of the persistent kernel (no counterpart in the reference, whose
// batched tuning is a set of fixed crossover tables,
// control/get_batched_crossover.cpp:300-342, 918-928).

namespace mlu {

// uniform(-1, 1) entries from a counter-based hash (splitmix64) for the
// autotuner's trial batches
template <typename T>
__global__ void vb_fill_kernel(T *buf, size_t count, unsigned long long seed)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        unsigned long long x = seed + i * 0x9e3779b97f4a7c15ull;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
        x ^= x >> 31;
        buf[i] = (T)((double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0);
    }
}

// pointer and size arrays of a uniform trial batch of k matrices of order n
template <typename T>
__global__ void vb_trial_arrays_kernel(int k, int n, T *A, int *P, T **dA, int **dP, int *dn,
                                       int *dld)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    dA[i] = A + (size_t)i * n * n;
    dP[i] = P + (size_t)i * n;
    dn[i] = n;
    dld[i] = n;
}

static const int VB_TUNE_NB[] = {16, 32};
constexpr int VB_TUNE_MAX_N = VB_PERSISTENT_MAX;   // larger bins do not use the table

template <typename T>
static magma_int_t vb_autotune(int max_n, magma_queue_t q, VbTune *out)
{
    VbTune t = current_tune<T>();
    cudaStream_t s = q->stream;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, q->device);
    magma_int_t rc = MAGMA_SUCCESS;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        return MAGMA_ERR_UNKNOWN;
    }
    int ub = 16;
    for (int b = 0; b < VB_TUNE_BINS && rc == MAGMA_SUCCESS; b++, ub <<= 1) {
        const int lo = b == 0 ? 1 : ub / 2 + 1;
        if (lo > max_n || lo > VB_TUNE_MAX_N) break;
        // representative order: three quarters of the bin's upper bound
        const int n = max(lo, min(min(max_n, VB_TUNE_MAX_N), 3 * ub / 4));
        const size_t smem = vb_smem_bytes<T>(n, n, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vb_lu_kernel<T>, VB_THREADS, smem);
        const double flops = 2.0 / 3.0 * n * (double)n * n;
        const int resident = sms * max(per_sm, 1);
        // enough matrices to keep every resident CTA busy several times over,
        // about 2 GFLOP per trial, at most 4096
        const int k = max(2 * resident, min(4096, (int)(2e9 / flops)));
        T *A = nullptr, **dA = nullptr;
        int *P = nullptr, **dP = nullptr, *dn = nullptr, *dld = nullptr, *info = nullptr;
        void *work = nullptr;
        const size_t wb = vb_work_bytes(k);
        if (mlu::device_malloc((void **)&A, (size_t)k * n * n * sizeof(T)) != cudaSuccess ||
            mlu::device_malloc((void **)&P, (size_t)k * n * sizeof(int)) != cudaSuccess ||
            mlu::device_malloc((void **)&dA, k * sizeof(T *)) != cudaSuccess ||
            mlu::device_malloc((void **)&dP, k * sizeof(int *)) != cudaSuccess ||
            mlu::device_malloc((void **)&dn, k * sizeof(int)) != cudaSuccess ||
            mlu::device_malloc((void **)&dld, k * sizeof(int)) != cudaSuccess ||
            mlu::device_malloc((void **)&info, k * sizeof(int)) != cudaSuccess ||
            mlu::device_malloc(&work, wb) != cudaSuccess) {
            cudaGetLastError();
            rc = MAGMA_ERR_DEVICE_ALLOC;
        }
        if (rc == MAGMA_SUCCESS) {
            MLU_LAUNCH(mlu::KC_OTHER, s, vb_trial_arrays_kernel<T><<<(k + 255) / 256, 256, 0, s>>>(
                k, n, A, P, dA, dP, dn, dld));
            float best = -1.f;
            int best_nb = t.nb[b], best_tile = t.tile[b];
            for (int nbw : VB_TUNE_NB) {
                for (int tile = 0; tile < VB_TILE_COUNT && rc == MAGMA_SUCCESS; tile++) {
                    VbTune trial = t;
                    trial.nb[b] = (unsigned char)nbw;
                    trial.tile[b] = (unsigned char)tile;
                    float tmin = -1.f;
                    for (int rep = 0; rep < 2; rep++) {
                        MLU_LAUNCH(mlu::KC_OTHER, s, vb_fill_kernel<T><<<4 * sms, 256, 0, s>>>(
                            A, (size_t)k * n * n, 0x5eedull + 977ull * b));
                        cudaEventRecord(e0, s);
                        rc = vb_run<T>(dn, dn, nullptr, n, n, 0, dA, dld, dP, nullptr, nullptr,
                                       info, work, k, q, &trial);
                        cudaEventRecord(e1, s);
                        float ms = 0.f;
                        if (rc != MAGMA_SUCCESS || cudaEventSynchronize(e1) != cudaSuccess ||
                            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                            cudaGetLastError();
                            if (rc == MAGMA_SUCCESS) rc = MAGMA_ERR_UNKNOWN;
                            break;
                        }
                        if (tmin < 0.f || ms < tmin) tmin = ms;
                    }
                    if (rc == MAGMA_SUCCESS && (best < 0.f || tmin < best)) {
                        best = tmin;
                        best_nb = nbw;
                        best_tile = tile;
                    }
                }
            }
            t.nb[b] = (unsigned char)best_nb;
            t.tile[b] = (unsigned char)best_tile;
        }
        cudaFree(A); cudaFree(P); cudaFree(dA); cudaFree(dP); cudaFree(dn); cudaFree(dld);
        cudaFree(info); cudaFree(work);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != MAGMA_SUCCESS) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[tune_index<T>()] = t;
    }
    if (out) *out = t;
    return MAGMA_SUCCESS;
}

template <typename T>
static magma_int_t tuning_get(magma_int_t *nb, magma_int_t *tile)
{
    const VbTune t = current_tune<T>();
    for (int b = 0; b < VB_TUNE_BINS; b++) {
        if (nb) nb[b] = t.nb[b];
        if (tile) tile[b] = t.tile[b];
    }
    return MAGMA_SUCCESS;
}

template <typename T>
static magma_int_t tuning_set(const magma_int_t *nb, const magma_int_t *tile)
{
    if (nb == nullptr) return -1;
    if (tile == nullptr) return -2;
    VbTune t;
    for (int b = 0; b < VB_TUNE_BINS; b++) {
        if (nb[b] != 8 && nb[b] != 16 && nb[b] != 32) return -1;
        if (tile[b] < 0 || tile[b] >= VB_TILE_COUNT) return -2;
        t.nb[b] = (unsigned char)nb[b];
        t.tile[b] = (unsigned char)tile[b];
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_index<T>()] = t;
    return MAGMA_SUCCESS;
}

template <typename T>
static magma_int_t autotune_entry(magma_int_t max_n, magma_int_t *nb, magma_int_t *tile,
                                  magma_queue_t queue)
{
    if (max_n < 0) return -1;
    if (queue == nullptr) return -4;
    if (max_n == 0) return tuning_get<T>(nb, tile);
    VbTune t;
    const magma_int_t rc = vb_autotune<T>(max_n, queue, &t);
    if (rc != MAGMA_SUCCESS) return rc;
    return tuning_get<T>(nb, tile);
}

}  // namespace mlu

extern "C" magma_int_t magma_dgetrf_vbatched_autotune(magma_int_t max_n, magma_int_t *nb,
                                                      magma_int_t *tile, magma_queue_t queue)
{
    return mlu::autotune_entry<double>(max_n, nb, tile, queue);
}

extern "C" magma_int_t magma_sgetrf_vbatched_autotune(magma_int_t max_n, magma_int_t *nb,
                                                      magma_int_t *tile, magma_queue_t queue)
{
    return mlu::autotune_entry<float>(max_n, nb, tile, queue);
}

extern "C" magma_int_t magma_dvbatched_tuning_get(magma_int_t *nb, magma_int_t *tile)
{
    return mlu::tuning_get<double>(nb, tile);
}

extern "C" magma_int_t magma_svbatched_tuning_get(magma_int_t *nb, magma_int_t *tile)
{
    return mlu::tuning_get<float>(nb, tile);
}

extern "C" magma_int_t magma_dvbatched_tuning_set(const magma_int_t *nb, const magma_int_t *tile)
{
    return mlu::tuning_set<double>(nb, tile);
}

extern "C" magma_int_t magma_svbatched_tuning_set(const magma_int_t *nb, const magma_int_t *tile)
{
    return mlu::tuning_set<float>(nb, tile);
}
