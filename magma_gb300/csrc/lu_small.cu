// lu_small.cu -- warp-per-matrix LU factor / solve for n <= 32.
//
// Replaces, for one warp per matrix instead of one CTA per matrix:
//   magma_dgesv_batched_small           magmablas/zgesv_batched_small.cu:49-162,376-493
//   magma_dgetrf_batched_smallsq_noshfl magmablas/zgetrf_batched_smallsq_noshfl.cu:40-285
//   the n <= 32 part of magma_dgetrs_batched  src/zgetrs_batched.cpp:86-181
//
// Layout: lane i of the warp holds row i of the matrix (n values in
// registers) and row i of the right-hand sides.  Rows never move during the
// elimination ("lazy" interchange, as the reference kernels do); each lane
// tracks the row's position in LAPACK's current row order, which is what the
// pivot search breaks ties on and where the row is written at the end.
//
// Pivot search runs on the integer pipes: |a| as an unsigned 63-bit key,
// reduced with redux.sync on the two 32-bit halves, ties to the smallest
// current position.  NaN follows idamax's strict '>' scan: a NaN at the
// current diagonal position wins, any other NaN never does.
//
// GB300 note: FP64 issues at a small fraction of the FP32 rate on this part,
// so the kernel keeps everything except the eliminations themselves (pivot
// search, interchanges, broadcasts) off the FP64 pipe, and the U solve reuses
// the pivot reciprocals computed during the factorisation.
#include "common.cuh"
#include "trace.cuh"

namespace mlu {

constexpr int SMALL_WARPS = 4;   // matrices per CTA (solve kernel)
constexpr int GESV_WARPS = 8;    // matrices per CTA (factor kernel, lockstep)

// The factor kernel runs its GESV_WARPS warps in lockstep so that the pivot
// reciprocals of all of them come from one FP64 division sequence issued by
// warp 0 (one lane per matrix): on this part the FP64 pipe, not latency, is
// the limit, and a division costs as many FP64 issue slots whether one lane or
// thirty-two use it.
template <typename T, int N, int NRHS>
__global__ void __launch_bounds__(GESV_WARPS * 32, 2)
small_gesv_kernel(int n, int nrhs, T **dA_array, int ldda, int **ipiv_array, T **dB_array,
                  int lddb, int *info_array, int batch)
{
    __shared__ T s_piv[GESV_WARPS], s_rcp[GESV_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int mat = blockIdx.x * GESV_WARPS + warp;
    const bool live = mat < batch;   // dead warps still take part in the barriers

    T *A = live ? dA_array[mat] : nullptr;
    const bool row_valid = lane < n;

    T a[N];
#pragma unroll
    for (int j = 0; j < N; j++)
        a[j] = (live && row_valid && j < n) ? A[lane + (size_t)j * ldda] : T(0);

    constexpr int NB = NRHS > 0 ? NRHS : 1;
    T b[NB];
    T *B = nullptr;
    if (NRHS > 0) {
        B = live ? dB_array[mat] : nullptr;
#pragma unroll
        for (int c = 0; c < NB; c++)
            b[c] = (live && row_valid && c < nrhs) ? B[lane + (size_t)c * lddb] : T(0);
    }

    unsigned pos = lane;      // position in LAPACK's current row order
    bool active = row_valid;  // not yet chosen as a pivot row
    int info = 0;
    int my_ipiv = 0;
    T my_rcp = T(0);          // reciprocal of this row's pivot, once it is one

#pragma unroll
    for (int k = 0; k < N; k++) {
        if (k >= n) break;
        const T v = a[k];
        unsigned long long key = 0ull;
        if (active) {
            unsigned long long mag = Prec<T>::absbits(v);
            if (Prec<T>::isnan_(v)) mag = (pos == (unsigned)k) ? 0x7fffffffffffffffull : 0ull;
            key = mag | 0x8000000000000000ull;
        }
        const unsigned ppos = warp_argmax_key(key, active ? pos : 0xffffffffu);
        const int plane = __ffs(__ballot_sync(FULL, active && pos == ppos)) - 1;
        const T piv = shfl(v, plane);
        const bool nz = Prec<T>::nonzero(piv);
        if (!nz && info == 0) info = k + 1;
        if (lane == 0) s_piv[warp] = piv;
        __syncthreads();
        if (warp == 0 && lane < GESV_WARPS) s_rcp[lane] = T(1) / s_piv[lane];
        __syncthreads();
        const T r = s_rcp[warp];
        if (lane == k) my_ipiv = (int)ppos + 1;
        const bool was_k = (pos == (unsigned)k);
        if (lane == plane) { pos = k; active = false; my_rcp = r; }
        else if (was_k) pos = ppos;

        const T l = (active && nz) ? rscale(v, piv, r) : v;
        if (active) a[k] = l;
#pragma unroll
        for (int j = k + 1; j < N; j++) {
            if (j < n) {
                const T u = shfl(a[j], plane);
                if (active) a[j] = Prec<T>::fma_(-l, u, a[j]);
            }
        }
        if (NRHS > 0) {
#pragma unroll
            for (int c = 0; c < NB; c++) {
                if (c < nrhs) {
                    const T u = shfl(b[c], plane);
                    if (active) b[c] = Prec<T>::fma_(-l, u, b[c]);
                }
            }
        }
    }

    if (NRHS > 0) {
        // U x = y, column-oriented, multiplying by the stored pivot reciprocals.
#pragma unroll
        for (int t = N - 1; t >= 0; t--) {
            if (t >= n) continue;
            const int tl = __ffs(__ballot_sync(FULL, row_valid && pos == (unsigned)t)) - 1;
            const T d = shfl(a[t], tl);
            const T rr = shfl(my_rcp, tl);
#pragma unroll
            for (int c = 0; c < NB; c++) {
                if (c < nrhs) {
                    const T x = rscale(shfl(b[c], tl), d, rr);
                    if (lane == tl) b[c] = x;
                    else if (row_valid && pos < (unsigned)t) b[c] = Prec<T>::fma_(-a[t], x, b[c]);
                }
            }
        }
    }

    if (live && row_valid) {
#pragma unroll
        for (int j = 0; j < N; j++)
            if (j < n) A[pos + (size_t)j * ldda] = a[j];
        ipiv_array[mat][lane] = my_ipiv;
        if (NRHS > 0) {
#pragma unroll
            for (int c = 0; c < NB; c++)
                if (c < nrhs) B[pos + (size_t)c * lddb] = b[c];
        }
    }
    if (live && lane == 0) info_array[mat] = info;
}

// Packed variant for 16 < n <= 32: the matrix of each warp sits row-major in
// shared memory and rows are interchanged physically.  The pivot search and
// the column scaling are lane = row as above, but the rank-1 update of step k
// spreads the (n-1-k)^2 trailing elements over all 32 lanes (element e of the
// step: row k+1+e/w, column k+1+e%w, w = n-1-k), so no FP64 instruction runs
// with the lanes of finished rows idle: 344 warp FMAs for the update of a
// 32 x 32 matrix instead of 496.  Every element receives the same operations
// in the same order as in small_gesv_kernel.
constexpr int PK_LD = 33;

template <typename T>
__host__ __device__ constexpr size_t packed_warp_elems(int nb)
{
    return (size_t)32 * PK_LD + (size_t)32 * nb + 32;
}

template <typename T, int NRHS>
__global__ void __launch_bounds__(GESV_WARPS * 32)
small_gesv_packed_kernel(int n, int nrhs, T **dA_array, int ldda, int **ipiv_array, T **dB_array,
                         int lddb, int *info_array, int batch)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T s_piv[GESV_WARPS], s_rcp[GESV_WARPS];
    constexpr int NB = NRHS > 0 ? NRHS : 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int mat = blockIdx.x * GESV_WARPS + warp;
    const bool live = mat < batch;   // dead warps still take part in the barriers
    T *sA = reinterpret_cast<T *>(smem_raw) + (size_t)warp * packed_warp_elems<T>(NB);  // [32][PK_LD]
    T *sB = sA + 32 * PK_LD;                                                           // [32][NB]
    T *sR = sB + 32 * NB;                                                              // pivot reciprocals
    const bool row_valid = lane < n;
    T *A = live ? dA_array[mat] : nullptr;
#pragma unroll 8
    for (int j = 0; j < 32; j++)
        sA[lane * PK_LD + j] = (live && row_valid && j < n) ? A[lane + (size_t)j * ldda] : T(0);
    // one right-hand side lives in column 32 of sA (the row padding), so that its
    // update rides in the packed update of each step
    auto bref = [&](int row, int c) -> T & { return NRHS == 1 ? sA[row * PK_LD + 32] : sB[row * NB + c]; };
    T *B = nullptr;
    if (NRHS > 0) {
        B = live ? dB_array[mat] : nullptr;
#pragma unroll
        for (int c = 0; c < NB; c++)
            bref(lane, c) = (live && row_valid && c < nrhs) ? B[lane + (size_t)c * lddb] : T(0);
    }
    __syncwarp();
    int info = 0, my_ipiv = 0;
    for (int k = 0; k < n; k++) {
        const T v = sA[lane * PK_LD + k];
        const bool cand = lane >= k && row_valid;
        unsigned long long key = 0ull;
        if (cand) {
            unsigned long long mag = Prec<T>::absbits(v);
            if (Prec<T>::isnan_(v)) mag = (lane == k) ? 0x7fffffffffffffffull : 0ull;
            key = mag | 0x8000000000000000ull;
        }
        const int p = (int)warp_argmax_key(key, cand ? (unsigned)lane : 0xffffffffu);
        const T piv = shfl(v, p);
        const bool nz = Prec<T>::nonzero(piv);
        if (!nz && info == 0) info = k + 1;
        if (lane == k) my_ipiv = p + 1;
        if (p != k && MLU_BC2(p, 0, n, 1, 601)) {       // whole rows k and p, and the right-hand sides
            if (row_valid) {
                const T x = sA[k * PK_LD + lane];
                sA[k * PK_LD + lane] = sA[p * PK_LD + lane];
                sA[p * PK_LD + lane] = x;
            }
            if (NRHS > 0 && lane < NB) {
                const T x = bref(k, lane);
                bref(k, lane) = bref(p, lane);
                bref(p, lane) = x;
            }
        }
        if (lane == 0) s_piv[warp] = piv;
        __syncthreads();
        if (warp == 0 && lane < GESV_WARPS) s_rcp[lane] = T(1) / s_piv[lane];
        __syncthreads();
        const T r = s_rcp[warp];
        if (lane == 0) sR[k] = r;
        if (lane > k && row_valid && nz) sA[lane * PK_LD + k] = rscale(sA[lane * PK_LD + k], piv, r);
        __syncwarp();
        const int w = n - 1 - k;
        if (w > 0) {
            // rows k+1.. by columns k+1..n-1, and column 32 (b) with one right-hand side
            const int wc = NRHS == 1 ? w + 1 : w;
            const float inv = 1.0f / (float)wc;
            for (int e = lane; e < w * wc; e += 32) {
                int i = __float2int_rz((float)e * inv);
                int j = e - i * wc;
                if (j < 0) { i--; j += wc; } else if (j >= wc) { i++; j -= wc; }
                const int col = (NRHS == 1 && j == w) ? 32 : k + 1 + j;
                T *dst = sA + (k + 1 + i) * PK_LD + col;
                *dst = Prec<T>::fma_(-sA[(k + 1 + i) * PK_LD + k], sA[k * PK_LD + col], *dst);
            }
            if (NRHS > 1 && lane > k && row_valid) {
#pragma unroll
                for (int c = 0; c < NB; c++)
                    if (c < nrhs)
                        sB[lane * NB + c] = Prec<T>::fma_(-sA[lane * PK_LD + k], sB[k * NB + c], sB[lane * NB + c]);
            }
        }
        __syncwarp();
    }
    if (NRHS > 0) {
        // U x = y, lane = row, multiplying by the stored pivot reciprocals
        for (int t = n - 1; t >= 0; t--) {
            const T d = sA[t * PK_LD + t], rr = sR[t];
            T x[NB];
#pragma unroll
            for (int c = 0; c < NB; c++) x[c] = rscale(bref(t, c), d, rr);
            __syncwarp();
#pragma unroll
            for (int c = 0; c < NB; c++) {
                if (c < nrhs) {
                    if (lane == t) bref(t, c) = x[c];
                    else if (lane < t) bref(lane, c) = Prec<T>::fma_(-sA[lane * PK_LD + t], x[c], bref(lane, c));
                }
            }
            __syncwarp();
        }
    }
    if (live && row_valid) {
#pragma unroll 8
        for (int j = 0; j < 32; j++)
            if (j < n) A[lane + (size_t)j * ldda] = sA[lane * PK_LD + j];
        ipiv_array[mat][lane] = my_ipiv;
        if (NRHS > 0) {
#pragma unroll
            for (int c = 0; c < NB; c++)
                if (c < nrhs) B[lane + (size_t)c * lddb] = bref(lane, c);
        }
    }
    if (live && lane == 0) info_array[mat] = info;
}

// Solve with existing factors, n <= 32.  NoTrans: lane i holds row i of LU.
// Trans: lane i holds column i of LU, so that U(t,i) and L(t,i) are static
// register indices.  RHS columns [blockIdx.y*NRHS, +NRHS).
template <typename T, int N, int NRHS, bool TRANS>
__global__ void __launch_bounds__(SMALL_WARPS * 32)
small_getrs_kernel(int n, int nrhs, T **dA_array, int ldda, int **ipiv_array, T **dB_array,
                   int lddb, int batch)
{
    const int lane = threadIdx.x & 31;
    const int mat = blockIdx.x * SMALL_WARPS + (threadIdx.x >> 5);
    if (mat >= batch) return;
    const int c0 = blockIdx.y * NRHS;
    const T *A = dA_array[mat];
    const int *ipiv = ipiv_array[mat];
    T *B = dB_array[mat] + (size_t)c0 * lddb;
    const int nr = min(NRHS, nrhs - c0);
    const bool valid = lane < n;

    T a[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        if (TRANS) a[j] = (valid && j < n) ? A[j + (size_t)lane * ldda] : T(0);
        else       a[j] = (valid && j < n) ? A[lane + (size_t)j * ldda] : T(0);
    }
    T b[NRHS];
#pragma unroll
    for (int c = 0; c < NRHS; c++) b[c] = (valid && c < nr) ? B[lane + (size_t)c * lddb] : T(0);
    const int my_piv = valid ? ipiv[lane] - 1 : lane;

    if (!TRANS) {
        // B <- P B, sequential interchanges k = 0..n-1
#pragma unroll
        for (int k = 0; k < N; k++) {
            if (k >= n) break;
            const int p = shfl(my_piv, k);
            if (p != k) {
#pragma unroll
                for (int c = 0; c < NRHS; c++) {
                    const T vk = shfl(b[c], k), vp = shfl(b[c], p);
                    if (lane == k) b[c] = vp;
                    if (lane == p) b[c] = vk;
                }
            }
        }
        // L y = b (unit lower)
#pragma unroll
        for (int t = 0; t < N; t++) {
            if (t >= n) break;
#pragma unroll
            for (int c = 0; c < NRHS; c++) {
                const T y = shfl(b[c], t);
                if (lane > t) b[c] = Prec<T>::fma_(-a[t], y, b[c]);
            }
        }
        // U x = y
#pragma unroll
        for (int t = N - 1; t >= 0; t--) {
            if (t >= n) continue;
            const T d = shfl(a[t], t);
            const T r = T(1) / d;
#pragma unroll
            for (int c = 0; c < NRHS; c++) {
                const T x = rscale(shfl(b[c], t), d, r);
                if (lane == t) b[c] = x;
                else if (lane < t) b[c] = Prec<T>::fma_(-a[t], x, b[c]);
            }
        }
    } else {
        // U^T y = b: lane i holds column i, so a[t] = U(t,i) for t <= i.
#pragma unroll
        for (int t = 0; t < N; t++) {
            if (t >= n) break;
            const T d = shfl(a[t], t);
            const T r = T(1) / d;
#pragma unroll
            for (int c = 0; c < NRHS; c++) {
                const T x = rscale(shfl(b[c], t), d, r);
                if (lane == t) b[c] = x;
                else if (lane > t) b[c] = Prec<T>::fma_(-a[t], x, b[c]);
            }
        }
        // L^T x = y: a[t] = L(t,i) for t > i.
#pragma unroll
        for (int t = N - 1; t >= 0; t--) {
            if (t >= n) continue;
#pragma unroll
            for (int c = 0; c < NRHS; c++) {
                const T x = shfl(b[c], t);
                if (lane < t) b[c] = Prec<T>::fma_(-a[t], x, b[c]);
            }
        }
        // B <- P^T B, interchanges in reverse order
#pragma unroll
        for (int k = N - 1; k >= 0; k--) {
            if (k >= n) continue;
            const int p = shfl(my_piv, k);
            if (p != k) {
#pragma unroll
                for (int c = 0; c < NRHS; c++) {
                    const T vk = shfl(b[c], k), vp = shfl(b[c], p);
                    if (lane == k) b[c] = vp;
                    if (lane == p) b[c] = vk;
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NRHS; c++)
        if (valid && c < nr) B[lane + (size_t)c * lddb] = b[c];
}

template <typename T, int N, int NRHS>
static void launch_small_gesv(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb,
                              int *info, int batch, cudaStream_t s)
{
    if (N == 32) {   // 16 < n <= 32: the packed shared-memory kernel
        constexpr int NB = NRHS > 0 ? NRHS : 1;
        const size_t smem = (size_t)GESV_WARPS * packed_warp_elems<T>(NB) * sizeof(T);
        static size_t dyn_cache[MLU_MAX_DEVICES];
        const size_t dyn = mlu_device_cached(
            dyn_cache, [] { return mlu_allow_dynamic_smem(small_gesv_packed_kernel<T, NRHS>); });
        if (smem <= dyn) {
            MLU_LAUNCH(mlu::KC_SMALL_GESV, s, small_gesv_packed_kernel<T, NRHS><<<mlu_ceildiv(batch, GESV_WARPS), GESV_WARPS * 32, smem, s>>>(
                n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch));
            return;
        }
    }
    MLU_LAUNCH(mlu::KC_SMALL_GESV, s, small_gesv_kernel<T, N, NRHS><<<mlu_ceildiv(batch, GESV_WARPS), GESV_WARPS * 32, 0, s>>>(
        n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch));
}

template <typename T, int N>
static void dispatch_nrhs(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb,
                          int *info, int batch, cudaStream_t s)
{
    if (nrhs == 0)      launch_small_gesv<T, N, 0>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
    else if (nrhs == 1) launch_small_gesv<T, N, 1>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
    else if (nrhs <= 4) launch_small_gesv<T, N, 4>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
    else                launch_small_gesv<T, N, 16>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
}

// Fused factor (+ solve when nrhs > 0) for n <= 32, nrhs <= 16.
template <typename T>
magma_int_t small_gesv(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb, int *info,
                       int batch, magma_queue_t q)
{
    if (n > 32 || n < 1 || nrhs > 16) return MAGMA_ERR;   // -100: not applicable
    if (batch <= 0) return MAGMA_SUCCESS;
    cudaStream_t s = q->stream;
    if (n <= 8)       dispatch_nrhs<T, 8>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
    else if (n <= 16) dispatch_nrhs<T, 16>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
    else              dispatch_nrhs<T, 32>(n, nrhs, dA, ldda, ipiv, dB, lddb, info, batch, s);
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

template <typename T, int N, bool TRANS>
static void launch_small_getrs(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb,
                               int batch, cudaStream_t s)
{
    constexpr int NR = 4;
    dim3 grid(mlu_ceildiv(batch, SMALL_WARPS), mlu_ceildiv(nrhs, NR));
    MLU_LAUNCH(mlu::KC_GETRS, s, small_getrs_kernel<T, N, NR, TRANS><<<grid, SMALL_WARPS * 32, 0, s>>>(
        n, nrhs, dA, ldda, ipiv, dB, lddb, batch));
}

template <typename T>
magma_int_t small_getrs(bool trans, int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB,
                        int lddb, int batch, magma_queue_t q)
{
    if (n > 32) return MAGMA_ERR;
    if (batch <= 0 || n == 0 || nrhs == 0) return MAGMA_SUCCESS;
    cudaStream_t s = q->stream;
    if (trans) {
        if (n <= 8)       launch_small_getrs<T, 8, true>(n, nrhs, dA, ldda, ipiv, dB, lddb, batch, s);
        else if (n <= 16) launch_small_getrs<T, 16, true>(n, nrhs, dA, ldda, ipiv, dB, lddb, batch, s);
        else              launch_small_getrs<T, 32, true>(n, nrhs, dA, ldda, ipiv, dB, lddb, batch, s);
    } else {
        if (n <= 8)       launch_small_getrs<T, 8, false>(n, nrhs, dA, ldda, ipiv, dB, lddb, batch, s);
        else if (n <= 16) launch_small_getrs<T, 16, false>(n, nrhs, dA, ldda, ipiv, dB, lddb, batch, s);
        else              launch_small_getrs<T, 32, false>(n, nrhs, dA, ldda, ipiv, dB, lddb, batch, s);
    }
    MLU_CHECK_LAUNCH();
    return MAGMA_SUCCESS;
}

template magma_int_t small_gesv<double>(int, int, double **, int, int **, double **, int, int *, int, magma_queue_t);
template magma_int_t small_gesv<float>(int, int, float **, int, int **, float **, int, int *, int, magma_queue_t);
template magma_int_t small_getrs<double>(bool, int, int, double **, int, int **, double **, int, int, magma_queue_t);
template magma_int_t small_getrs<float>(bool, int, int, float **, int, int **, float **, int, int, magma_queue_t);

}  // namespace mlu
