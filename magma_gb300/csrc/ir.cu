// ir.cu -- batched mixed-precision iterative refinement.
//
// MAGMA has iterative refinement only for one matrix at a time
// (magma_dsgesv_gpu, src/zcgesv_gpu.cpp:144-366; magma_dhgesv_iteref_gpu,
// src/dxgesv_gmres_gpu.cpp:1122).  This file applies the same algorithm to a
// whole batch on the device, per matrix:
//   anrm = ||A||_inf, cte = anrm * eps * sqrt(n)           (zcgesv_gpu.cpp:208-209)
//   As = float(A) (overflow -> iter = -2), LU of As in FP32 (info > 0 -> iter = -3)
//   X = 0, R = B; repeat: X += float-solve(R); R = B - A X in FP64;
//   converged when, for every right-hand side c, ||R_c||_inf <= ||X_c||_inf * cte
//   (zcgesv_gpu.cpp:266-278), checked first after the initial solve (iter = 0)
//   and after each refinement; ITERMAX = 30 refinements, then iter = -31
//   (zcgesv_gpu.cpp:160-161, 345); failed matrices are re-solved in FP64 with
//   A overwritten by its FP64 factors (zcgesv_gpu.cpp:352-362).
// A second stopping rule is available: the scaled residual
// ||B - A X||_inf / (||A||_inf ||X||_inf n eps) <= tol (the reference tester's
// acceptance metric, testing/testing_zgesv_batched.cpp:131-152).
//
// Everything except the optional FP64 fallback runs without host
// synchronisation; converged matrices drop out of every later launch at the
// cost of one flag read.  The arithmetic is deterministic (fixed fma order in
// the FP64 residual, the oracle's order in the FP32 factor and solves), so the
// CPU oracle reproduces iterates and iteration counts exactly.
#include "common.cuh"
#include "solve_core.cuh"

namespace mlu {
template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q);
template <typename T>
magma_int_t small_gesv(int n, int nrhs, T **dA, int ldda, int **ipiv, T **dB, int lddb, int *info,
                       int batch, magma_queue_t q);
}  // namespace mlu

extern "C" magma_int_t magma_sgetrf_batched(magma_int_t m, magma_int_t n, float **dA_array,
                                            magma_int_t ldda, magma_int_t **ipiv_array,
                                            magma_int_t *info_array, magma_int_t batchCount,
                                            magma_queue_t queue);
extern "C" magma_int_t magma_dgesv_batched(magma_int_t n, magma_int_t nrhs, double **dA_array,
                                           magma_int_t ldda, magma_int_t **dipiv_array,
                                           double **dB_array, magma_int_t lddb,
                                           magma_int_t *dinfo_array, magma_int_t batchCount,
                                           magma_queue_t queue);

namespace mlu {

constexpr int IR_ROWS = 128;       // rows per CTA in the FP64 kernels
constexpr int IR_NRHS_MAX = 16;
constexpr int IR_SOLVE_NR = 8;
constexpr int IR_ACTIVE = 0, IR_CONVERGED = 1, IR_FAILED = 2;

// per-matrix statistics block (8-byte words)
//   [0] anorm bits  [1] state  [2 + par*(2*NRMAX+2) + ...] norms for parity par:
//   rcol[NRMAX], xcol[NRMAX], rrow, xrow
constexpr int IR_STATS_WORDS = 2 + 2 * (2 * IR_NRHS_MAX + 2);

__device__ __forceinline__ unsigned long long dbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ unsigned long long *norms_of(unsigned long long *st, int par) {
    return st + 2 + par * (2 * IR_NRHS_MAX + 2);
}

// Warp max of a non-negative double, then one atomicMax per warp.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v) {
    unsigned long long b = dbits(v);
    unsigned hi = __reduce_max_sync(FULL, (unsigned)(b >> 32));
    unsigned lo = __reduce_max_sync(FULL, ((unsigned)(b >> 32) == hi) ? (unsigned)b : 0u);
    if ((threadIdx.x & 31) == 0) atomicMax(addr, ((unsigned long long)hi << 32) | lo);
}

// As = float(A), ||A||_inf, R = B, X = 0.
__global__ void __launch_bounds__(IR_ROWS)
ir_init_kernel(int n, int nrhs, double **dA_array, int ldda, float **dAs_array, int ldas,
               double **dB_array, int lddb, double **dX_array, int lddx, double *R,
               unsigned long long *stats, int *iter)
{
    const int mat = blockIdx.y;
    const int i = blockIdx.x * IR_ROWS + threadIdx.x;
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    const double *A = dA_array[mat];
    float *As = dAs_array[mat];
    double rs = 0.0;
    bool ovf = false;
    if (i < n) {
        for (int j = 0; j < n; j++) {
            const double a = A[i + (size_t)j * ldda];
            rs += fabs(a);
            const float f = __double2float_rn(a);
            ovf |= (isinf(f) && !isinf(a));
            As[i + (size_t)j * ldas] = f;
        }
        const double *B = dB_array[mat];
        double *X = dX_array[mat];
        double *Rm = R + (size_t)mat * nrhs * n;
        for (int c = 0; c < nrhs; c++) {
            Rm[i + (size_t)c * n] = B[i + (size_t)c * lddb];
            X[i + (size_t)c * lddx] = 0.0;
        }
    }
    atomic_max_nonneg(&st[0], i < n ? rs : 0.0);
    if (__any_sync(FULL, ovf) && (threadIdx.x & 31) == 0) {
        st[1] = IR_FAILED;
        iter[mat] = -2;
    }
}

// Convergence test on the norms of parity `par`; called by one thread.
__device__ __forceinline__ bool ir_converged(const unsigned long long *st, int par, int n, int nrhs,
                                             double tol)
{
    const unsigned long long *nm = norms_of(const_cast<unsigned long long *>(st), par);
    const double anrm = bitsd(st[0]);
    const double eps = 1.1102230246251565e-16;   // LAPACK dlamch('Epsilon') = 2^-53
    if (tol > 0.0) {
        // scaled residual ||R||_inf / (||A||_inf ||X||_inf n eps) <= tol
        const double rr = bitsd(nm[2 * IR_NRHS_MAX]), xr = bitsd(nm[2 * IR_NRHS_MAX + 1]);
        return rr <= tol * (anrm * xr * (double)n * eps);
    }
    const double cte = anrm * eps * sqrt((double)n);
    for (int c = 0; c < nrhs; c++) {
        const double rc = bitsd(nm[c]), xc = bitsd(nm[IR_NRHS_MAX + c]);
        if (!(rc <= xc * cte)) return false;
    }
    return true;
}

// check (when it >= 0) + correction solve X += float-solve(R) with the FP32
// factors.  One CTA per (matrix, group of IR_SOLVE_NR right-hand sides).
__global__ void __launch_bounds__(256)
ir_solve_kernel(int n, int nrhs, float **dAs_array, int ldas, int **ipiv_array,
                double **dX_array, int lddx, const double *R, unsigned long long *stats,
                int *iter, const int *info, int it, double tol)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sB = reinterpret_cast<float *>(smem_raw);
    __shared__ int s_go;
    const int mat = blockIdx.y, tid = threadIdx.x;
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (tid == 0) {
        int go = st[1] == IR_ACTIVE;
        if (go && it < 0 && info[mat] > 0) {          // FP32 factorisation hit a zero pivot
            go = 0;
            if (blockIdx.x == 0) { st[1] = IR_FAILED; iter[mat] = -3; }
        }
        if (go && it >= 0 && ir_converged(st, it & 1, n, nrhs, tol)) {
            go = 0;
            if (blockIdx.x == 0) { st[1] = IR_CONVERGED; iter[mat] = it; }
        }
        s_go = go;
    }
    __syncthreads();
    if (!s_go) return;
    // clear the norms the next residual accumulates into
    if (blockIdx.x == 0) {
        unsigned long long *nx = norms_of(st, (it + 1) & 1);
        for (int e = tid; e < 2 * IR_NRHS_MAX + 2; e += blockDim.x) nx[e] = 0ull;
    }
    const int c0 = blockIdx.x * IR_SOLVE_NR;
    const int nr = min(IR_SOLVE_NR, nrhs - c0);
    const double *Rm = R + ((size_t)mat * nrhs + c0) * n;
    for (int e = tid; e < IR_SOLVE_NR * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        sB[c * n + i] = c < nr ? __double2float_rn(Rm[i + (size_t)c * n]) : 0.f;
    }
    __syncthreads();
    solve_smem<float, false, IR_SOLVE_NR>(n, dAs_array[mat], ldas, ipiv_array[mat], sB, nr);
    double *X = dX_array[mat] + (size_t)c0 * lddx;
    for (int e = tid; e < nr * n; e += blockDim.x) {
        const int c = e / n, i = e % n;
        X[i + (size_t)c * lddx] = X[i + (size_t)c * lddx] + (double)sB[c * n + i];
    }
}

// R = B - A X in FP64 (acc = b_i, then acc = fma(-a_ij, x_j, acc) for j = 0..n-1),
// with the column and row-sum infinity norms of R and X.
template <int NR>
__global__ void __launch_bounds__(IR_ROWS)
ir_residual_kernel(int n, int nrhs, double **dA_array, int ldda, double **dB_array, int lddb,
                   double **dX_array, int lddx, double *R, unsigned long long *stats, int par)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sX = reinterpret_cast<double *>(smem_raw);   // [n][NR]
    const int mat = blockIdx.y, tid = threadIdx.x;
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (st[1] != IR_ACTIVE) return;
    const double *X = dX_array[mat];
    for (int e = tid; e < n * NR; e += IR_ROWS) {
        const int j = e / NR, c = e % NR;
        sX[e] = c < nrhs ? X[j + (size_t)c * lddx] : 0.0;
    }
    __syncthreads();
    const int i = blockIdx.x * IR_ROWS + tid;
    double acc[NR];
    const double *A = dA_array[mat];
    const double *B = dB_array[mat];
    if (i < n) {
#pragma unroll
        for (int c = 0; c < NR; c++) acc[c] = c < nrhs ? B[i + (size_t)c * lddb] : 0.0;
        const double *Ai = A + i;
        for (int j = 0; j < n; j++) {
            const double a = Ai[(size_t)j * ldda];
#pragma unroll
            for (int c = 0; c < NR; c++) acc[c] = fma(-a, sX[j * NR + c], acc[c]);
        }
        double *Rm = R + (size_t)mat * nrhs * n;
#pragma unroll
        for (int c = 0; c < NR; c++) if (c < nrhs) Rm[i + (size_t)c * n] = acc[c];
    } else {
#pragma unroll
        for (int c = 0; c < NR; c++) acc[c] = 0.0;
    }
    unsigned long long *nm = norms_of(st, par);
    double rrow = 0.0, xrow = 0.0;
#pragma unroll
    for (int c = 0; c < NR; c++) {
        const double xa = i < n ? fabs(sX[i * NR + c]) : 0.0;
        const double ra = fabs(acc[c]);
        rrow += ra;
        xrow += xa;
        if (c < nrhs) {
            atomic_max_nonneg(&nm[c], ra);
            atomic_max_nonneg(&nm[IR_NRHS_MAX + c], xa);
        }
    }
    atomic_max_nonneg(&nm[2 * IR_NRHS_MAX], rrow);
    atomic_max_nonneg(&nm[2 * IR_NRHS_MAX + 1], xrow);
}

__global__ void ir_final_kernel(int n, int nrhs, unsigned long long *stats, int *iter, int itermax,
                                double tol, int batch, int *failed_count)
{
    const int mat = blockIdx.x * blockDim.x + threadIdx.x;
    if (mat >= batch) return;
    unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (st[1] == IR_ACTIVE) {
        if (ir_converged(st, itermax & 1, n, nrhs, tol)) {
            st[1] = IR_CONVERGED;
            iter[mat] = itermax;
        } else {
            st[1] = IR_FAILED;
            iter[mat] = -itermax - 1;
        }
    }
    if (st[1] == IR_FAILED) atomicAdd(failed_count, 1);
}

// Gathers the failed matrices into compact pointer arrays and restarts their
// X from B for the FP64 re-solve.
__global__ void ir_compact_kernel(int n, int nrhs, double **dA_array, int **ipiv_array,
                                  double **dB_array, int lddb, double **dX_array, int lddx,
                                  const unsigned long long *stats, int batch, int *counter,
                                  double **cA, int **cP, double **cX, int *cidx)
{
    const int mat = blockIdx.x;
    const unsigned long long *st = stats + (size_t)mat * IR_STATS_WORDS;
    if (st[1] != IR_FAILED) return;
    __shared__ int slot;
    if (threadIdx.x == 0) {
        slot = atomicAdd(counter, 1);
        cA[slot] = dA_array[mat];
        cP[slot] = ipiv_array[mat];
        cX[slot] = dX_array[mat];
        cidx[slot] = mat;
    }
    const double *B = dB_array[mat];
    double *X = dX_array[mat];
    for (int e = threadIdx.x; e < n * nrhs; e += blockDim.x) {
        const int c = e / n, i = e % n;
        X[i + (size_t)c * lddx] = B[i + (size_t)c * lddb];
    }
}

__global__ void ir_scatter_info_kernel(int count, const int *cidx, const int *cinfo, int *info)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) info[cidx[k]] = cinfo[k];
}

__global__ void set_float_pointers(float **out, float *base, size_t stride, int batch)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < batch) out[k] = base + (size_t)k * stride;
}

static inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct IrLayout {
    size_t stats, count, asp, as, r, ca, cp, cx, cidx, cinfo, total;
    int ldas;
};

static IrLayout ir_layout(int n, int nrhs, int batch)
{
    IrLayout L;
    L.ldas = (n + 31) & ~31;
    size_t o = 0;
    L.stats = o; o = align256(o + (size_t)batch * IR_STATS_WORDS * 8);
    L.count = o; o = align256(o + 16);
    L.asp = o;   o = align256(o + (size_t)batch * sizeof(float *));
    L.as = o;    o = align256(o + (size_t)batch * n * L.ldas * sizeof(float));
    L.r = o;     o = align256(o + (size_t)batch * nrhs * n * sizeof(double));
    L.ca = o;    o = align256(o + (size_t)batch * sizeof(double *));
    L.cp = o;    o = align256(o + (size_t)batch * sizeof(int *));
    L.cx = o;    o = align256(o + (size_t)batch * sizeof(double *));
    L.cidx = o;  o = align256(o + (size_t)batch * sizeof(int));
    L.cinfo = o; o = align256(o + (size_t)batch * sizeof(int));
    L.total = o;
    return L;
}

template <int NR>
static void launch_residual(int n, int nrhs, double **dA, int ldda, double **dB, int lddb,
                            double **dX, int lddx, double *R, unsigned long long *stats, int par,
                            int batch, cudaStream_t s)
{
    const size_t smem = (size_t)n * NR * sizeof(double);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(ir_residual_kernel<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        attr = true;
    }
    ir_residual_kernel<NR><<<dim3((n + IR_ROWS - 1) / IR_ROWS, batch), IR_ROWS, smem, s>>>(
        n, nrhs, dA, ldda, dB, lddb, dX, lddx, R, stats, par);
}

static void residual(int n, int nrhs, double **dA, int ldda, double **dB, int lddb, double **dX,
                     int lddx, double *R, unsigned long long *stats, int par, int batch,
                     cudaStream_t s)
{
    if (nrhs <= 1)      launch_residual<1>(n, nrhs, dA, ldda, dB, lddb, dX, lddx, R, stats, par, batch, s);
    else if (nrhs <= 2) launch_residual<2>(n, nrhs, dA, ldda, dB, lddb, dX, lddx, R, stats, par, batch, s);
    else if (nrhs <= 4) launch_residual<4>(n, nrhs, dA, ldda, dB, lddb, dX, lddx, R, stats, par, batch, s);
    else if (nrhs <= 8) launch_residual<8>(n, nrhs, dA, ldda, dB, lddb, dX, lddx, R, stats, par, batch, s);
    else                launch_residual<16>(n, nrhs, dA, ldda, dB, lddb, dX, lddx, R, stats, par, batch, s);
}

}  // namespace mlu

using namespace mlu;

extern "C" magma_int_t
magma_dsgesv_batched_work(magma_int_t n, magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                          magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                          double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                          magma_int_t *diter_array, magma_int_t itermax, double tol,
                          magma_int_t fallback, void *work, size_t *lwork,
                          magma_int_t batchCount, magma_queue_t queue)
{
    magma_int_t info = 0;
    if (n < 0) info = -1;
    else if (nrhs < 0 || nrhs > IR_NRHS_MAX) info = -2;
    else if (ldda < mlu_max(1, n)) info = -4;
    else if (lddb < mlu_max(1, n)) info = -7;
    else if (lddx < mlu_max(1, n)) info = -9;
    else if (itermax < 0) info = -12;
    if (info != 0) {
        magma_xerbla(__func__, -info);
        return info;
    }
    const IrLayout L = ir_layout(n, nrhs, mlu_max(batchCount, 0));
    if (work == nullptr) {          // workspace query
        *lwork = L.total;
        return 0;
    }
    if (*lwork < L.total) return -15;
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;

    cudaStream_t s = queue->stream;
    char *w = (char *)work;
    unsigned long long *stats = (unsigned long long *)(w + L.stats);
    int *count = (int *)(w + L.count);
    float **As_array = (float **)(w + L.asp);
    float *As = (float *)(w + L.as);
    double *R = (double *)(w + L.r);

    cudaMemsetAsync(w, 0, L.asp, s);   // stats, counters
    set_float_pointers<<<mlu_ceildiv(batchCount, 256), 256, 0, s>>>(As_array, As,
                                                                     (size_t)n * L.ldas, batchCount);
    const dim3 rows_grid((n + IR_ROWS - 1) / IR_ROWS, batchCount);
    ir_init_kernel<<<rows_grid, IR_ROWS, 0, s>>>(n, nrhs, dA_array, ldda, As_array, L.ldas,
                                                 dB_array, lddb, dX_array, lddx, R, stats,
                                                 diter_array);
    magma_int_t rc = magma_sgetrf_batched(n, n, As_array, L.ldas, dipiv_array, dinfo_array,
                                          batchCount, queue);
    if (rc != 0) return rc;
    const size_t ssmem = (size_t)IR_SOLVE_NR * n * sizeof(float);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(ir_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    const dim3 solve_grid(mlu_ceildiv(nrhs, IR_SOLVE_NR), batchCount);
    ir_solve_kernel<<<solve_grid, 256, ssmem, s>>>(n, nrhs, As_array, L.ldas, dipiv_array,
                                                   dX_array, lddx, R, stats, diter_array,
                                                   dinfo_array, -1, tol);
    residual(n, nrhs, dA_array, ldda, dB_array, lddb, dX_array, lddx, R, stats, 0, batchCount, s);
    for (int it = 0; it < itermax; it++) {
        ir_solve_kernel<<<solve_grid, 256, ssmem, s>>>(n, nrhs, As_array, L.ldas, dipiv_array,
                                                       dX_array, lddx, R, stats, diter_array,
                                                       dinfo_array, it, tol);
        residual(n, nrhs, dA_array, ldda, dB_array, lddb, dX_array, lddx, R, stats, (it + 1) & 1,
                 batchCount, s);
    }
    ir_final_kernel<<<mlu_ceildiv(batchCount, 256), 256, 0, s>>>(n, nrhs, stats, diter_array,
                                                                 itermax, tol, batchCount, count);
    MLU_CHECK_LAUNCH();
    if (!fallback) return 0;

    int failed = 0;
    cudaMemcpyAsync(&failed, count, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MAGMA_ERR_UNKNOWN;
    if (failed == 0) return 0;
    double **cA = (double **)(w + L.ca);
    int **cP = (int **)(w + L.cp);
    double **cX = (double **)(w + L.cx);
    int *cidx = (int *)(w + L.cidx);
    int *cinfo = (int *)(w + L.cinfo);
    cudaMemsetAsync(count + 1, 0, sizeof(int), s);
    ir_compact_kernel<<<batchCount, 256, 0, s>>>(n, nrhs, dA_array, dipiv_array, dB_array, lddb,
                                                 dX_array, lddx, stats, batchCount, count + 1, cA,
                                                 cP, cX, cidx);
    rc = magma_dgesv_batched(n, nrhs, cA, ldda, cP, cX, lddx, cinfo, failed, queue);
    if (rc != 0) return rc;
    ir_scatter_info_kernel<<<mlu_ceildiv(failed, 256), 256, 0, s>>>(failed, cidx, cinfo,
                                                                    dinfo_array);
    MLU_CHECK_LAUNCH();
    return 0;
}

extern "C" magma_int_t
magma_dsgesv_batched(magma_int_t n, magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                     magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                     double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                     magma_int_t *diter_array, magma_int_t batchCount, magma_queue_t queue)
{
    size_t lwork = 0;
    magma_int_t rc = magma_dsgesv_batched_work(n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                               lddb, dX_array, lddx, dinfo_array, diter_array, 30,
                                               0.0, 1, nullptr, &lwork, batchCount, queue);
    if (rc != 0) return rc;
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    if (queue->work_bytes < lwork) {
        if (queue->work) {
            cudaStreamSynchronize(queue->stream);
            cudaFree(queue->work);
        }
        queue->work = nullptr;
        queue->work_bytes = 0;
        if (cudaMalloc(&queue->work, lwork) != cudaSuccess) return MAGMA_ERR_DEVICE_ALLOC;
        queue->work_bytes = lwork;
    }
    return magma_dsgesv_batched_work(n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                     dX_array, lddx, dinfo_array, diter_array, 30, 0.0, 1,
                                     queue->work, &lwork, batchCount, queue);
}
