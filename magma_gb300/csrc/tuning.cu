// tuning.cu -- tuning of the fixed-size factorisation (magma_?getrf_batched and
// everything built on it) and the persisted tuning file.
//
// MAGMA chooses its batched LU blocking from fixed crossover tables per size
// (control/get_batched_crossover.cpp:300-342 nb/recnb, :918-928 the TRSM stop
// size, control/get_batched_gemm_decision.cpp:233-253 the GEMM path).  Here
// the choices that matter on GB300 are a table per precision and size bin of
// max(m, n) (<= 64, 128, 256, 512, 1024, larger):
//   two_level   FP32: 128-column blocks with one rank-128 update right of each
//               (lu_outer.cu), or a rank-32 update after every panel;
//   band_ctas   FP32: the fused band kernel when the step gives at least this
//               many CTAs per SM (1, 2 or 4), else separate interchange and
//               update kernels;
//   tile64      FP64: 64 x 64 update tiles (32 x 32 for thin trailing blocks),
//               or 32 x 32 always.
// Every choice performs the same operations on every element in the same
// order, so tuning never changes a result.  magma_?getrf_batched_autotune times
// the candidates on the device and installs the fastest;
// magma_lu_tuning_save / _load write and read both this table and the
// variable-size one as JSON, and a queue created while MAGMA_LU_TUNING_FILE
// names a file loads it (once per process).
#include "common.cuh"
#include "trace.cuh"
#include "lu_core.cuh"

#include <algorithm>
#include <mutex>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>

extern "C" magma_int_t magma_dvbatched_tuning_get(magma_int_t *nb, magma_int_t *tile);
extern "C" magma_int_t magma_svbatched_tuning_get(magma_int_t *nb, magma_int_t *tile);
extern "C" magma_int_t magma_dvbatched_tuning_set(const magma_int_t *nb, const magma_int_t *tile);
extern "C" magma_int_t magma_svbatched_tuning_set(const magma_int_t *nb, const magma_int_t *tile);

namespace mlu {

namespace {
std::mutex g_fixed_mu;
FixedTune g_fixed[2] = {
    {{1, 1, 1, 1, 1, 1}, {2, 2, 2, 2, 2, 2}, {1, 1, 1, 1, 1, 1}},   // double (two_level unused)
    {{1, 1, 1, 1, 1, 1}, {2, 2, 2, 2, 2, 2}, {1, 1, 1, 1, 1, 1}},   // float (tile64 unused)
};
constexpr int VB_BINS = 8;      // the variable-size table (lu_vbatched.cu)
}  // namespace

int fixed_tune_bin(int m, int n)
{
    const int mx = m > n ? m : n;
    int b = 0;
    for (int ub = 64; b < FIXED_TUNE_BINS - 1 && mx > ub; ub <<= 1) b++;
    return b;
}

FixedChoice fixed_choice(bool fp64, int m, int n)
{
    const int b = fixed_tune_bin(m, n);
    std::lock_guard<std::mutex> lk(g_fixed_mu);
    const FixedTune &t = g_fixed[fp64 ? 0 : 1];
    return FixedChoice{t.two_level[b] != 0, (int)t.band_ctas[b], t.tile64[b] != 0};
}

static FixedTune fixed_get(bool fp64)
{
    std::lock_guard<std::mutex> lk(g_fixed_mu);
    return g_fixed[fp64 ? 0 : 1];
}

static void fixed_put(bool fp64, const FixedTune &t)
{
    std::lock_guard<std::mutex> lk(g_fixed_mu);
    g_fixed[fp64 ? 0 : 1] = t;
}

static bool fixed_valid(const FixedTune &t)
{
    for (int b = 0; b < FIXED_TUNE_BINS; b++) {
        if (t.two_level[b] > 1 || t.tile64[b] > 1) return false;
        if (t.band_ctas[b] != 1 && t.band_ctas[b] != 2 && t.band_ctas[b] != 4) return false;
    }
    return true;
}

// uniform(-1, 1) trial entries from a counter-based hash (splitmix64)
template <typename T>
__global__ void tune_fill_kernel(T *buf, size_t count, unsigned long long seed)
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

template <typename T>
__global__ void tune_arrays_kernel(int k, int n, T *A, int *P, T **dA, int **dP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    dA[i] = A + (size_t)i * n * n;
    dP[i] = P + (size_t)i * n;
}

template <typename T>
magma_int_t blocked_getrf(int m, int n, T **dA, int ldda, int **ipiv, int *info, int batch,
                          magma_queue_t q);
bool two_level_possible(int m, int n);

// Times every candidate of every bin up to max_n on `batch` trial matrices of
// three quarters of the bin's largest order (max_n itself for the last bin);
// installs the fastest per bin.  Other calls must not run meanwhile: the trials
// run through the shared table.
template <typename T>
static magma_int_t fixed_autotune(int max_n, int batch, magma_queue_t q)
{
    const bool fp64 = sizeof(T) == 8;
    FixedTune t = fixed_get(fp64);
    const FixedTune start = t;
    cudaStream_t s = q->stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        return MAGMA_ERR_UNKNOWN;
    }
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, q->device);
    magma_int_t rc = MAGMA_SUCCESS;
    for (int b = 0, ub = 64; b < FIXED_TUNE_BINS && rc == MAGMA_SUCCESS; b++, ub <<= 1) {
        const int lo = b == 0 ? 33 : ub / 2 + 1;     // n <= 32 is the fused small kernel
        if (lo > max_n) break;
        const int n = b == FIXED_TUNE_BINS - 1 ? max_n : max(lo, min(max_n, 3 * ub / 4));
        // at most ~1 GB of trial matrices
        const int k = (int)std::max<size_t>(
            1, std::min<size_t>((size_t)batch, ((size_t)1 << 30) / ((size_t)n * n * sizeof(T))));
        T *A = nullptr, **dA = nullptr;
        int *P = nullptr, **dP = nullptr, *info = nullptr;
        if (device_malloc((void **)&A, (size_t)k * n * n * sizeof(T)) != cudaSuccess ||
            device_malloc((void **)&P, (size_t)k * n * sizeof(int)) != cudaSuccess ||
            device_malloc((void **)&dA, k * sizeof(T *)) != cudaSuccess ||
            device_malloc((void **)&dP, k * sizeof(int *)) != cudaSuccess ||
            device_malloc((void **)&info, k * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            rc = MAGMA_ERR_DEVICE_ALLOC;
        }
        if (rc == MAGMA_SUCCESS) {
            MLU_LAUNCH(mlu::KC_OTHER, s, tune_arrays_kernel<T><<<(k + 255) / 256, 256, 0, s>>>(k, n, A, P, dA, dP));
            // candidates: (two_level, band_ctas, tile64)
            int cand[12][3], nc = 0;
            if (fp64) {
                for (int t64 = 0; t64 < 2; t64++) { cand[nc][0] = 1; cand[nc][1] = 2; cand[nc][2] = t64; nc++; }
            } else {
                const int tl_max = two_level_possible(n, n) ? 1 : 0;
                for (int tl = 0; tl <= tl_max; tl++)
                    for (int bc : {1, 2, 4}) { cand[nc][0] = tl; cand[nc][1] = bc; cand[nc][2] = 1; nc++; }
            }
            float best = -1.f;
            int bi = 0;
            for (int c = 0; c < nc && rc == MAGMA_SUCCESS; c++) {
                FixedTune trial = t;
                trial.two_level[b] = (unsigned char)cand[c][0];
                trial.band_ctas[b] = (unsigned char)cand[c][1];
                trial.tile64[b] = (unsigned char)cand[c][2];
                fixed_put(fp64, trial);
                float tmin = -1.f;
                for (int rep = 0; rep < 2 && rc == MAGMA_SUCCESS; rep++) {
                    MLU_LAUNCH(mlu::KC_OTHER, s, tune_fill_kernel<T><<<4 * sms, 256, 0, s>>>(
                        A, (size_t)k * n * n, 0x7e57ull + 131ull * b));
                    cudaEventRecord(e0, s);
                    rc = blocked_getrf<T>(n, n, dA, n, dP, info, k, q);
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
                    bi = c;
                }
            }
            t.two_level[b] = (unsigned char)cand[bi][0];
            t.band_ctas[b] = (unsigned char)cand[bi][1];
            t.tile64[b] = (unsigned char)cand[bi][2];
        }
        cudaFree(A); cudaFree(P); cudaFree(dA); cudaFree(dP); cudaFree(info);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    fixed_put(fp64, rc == MAGMA_SUCCESS ? t : start);
    return rc;
}

template <typename T>
static magma_int_t fixed_get_entry(magma_int_t *two_level, magma_int_t *band_ctas, magma_int_t *tile64)
{
    const FixedTune t = fixed_get(sizeof(T) == 8);
    for (int b = 0; b < FIXED_TUNE_BINS; b++) {
        if (two_level) two_level[b] = t.two_level[b];
        if (band_ctas) band_ctas[b] = t.band_ctas[b];
        if (tile64) tile64[b] = t.tile64[b];
    }
    return MAGMA_SUCCESS;
}

template <typename T>
static magma_int_t fixed_set_entry(const magma_int_t *two_level, const magma_int_t *band_ctas,
                                   const magma_int_t *tile64)
{
    if (!two_level) return -1;
    if (!band_ctas) return -2;
    if (!tile64) return -3;
    FixedTune t;
    for (int b = 0; b < FIXED_TUNE_BINS; b++) {
        if (two_level[b] < 0 || two_level[b] > 1) return -1;
        if (band_ctas[b] != 1 && band_ctas[b] != 2 && band_ctas[b] != 4) return -2;
        if (tile64[b] < 0 || tile64[b] > 1) return -3;
        t.two_level[b] = (unsigned char)two_level[b];
        t.band_ctas[b] = (unsigned char)band_ctas[b];
        t.tile64[b] = (unsigned char)tile64[b];
    }
    fixed_put(sizeof(T) == 8, t);
    return MAGMA_SUCCESS;
}

// ---------------------------------------------------------------------------
// The tuning file (JSON, written and read by this library only).

static void put_array(FILE *f, const char *key, const magma_int_t *v, int count, bool last)
{
    fprintf(f, "\"%s\": [", key);
    for (int i = 0; i < count; i++) fprintf(f, "%s%d", i ? ", " : "", (int)v[i]);
    fprintf(f, "]%s", last ? "" : ", ");
}

// Reads the integer array that follows `key` (searched from *pos on) into v;
// advances *pos.  False when the key or `count` integers are missing.
static bool get_array(const std::string &s, size_t *pos, const char *key, magma_int_t *v, int count)
{
    const std::string k = std::string("\"") + key + "\"";
    size_t p = s.find(k, *pos);
    if (p == std::string::npos) return false;
    p = s.find('[', p + k.size());
    if (p == std::string::npos) return false;
    p++;
    for (int i = 0; i < count; i++) {
        while (p < s.size() && (s[p] == ' ' || s[p] == ',' || s[p] == '\n' || s[p] == '\t')) p++;
        char *end = nullptr;
        const long x = strtol(s.c_str() + p, &end, 10);
        if (end == s.c_str() + p) return false;
        v[i] = (magma_int_t)x;
        p = end - s.c_str();
    }
    *pos = p;
    return true;
}

static bool find_key(const std::string &s, size_t *pos, const char *key)
{
    const size_t p = s.find(std::string("\"") + key + "\"", *pos);
    if (p == std::string::npos) return false;
    *pos = p;
    return true;
}

}  // namespace mlu

using namespace mlu;

extern "C" magma_int_t magma_dgetrf_batched_autotune(magma_int_t max_n, magma_int_t batch,
                                                     magma_queue_t queue)
{
    if (max_n < 0) return -1;
    if (batch < 1) return -2;
    if (queue == nullptr) return -3;
    return max_n <= 32 ? MAGMA_SUCCESS : fixed_autotune<double>(max_n, batch, queue);
}

extern "C" magma_int_t magma_sgetrf_batched_autotune(magma_int_t max_n, magma_int_t batch,
                                                     magma_queue_t queue)
{
    if (max_n < 0) return -1;
    if (batch < 1) return -2;
    if (queue == nullptr) return -3;
    return max_n <= 32 ? MAGMA_SUCCESS : fixed_autotune<float>(max_n, batch, queue);
}

extern "C" magma_int_t magma_dgetrf_batched_tuning_get(magma_int_t *two_level, magma_int_t *band_ctas,
                                                       magma_int_t *tile64)
{
    return fixed_get_entry<double>(two_level, band_ctas, tile64);
}
extern "C" magma_int_t magma_sgetrf_batched_tuning_get(magma_int_t *two_level, magma_int_t *band_ctas,
                                                       magma_int_t *tile64)
{
    return fixed_get_entry<float>(two_level, band_ctas, tile64);
}
extern "C" magma_int_t magma_dgetrf_batched_tuning_set(const magma_int_t *two_level,
                                                       const magma_int_t *band_ctas,
                                                       const magma_int_t *tile64)
{
    return fixed_set_entry<double>(two_level, band_ctas, tile64);
}
extern "C" magma_int_t magma_sgetrf_batched_tuning_set(const magma_int_t *two_level,
                                                       const magma_int_t *band_ctas,
                                                       const magma_int_t *tile64)
{
    return fixed_set_entry<float>(two_level, band_ctas, tile64);
}

extern "C" magma_int_t magma_lu_tuning_save(const char *path)
{
    if (path == nullptr) return -1;
    FILE *f = fopen(path, "w");
    if (!f) return MAGMA_ERR_UNKNOWN;
    magma_int_t a[FIXED_TUNE_BINS], b[FIXED_TUNE_BINS], c[FIXED_TUNE_BINS];
    magma_int_t vn[VB_BINS], vt[VB_BINS];
    fprintf(f, "{\"format\": \"magma_lu tuning 1\",\n \"getrf_batched\": {\"bins_max_order\": "
               "[64, 128, 256, 512, 1024, 0],\n");
    for (int p = 0; p < 2; p++) {
        if (p == 0) magma_dgetrf_batched_tuning_get(a, b, c);
        else magma_sgetrf_batched_tuning_get(a, b, c);
        fprintf(f, "  \"%s\": {", p == 0 ? "d" : "s");
        put_array(f, "two_level", a, FIXED_TUNE_BINS, false);
        put_array(f, "band_ctas", b, FIXED_TUNE_BINS, false);
        put_array(f, "tile64", c, FIXED_TUNE_BINS, true);
        fprintf(f, "}%s\n", p == 0 ? "," : "");
    }
    fprintf(f, " },\n \"getrf_vbatched\": {\"bins_max_order\": [16, 32, 64, 128, 256, 512, 1024, 0],\n");
    for (int p = 0; p < 2; p++) {
        if (p == 0) magma_dvbatched_tuning_get(vn, vt);
        else magma_svbatched_tuning_get(vn, vt);
        fprintf(f, "  \"%s\": {", p == 0 ? "d" : "s");
        put_array(f, "nb", vn, VB_BINS, false);
        put_array(f, "tile", vt, VB_BINS, true);
        fprintf(f, "}%s\n", p == 0 ? "," : "");
    }
    fprintf(f, " }\n}\n");
    const bool ok = fflush(f) == 0;
    return fclose(f) == 0 && ok ? MAGMA_SUCCESS : MAGMA_ERR_UNKNOWN;
}

extern "C" magma_int_t magma_lu_tuning_load(const char *path)
{
    if (path == nullptr) return -1;
    FILE *f = fopen(path, "r");
    if (!f) return MAGMA_ERR_UNKNOWN;
    std::string s;
    char buf[4096];
    size_t got;
    while ((got = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, got);
    fclose(f);
    if (s.find("\"magma_lu tuning 1\"") == std::string::npos) return MAGMA_ERR_UNKNOWN;
    magma_int_t a[2][FIXED_TUNE_BINS], b[2][FIXED_TUNE_BINS], c[2][FIXED_TUNE_BINS];
    magma_int_t vn[2][VB_BINS], vt[2][VB_BINS];
    size_t pos = 0;
    if (!find_key(s, &pos, "getrf_batched")) return MAGMA_ERR_UNKNOWN;
    for (int p = 0; p < 2; p++) {
        if (!find_key(s, &pos, p == 0 ? "d" : "s") || !get_array(s, &pos, "two_level", a[p], FIXED_TUNE_BINS) ||
            !get_array(s, &pos, "band_ctas", b[p], FIXED_TUNE_BINS) ||
            !get_array(s, &pos, "tile64", c[p], FIXED_TUNE_BINS))
            return MAGMA_ERR_UNKNOWN;
    }
    if (!find_key(s, &pos, "getrf_vbatched")) return MAGMA_ERR_UNKNOWN;
    for (int p = 0; p < 2; p++) {
        if (!find_key(s, &pos, p == 0 ? "d" : "s") || !get_array(s, &pos, "nb", vn[p], VB_BINS) ||
            !get_array(s, &pos, "tile", vt[p], VB_BINS))
            return MAGMA_ERR_UNKNOWN;
    }
    // validate everything before installing anything
    for (int p = 0; p < 2; p++) {
        FixedTune t;
        for (int i = 0; i < FIXED_TUNE_BINS; i++) {
            t.two_level[i] = (unsigned char)a[p][i];
            t.band_ctas[i] = (unsigned char)b[p][i];
            t.tile64[i] = (unsigned char)c[p][i];
            if (a[p][i] < 0 || b[p][i] < 0 || c[p][i] < 0) return MAGMA_ERR_UNKNOWN;
        }
        if (!fixed_valid(t)) return MAGMA_ERR_UNKNOWN;
        for (int i = 0; i < VB_BINS; i++)
            if ((vn[p][i] != 8 && vn[p][i] != 16 && vn[p][i] != 32) || vt[p][i] < 0 || vt[p][i] > 2)
                return MAGMA_ERR_UNKNOWN;
    }
    magma_dgetrf_batched_tuning_set(a[0], b[0], c[0]);
    magma_sgetrf_batched_tuning_set(a[1], b[1], c[1]);
    if (magma_dvbatched_tuning_set(vn[0], vt[0]) != 0 || magma_svbatched_tuning_set(vn[1], vt[1]) != 0)
        return MAGMA_ERR_UNKNOWN;
    return MAGMA_SUCCESS;
}

// Called at queue creation: loads the file MAGMA_LU_TUNING_FILE names, once per
// process (a file that cannot be read is reported and ignored).
void mlu::tuning_load_env_once()
{
    static std::once_flag once;
    std::call_once(once, [] {
        const char *p = getenv("MAGMA_LU_TUNING_FILE");
        if (p && *p && magma_lu_tuning_load(p) != MAGMA_SUCCESS)
            fprintf(stderr, "magma_lu: could not load the tuning file %s (MAGMA_LU_TUNING_FILE)\n", p);
    });
}
