// ir_noalloc.cu -- batched mixed-precision refinement without any device
// allocation: magma_dsgesv_batched_noalloc.
//
// Who needs it.  magma_dsgesv_batched grows a workspace with cudaMalloc and
// magma_dsgesv_batched_work needs the caller to provide one.  Some callers can
// do neither: a process whose device memory is already reserved in full by
// another allocator (a framework's caching allocator owns the pool, so a
// cudaMalloc from inside a library either fails or fragments it), code running
// in a context whose rules forbid allocation calls, and thin foreign-language
// bindings (a Fortran bind(C) interface, a cgo stub) that have no way to own
// and free a device buffer.  This entry point takes the same arguments as
// magma_dsgesv_batched and finds its scratch in a fixed array compiled into
// the library.
//
// The array.  NOALLOC_SCRATCH_BYTES (32 MiB) of device memory, declared at file
// scope below, exists on every GPU that loads this library until the process
// exits.  Requests whose workspace does not fit are rejected before any work
// is enqueued.
//
// Set-up.  Host code cannot pass the array's name to a kernel (on the host it
// is only a stand-in for the device symbol), so the first call on each device
// looks up the array's device address with cudaGetSymbolAddress, with that
// device current, and keeps it; that first call on a device should come
// before any stream capture.  The kept address belongs to the device's
// primary context (the CUDA runtime's): a process that resets the device
// (cudaDeviceReset) or runs the queue's stream in another context must not
// call this entry afterwards, since the kept address would then be stale.
//
// Sharing.  Every call uses the same array and the array keeps whatever the
// previous call left in it; the refinement clears everything that must start
// at zero (statistics, counters) at the start of each call.  Calls whose work
// overlaps on the GPU -- two streams, or two host threads -- race on the
// array; issue them one after another on one stream.
#include "common.cuh"
#include <mutex>

extern "C" magma_int_t
magma_dsgesv_batched_work(magma_int_t n, magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                          magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                          double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                          magma_int_t *diter_array, magma_int_t itermax, double tol,
                          magma_int_t fallback, void *work, size_t *lwork,
                          magma_int_t batchCount, magma_queue_t queue);

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)32 << 20;
constexpr int NOALLOC_MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_lock;
void *g_scratch_addr[NOALLOC_MAX_DEVICES] = {nullptr};

// Device address of the scratch array on `device`, looked up once per device
// with that device current.  Returns nullptr on failure.
void *scratch_address(int device)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return nullptr;
    std::lock_guard<std::mutex> guard(g_setup_lock);
    if (g_scratch_addr[device]) return g_scratch_addr[device];
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return nullptr;
    if (prev != device && cudaSetDevice(device) != cudaSuccess) return nullptr;
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        fprintf(stderr, "magma_dsgesv_batched_noalloc: cudaGetSymbolAddress failed on device %d: %s\n",
                device, cudaGetErrorString(e));
        return nullptr;
    }
    g_scratch_addr[device] = ptr;
    return ptr;
}

}  // namespace

extern "C" magma_int_t
magma_dsgesv_batched_noalloc(magma_int_t n, magma_int_t nrhs, double **dA_array, magma_int_t ldda,
                             magma_int_t **dipiv_array, double **dB_array, magma_int_t lddb,
                             double **dX_array, magma_int_t lddx, magma_int_t *dinfo_array,
                             magma_int_t *diter_array, magma_int_t batchCount,
                             magma_queue_t queue)
{
    // argument checks and the workspace size, without touching the device
    size_t need = 0;
    magma_int_t rc = magma_dsgesv_batched_work(n, nrhs, dA_array, ldda, dipiv_array, dB_array,
                                               lddb, dX_array, lddx, dinfo_array, diter_array, 30,
                                               0.0, 1, nullptr, &need, batchCount, queue);
    if (rc != 0) return rc;
    if (n == 0 || nrhs == 0 || batchCount <= 0) return 0;
    if (need > NOALLOC_SCRATCH_BYTES) {
        fprintf(stderr,
                "magma_dsgesv_batched_noalloc: n=%d nrhs=%d batchCount=%d needs %zu bytes of "
                "scratch; the static scratch holds %zu bytes. Split the batch, or use "
                "magma_dsgesv_batched_work with a caller-provided workspace.\n",
                (int)n, (int)nrhs, (int)batchCount, need, NOALLOC_SCRATCH_BYTES);
        return MAGMA_ERR_NOT_SUPPORTED;
    }
    void *scratch = scratch_address(queue->device);
    if (!scratch) return MAGMA_ERR_UNKNOWN;
    size_t have = NOALLOC_SCRATCH_BYTES;
    return magma_dsgesv_batched_work(n, nrhs, dA_array, ldda, dipiv_array, dB_array, lddb,
                                     dX_array, lddx, dinfo_array, diter_array, 30, 0.0, 1,
                                     scratch, &have, batchCount, queue);
}
