// lu_blocked.cu -- blocked right-looking LU and solves for n > 32.
#include "common.cuh"

namespace mlu {

template <typename T>
magma_int_t blocked_getrf(int, int, T **, int, int **, int *, int, magma_queue_t)
{
    return MAGMA_ERR_NOT_IMPLEMENTED;
}

template <typename T>
magma_int_t blocked_getrs(bool, int, int, T **, int, int **, T **, int, int, magma_queue_t)
{
    return MAGMA_ERR_NOT_IMPLEMENTED;
}

template magma_int_t blocked_getrf<double>(int, int, double **, int, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrf<float>(int, int, float **, int, int **, int *, int, magma_queue_t);
template magma_int_t blocked_getrs<double>(bool, int, int, double **, int, int **, double **, int, int, magma_queue_t);
template magma_int_t blocked_getrs<float>(bool, int, int, float **, int, int **, float **, int, int, magma_queue_t);

}  // namespace mlu
