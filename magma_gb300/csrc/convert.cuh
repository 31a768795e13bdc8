// convert.cuh -- double -> float conversion on the integer pipes.
//
// On this part FP64 instructions issue at 1/64 of the FP32 rate, and a
// conversion from double is an FP64-pipe instruction.  Converting a whole FP64
// matrix to FP32 that way makes a memory-bound pass FP64-bound, so the
// refinement converts with this integer implementation of IEEE 754
// round-to-nearest-even instead (derived from the binary64/binary32 formats:
// 53-bit significand rounded to 24 bits, ties to even, gradual underflow,
// overflow to infinity).  NaN inputs give a quiet NaN of the same sign.
#pragma once
#include <cuda_runtime.h>

namespace mlu {

__device__ __forceinline__ float d2f_rn_int(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (e == 0x7ff) return __uint_as_float(sign | (m ? 0x7fc00000u | (unsigned)(m >> 29) : 0x7f800000u));
    if (e == 0) return __uint_as_float(sign);          // binary64 subnormals are far below 2^-150
    int E = e - 1023 + 127;                            // binary32 biased exponent
    const unsigned long long full = m | (1ull << 52);  // 53-bit significand
    int shift = 29;
    if (E <= 0) {                                      // binary32 subnormal range
        shift += 1 - E;
        if (shift >= 54) return __uint_as_float(sign); // below half the smallest subnormal
        E = 0;
    }
    unsigned long long q = full >> shift;
    const unsigned long long rem = full & ((1ull << shift) - 1);
    const unsigned long long half = 1ull << (shift - 1);
    if (rem > half || (rem == half && (q & 1ull))) q++;
    if (E == 0) return __uint_as_float(sign | (unsigned)q);   // a carry into bit 23 is the min normal
    if (q == (1ull << 24)) {
        q >>= 1;
        E++;
    }
    if (E >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)E << 23) | ((unsigned)q & 0x7fffffu));
}

// true when x (a double) is finite and its float image overflowed
__device__ __forceinline__ bool d2f_overflowed(double x, float f)
{
    const unsigned fb = __float_as_uint(f);
    const bool f_inf = (fb & 0x7fffffffu) == 0x7f800000u;
    const bool x_finite = ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) !=
                          0x7ff0000000000000ull;
    return f_inf && x_finite;
}

}  // namespace mlu
