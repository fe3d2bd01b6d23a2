// gbp_convert.cuh -- double -> float conversion from integer instructions.
//
// On this GPU the FP64 pipe issues about one operation per clock per SM,
// and a double -> float conversion (F2F) runs on it: kernels that only
// narrow FP64 values to FP32 (the FP32 copy of the assembled operator, the
// FP32 copy of the refinement residual, the float pressure) were bound by
// that pipe. d2f_rn rounds the same way with integer operations: the
// float's exponent is the double's re-biased, its 23 mantissa bits the
// double's top 23, rounded to nearest with ties to even on the 29 bits
// dropped; a carry out of the mantissa moves into the exponent (and from the
// largest finite float to infinity, as the rounding requires). Inputs whose
// result is not a normal float before rounding (zero, float subnormals,
// overflow, infinities, NaN) take the hardware conversion. The result equals
// (float)d bit for bit for every double; tests/test_kernel_host.py checks
// that on the host.
#pragma once

#include <cstring>

namespace gbp {

__host__ __device__ __forceinline__ unsigned long long d2f_bits_of(double d) {
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(d);
#else
    unsigned long long b;
    std::memcpy(&b, &d, sizeof b);
    return b;
#endif
}

__host__ __device__ __forceinline__ float d2f_from_bits(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
#endif
}

__host__ __device__ __forceinline__ float d2f_rn(double d) {
    const unsigned long long b = d2f_bits_of(d);
    const int e32 = (int)((b >> 52) & 0x7ffu) - 1023 + 127;
    if (e32 >= 1 && e32 <= 254) {
        const unsigned long long m = b & 0xfffffffffffffull;
        const unsigned long long rem = m & 0x1fffffffull, half = 0x10000000ull;
        unsigned mm = (unsigned)(m >> 29);
        mm += (rem > half || (rem == half && (mm & 1u))) ? 1u : 0u;
        const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
        return d2f_from_bits(sign | (((unsigned)e32 << 23) + mm));
    }
    return (float)d;
}

}  // namespace gbp
