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
// that on the host (and f2d_exact against (double)f).
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

// The hardware conversions, for the rare operands the integer forms leave
// to them. On the device they are volatile inline PTX: the compiler may not
// execute them speculatively on every lane (a plain cast in the untaken
// branch was if-converted and issued for every element, on the FP64 pipe).
__host__ __device__ __forceinline__ float d2f_hw(double d) {
#ifdef __CUDA_ARCH__
    float r;
    asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(d));
    return r;
#else
    return (float)d;
#endif
}
__host__ __device__ __forceinline__ double f2d_hw(float f) {
#ifdef __CUDA_ARCH__
    double r;
    asm volatile("cvt.f64.f32 %0, %1;" : "=d"(r) : "f"(f));
    return r;
#else
    return (double)f;
#endif
}

#ifdef __CUDA_ARCH__
// the hardware form of split_lo (volatile: never issued speculatively)
__device__ __forceinline__ float split_lo_hw(double c, float hi) {
    double h, dlo;
    float r;
    asm volatile("cvt.f64.f32 %0, %1;" : "=d"(h) : "f"(hi));
    asm volatile("sub.rn.f64 %0, %1, %2;" : "=d"(dlo) : "d"(c), "d"(h));
    asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(r) : "d"(dlo));
    return r;
}
#endif

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
    if ((b << 1) == 0) return d2f_from_bits((unsigned)(b >> 32) & 0x80000000u);  // +-0
    return d2f_hw(d);
}

// (double)f exactly, from integer instructions for normal floats and zeros
// (the exponent re-biased, the 23 mantissa bits moved up); subnormals,
// infinities and NaN take the hardware conversion.
__host__ __device__ __forceinline__ double f2d_exact(float f) {
#ifdef __CUDA_ARCH__
    const unsigned u = __float_as_uint(f);
#else
    unsigned u;
    std::memcpy(&u, &f, sizeof u);
#endif
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    if (ex != 0u && ex != 0xffu) {
        const unsigned long long bits =
            sign | ((unsigned long long)(ex + (1023 - 127)) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
#ifdef __CUDA_ARCH__
        return __longlong_as_double((long long)bits);
#else
        double d;
        std::memcpy(&d, &bits, sizeof d);
        return d;
#endif
    }
    if ((u << 1) == 0u) {
#ifdef __CUDA_ARCH__
        return __longlong_as_double((long long)sign);
#else
        double d;
        std::memcpy(&d, &sign, sizeof d);
        return d;
#endif
    }
    return f2d_hw(f);
}

// The low part of a double c against its float rounding hi = d2f_rn(c):
// (float)(c - (double)hi), the exact difference (at most 29 significant
// bits) rounded to nearest even, from integer instructions. c == hi + lo
// within 2^-48 |c|: a float pair carries c to about 48 bits. Operands whose
// parts leave the normal float range take the hardware path.
__host__ __device__ __forceinline__ float split_lo(double c, float hi) {
    const unsigned long long b = d2f_bits_of(c);
    const int ec = (int)((b >> 52) & 0x7ffu);  // biased
#ifdef __CUDA_ARCH__
    const unsigned hb = __float_as_uint(hi);
#else
    unsigned hb;
    std::memcpy(&hb, &hi, sizeof hb);
#endif
    const int eh = (int)((hb >> 23) & 0xffu);  // biased
    // c and hi normal; the low part's exponent stays normal for |c| >= 2^-97
    if (ec >= 1023 - 97 && ec <= 1023 + 127 && eh >= 1 && eh <= 254) {
        const long long mc = (long long)((b & 0xfffffffffffffull) | (1ull << 52));  // c = mc 2^(ec-1075)
        const int sh = (eh - 127 - 23) - (ec - 1075);                                  // 29, or 30 on a carry
        const long long mh = (long long)((hb & 0x7fffffu) | 0x800000u) << sh;          // hi in the same unit
        long long r = mc - mh;  // |c| - |hi| in units of 2^(ec-1075), |r| <= 2^28
        if (r == 0) return d2f_from_bits(0u);
        const unsigned sign = ((unsigned)(b >> 32) & 0x80000000u) ^ (r < 0 ? 0x80000000u : 0u);
        unsigned long long a = (unsigned long long)(r < 0 ? -r : r);
#ifdef __CUDA_ARCH__
        const int len = 64 - __clzll((long long)a);  // bit length (at most 29)
#else
        const int len = 64 - __builtin_clzll(a);
#endif
        int e = ec - 1075 + len - 1;                // unbiased exponent of |r| 2^(ec-1075)
        unsigned long long m;
        if (len <= 24) {
            m = a << (24 - len);
        } else {
            const int drop = len - 24;
            const unsigned long long rem = a & ((1ull << drop) - 1), half = 1ull << (drop - 1);
            m = a >> drop;
            m += (rem > half || (rem == half && (m & 1ull))) ? 1ull : 0ull;
            if (m >> 24) {
                m >>= 1;
                e += 1;
            }
        }
        if (e >= -126 && e <= 127) return d2f_from_bits(sign | ((unsigned)(e + 127) << 23) | ((unsigned)m & 0x7fffffu));
    }
    // c = +-0: hi is the same zero and c - hi = +0
    if ((b << 1) == 0 && (hb << 1) == 0) return d2f_from_bits(0u);
#ifdef __CUDA_ARCH__
    return split_lo_hw(c, hi);
#else
    return (float)(c - (double)hi);
#endif
}

// d != 0.0 and d > 0.0 from the bit pattern (no FP64 comparison; a NaN is
// nonzero and not positive, as the comparisons have it)
__host__ __device__ __forceinline__ bool nonzero_bits(double d) { return (d2f_bits_of(d) << 1) != 0; }
__host__ __device__ __forceinline__ bool positive_bits(double d) {
    const unsigned long long b = d2f_bits_of(d);
    return !(b >> 63) && b != 0 && b <= 0x7ff0000000000000ull;
}

}  // namespace gbp
