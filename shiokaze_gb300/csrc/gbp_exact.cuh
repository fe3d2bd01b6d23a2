// gbp_exact.cuh -- FP64 results of the setup's arithmetic from integer
// instructions.
//
// On this GPU the FP64 pipe issues about two operations per clock per SM (a
// sixty-fourth of the integer rate), and the assembly's FP64 sums and the
// velocity update's FP64 products were bound by it. Where the operands allow,
// the functions here produce the bit-identical double (or float) with
// integer instructions and return true; otherwise they return false and the
// caller evaluates the FP64 expression as before.
//
// * exact_sum: the sequential FP64 sum 0 + t_0 + t_1 + ... of terms
//   t_i = f_i 2^k (floats f_i, one power of two; the face fluxes u/dx of the
//   right-hand side when dx is a power of two). If every partial sum is a
//   double, no addition rounds and the result is the exact sum, which a
//   64-bit integer holds when the terms' exponents span at most 36 binary
//   orders. Both conditions are checked.
// * mul_round: fl32(fl64(a f) 2^s) for a double a fixed per launch (dt) and
//   a float f (a pressure difference): the 77-bit product of the
//   significands rounded to 53 bits and then to 24, each to nearest with
//   ties to even, as the two hardware roundings do; results outside the
//   normal ranges take the FP64 path.
//
// The same source compiles for the host (tests/test_kernel_host.py checks
// both functions against the compiler's FP64 arithmetic).
#pragma once

#include <cstring>

namespace gbp {

__host__ __device__ __forceinline__ unsigned ex_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned u;
    std::memcpy(&u, &f, sizeof u);
    return u;
#endif
}
__host__ __device__ __forceinline__ float ex_float(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, sizeof f);
    return f;
#endif
}
__host__ __device__ __forceinline__ double ex_double(unsigned long long u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    std::memcpy(&d, &u, sizeof d);
    return d;
#endif
}
__host__ __device__ __forceinline__ int ex_clz64(unsigned long long a) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)a);
#else
    return a ? __builtin_clzll(a) : 64;
#endif
}
__host__ __device__ __forceinline__ int ex_ctz64(unsigned long long a) {
#ifdef __CUDA_ARCH__
    return __ffsll((long long)a) - 1;
#else
    return a ? __builtin_ctzll(a) : 64;
#endif
}
__host__ __device__ __forceinline__ unsigned long long ex_mulhi(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

// Sequential FP64 sum of n terms sgn_i f_i 2^k, sgn_i = -1 where bit i of
// neg is set; false if an addition could round or a value leaves the normal
// ranges (subnormal, infinite or NaN f_i included).
__host__ __device__ __forceinline__ bool exact_sum(const float *f, int n, unsigned neg, int k, double &out) {
    int emin = 1 << 20, emax = -(1 << 20);
#pragma unroll
    for (int i = 0; i < n; ++i) {
        const unsigned b = ex_bits(f[i]) & 0x7fffffffu;
        if (!b) continue;
        const int ex = (int)(b >> 23);
        if (ex == 0 || ex == 255) return false;
        const int e = ex - 150;  // f = m 2^e, m the 24-bit significand
        emin = e < emin ? e : emin;
        emax = e > emax ? e : emax;
    }
    if (emax < emin) {  // every term is +-0: 0 + (+-0) + ... = +0
        out = 0.0;
        return true;
    }
    if (emax - emin > 36 || emin + k < -1000 || emax + k > 1000) return false;
    // within 26 binades every term is below 2^50 in units of 2^emin, so a
    // partial sum of at most 7 terms stays below 2^53: none can round
    const bool spread = emax - emin > 26;
    long long s = 0;
#pragma unroll
    for (int i = 0; i < n; ++i) {
        const unsigned b = ex_bits(f[i]);
        const unsigned a = b & 0x7fffffffu;
        if (!a) continue;
        const long long m = (long long)((a & 0x7fffffu) | 0x800000u) << ((int)(a >> 23) - 150 - emin);
        // the term's sign: the float's, flipped where neg says
        s += (((b >> 31) ^ (neg >> i)) & 1u) ? -m : m;
        const unsigned long long mag = (unsigned long long)(s < 0 ? -s : s);
        if (spread && (mag >> 53) && ((mag >> ex_ctz64(mag)) >> 53)) return false;  // this partial sum would round
    }
    if (!s) {  // x + (-x) = +0 in round to nearest
        out = 0.0;
        return true;
    }
    const unsigned long long sign = s < 0 ? 1ull << 63 : 0ull;
    unsigned long long mag = (unsigned long long)(s < 0 ? -s : s);
    const int len = 64 - ex_clz64(mag);
    // exact: at most 53 significant bits (checked above)
    mag = len <= 53 ? mag << (53 - len) : mag >> (len - 53);
    const int e = emin + k + len - 1;  // unbiased exponent of the sum
    out = ex_double(sign | ((unsigned long long)(e + 1023) << 52) | (mag & 0xfffffffffffffull));
    return true;
}

// a = m 2^e (m with its hidden bit), prepared on the host for mul_round.
struct MulConst {
    unsigned long long m;
    int e;       // a's exponent with the significand as an integer (unbiased - 52)
    int s;       // the power of two applied after the FP64 rounding
    unsigned sign;  // a's sign in bit 31
    int ok;      // a is a normal double (else every call takes the FP64 path)
};

inline MulConst make_mul_const(double a, int s) {
    unsigned long long b;
    std::memcpy(&b, &a, sizeof b);
    MulConst c{};
    const int ex = (int)((b >> 52) & 0x7ff);
    c.ok = ex != 0 && ex != 0x7ff;
    c.m = (b & 0xfffffffffffffull) | (1ull << 52);
    c.e = ex - 1075;
    c.s = s;
    c.sign = (unsigned)(b >> 63) << 31;
    return c;
}

// fl32(fl64(a f) 2^s), false where the FP64 path must decide.
__host__ __device__ __forceinline__ bool mul_round(const MulConst c, float f, float &out) {
    const unsigned fb = ex_bits(f);
    const unsigned sign = (fb & 0x80000000u) ^ c.sign;
    const unsigned fa = fb & 0x7fffffffu;
    if (!c.ok) return false;
    if (!fa) {  // +-0 * a = +-0, exactly
        out = ex_float(sign);
        return true;
    }
    const int fe = (int)(fa >> 23);
    if (fe == 0 || fe == 255) return false;
    const unsigned long long mf = (fa & 0x7fffffu) | 0x800000u;
    // P = mf c.m in [2^75, 2^77): hi holds bits 64..76
    const unsigned long long lo = mf * c.m, hi = ex_mulhi(mf, c.m);
    const int sh = (hi >> 12) ? 24 : 23;  // bits dropped to keep 53
    unsigned long long q = (hi << (64 - sh)) | (lo >> sh);
    const unsigned long long rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
    int e = (fe - 150) + c.e + sh;  // fl64(a f) = q 2^e
    if (q >> 53) {
        q >>= 1;
        e += 1;
    }
    // fl64(a f) and its scaled value must be normal doubles
    const int e64 = e + 52;
    if (e64 < -1022 || e64 > 1023 || e64 + c.s < -1022 || e64 + c.s > 1023) return false;
    int e32 = e64 + c.s;
    if (e32 < -126 || e32 > 127) return false;
    const unsigned long long r29 = q & 0x1fffffffull, h29 = 0x10000000ull;
    unsigned long long r = q >> 29;
    r += (r29 > h29 || (r29 == h29 && (r & 1ull))) ? 1ull : 0ull;
    if (r >> 24) {
        r >>= 1;
        e32 += 1;
        if (e32 > 127) return false;  // rounds to infinity: the FP64 path says so
    }
    out = ex_float(sign | ((unsigned)(e32 + 127) << 23) | ((unsigned)r & 0x7fffffu));
    return true;
}

}  // namespace gbp
