// gbp_floatfloat.cuh -- float-float accumulation from FP32 instructions.
//
// The FP32 paths sum in float-float (an unevaluated pair hi + lo) where a
// plain float sum would lose digits and an FP64 sum would run on this GPU's
// scarce FP64 pipe (about one operation per clock per SM):
//
// * add(b) -- TwoSum (Knuth) of b into hi, its rounding error summed into lo
//   without renormalisation: the Galerkin coarsening's sums of at most 27
//   float terms, rounded once to float by value().
// * add_product(a, b) -- the dot products and norms of the FP32 inner solve:
//   the product is split exactly by an FMA (a b = p + e), p goes into hi by
//   TwoSum, both errors into lo, and the pair is renormalised (FastTwoSum)
//   after every term. After n terms hi + lo is within gamma_n^2 sum |a_i b_i|
//   of the exact dot product, gamma_n = n u / (1 - n u), u = 2^-24 (the
//   bound of Ogita, Rump and Oishi's Dot2, "Accurate sum and dot product",
//   SIAM J. Sci. Comput. 26(6), 2005, without its final rounding to float:
//   the pair is converted to FP64 instead); tests/test_kernel_host.py checks
//   that bound on the host with this source. It assumes every |a b| is a
//   normal float.
//
// The same source compiles for the host (g++ with -ffp-contract=off, where
// a + b is one rounded float addition) so the host test runs the kernels'
// arithmetic.
#pragma once

#ifndef __CUDA_ARCH__
#include <cmath>
#endif

namespace gbp {

__host__ __device__ __forceinline__ float ff_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float ff_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ float ff_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ float ff_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

struct FloatFloat {
    float hi = 0.0f, lo = 0.0f;
    __host__ __device__ __forceinline__ void reset() { hi = lo = 0.0f; }
    __host__ __device__ __forceinline__ void add(float b) {
        const float sum = ff_add(hi, b);
        const float bb = ff_sub(sum, hi);
        lo = ff_add(lo, ff_add(ff_sub(hi, ff_sub(sum, bb)), ff_sub(b, bb)));
        hi = sum;
    }
    __host__ __device__ __forceinline__ void add_product(float a, float b) {
        const float p = ff_mul(a, b);
        const float e = ff_fma(a, b, -p);
        const float s = ff_add(hi, p);
        const float bb = ff_sub(s, hi);
        const float err = ff_add(ff_sub(hi, ff_sub(s, bb)), ff_sub(p, bb));
        const float t = ff_add(lo, ff_add(err, e));
        hi = ff_add(s, t);
        lo = ff_sub(t, ff_sub(hi, s));
    }
    __host__ __device__ __forceinline__ float value() const { return ff_add(hi, lo); }
    __host__ __device__ __forceinline__ double value_fp64() const { return (double)hi + (double)lo; }
};

}  // namespace gbp
