// TEST INFRASTRUCTURE: the GPU kernels' float-float accumulation
// (shiokaze_gb300/csrc/gbp_floatfloat.cuh) compiled for the host, for
// tests/test_kernel_host.py to bound its error against exact sums.
#define __host__
#define __device__
#define __forceinline__ inline
#include "gbp_floatfloat.cuh"

// One thread's partial of the FP32 inner solve's dot product: n terms
// a_i b_i through add_product, converted to FP64 as a block flush does.
extern "C" double host_ff_dot(const float *a, const float *b, long long n) {
    gbp::FloatFloat f;
    for (long long i = 0; i < n; ++i) f.add_product(a[i], b[i]);
    return f.value_fp64();
}

// The coarsening's sums: n float terms through add, rounded once to float.
extern "C" float host_ff_sum(const float *x, long long n) {
    gbp::FloatFloat f;
    for (long long i = 0; i < n; ++i) f.add(x[i]);
    return f.value();
}
