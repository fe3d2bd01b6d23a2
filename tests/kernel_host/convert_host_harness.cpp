// TEST INFRASTRUCTURE: the GPU kernels' integer double -> float conversion
// (shiokaze_gb300/csrc/gbp_convert.cuh) compiled for the host, for
// tests/test_kernel_host.py to compare with the compiler's own conversion.
#define __host__
#define __device__
#define __forceinline__ inline
#include "gbp_convert.cuh"

extern "C" void host_d2f(const double *in, float *out, long long n) {
    for (long long i = 0; i < n; ++i) out[i] = gbp::d2f_rn(in[i]);
}

extern "C" void host_f2d(const float *in, double *out, long long n) {
    for (long long i = 0; i < n; ++i) out[i] = gbp::f2d_exact(in[i]);
}

extern "C" void host_bits_tests(const double *in, unsigned char *nonzero, unsigned char *positive, long long n) {
    for (long long i = 0; i < n; ++i) {
        nonzero[i] = gbp::nonzero_bits(in[i]) ? 1 : 0;
        positive[i] = gbp::positive_bits(in[i]) ? 1 : 0;
    }
}

extern "C" void host_split(const double *in, float *hi, float *lo, long long n) {
    for (long long i = 0; i < n; ++i) {
        hi[i] = gbp::d2f_rn(in[i]);
        lo[i] = gbp::split_lo(in[i], hi[i]);
    }
}
