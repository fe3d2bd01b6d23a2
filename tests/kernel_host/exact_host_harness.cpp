// TEST INFRASTRUCTURE: the setup kernels' integer forms of FP64 arithmetic
// (shiokaze_gb300/csrc/gbp_exact.cuh) compiled for the host, for
// tests/test_kernel_host.py to compare with the compiler's FP64 arithmetic.
#define __host__
#define __device__
#define __forceinline__ inline
#include "gbp_exact.cuh"

// Per row of 6 terms: 1 and the integer sum where exact_sum decides, else 0.
extern "C" void host_exact_sum(const float *f, const unsigned *neg, const int *n, int k, long long rows,
                               double *out, unsigned char *ok) {
    for (long long r = 0; r < rows; ++r) ok[r] = gbp::exact_sum(f + 6 * r, n[r], neg[r], k, out[r]) ? 1 : 0;
}

// Per value: 1 and fl32(fl64(a f) 2^s) where mul_round decides, else 0.
extern "C" void host_mul_round(double a, int s, const float *f, long long n, float *out, unsigned char *ok) {
    const gbp::MulConst c = gbp::make_mul_const(a, s);
    for (long long i = 0; i < n; ++i) ok[i] = gbp::mul_round(c, f[i], out[i]) ? 1 : 0;
}
