/*
 * Naive level-1 CBLAS for building the reference projection as an oracle.
 *
 * The reference links GSL's cblas (unpinned: Ubuntu's libgsl0-dev /
 * libblas-dev, see scripts/Dockerfile in the reference). Neither is installed
 * here, so these plain loops stand in. Sums run in index order with one
 * accumulator, which is what a reference (netlib-style) BLAS does for unit
 * stride; an optimised BLAS may differ at roundoff level. idamax returns the
 * first index of the largest |x_i|, as BLAS specifies.
 *
 * Test infrastructure only: the oracle build links it; the product does not.
 */
#include <math.h>
#include <stddef.h>

float cblas_sdot(int n, const float *x, int incx, const float *y, int incy) {
    float s = 0.0f;
    for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
    return s;
}
double cblas_dsdot(int n, const float *x, int incx, const float *y, int incy) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += (double)x[(size_t)i * incx] * (double)y[(size_t)i * incy];
    return s;
}
double cblas_ddot(int n, const double *x, int incx, const double *y, int incy) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
    return s;
}
float cblas_snrm2(int n, const float *x, int incx) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += (double)x[(size_t)i * incx] * x[(size_t)i * incx];
    return (float)sqrt(s);
}
double cblas_dnrm2(int n, const double *x, int incx) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * x[(size_t)i * incx];
    return sqrt(s);
}
float cblas_sasum(int n, const float *x, int incx) {
    float s = 0.0f;
    for (int i = 0; i < n; ++i) s += fabsf(x[(size_t)i * incx]);
    return s;
}
double cblas_dasum(int n, const double *x, int incx) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += fabs(x[(size_t)i * incx]);
    return s;
}
size_t cblas_isamax(int n, const float *x, int incx) {
    size_t best = 0;
    float m = -1.0f;
    for (int i = 0; i < n; ++i) {
        float a = fabsf(x[(size_t)i * incx]);
        if (a > m) { m = a; best = (size_t)i; }
    }
    return best;
}
size_t cblas_idamax(int n, const double *x, int incx) {
    size_t best = 0;
    double m = -1.0;
    for (int i = 0; i < n; ++i) {
        double a = fabs(x[(size_t)i * incx]);
        if (a > m) { m = a; best = (size_t)i; }
    }
    return best;
}
void cblas_saxpy(int n, float alpha, const float *x, int incx, float *y, int incy) {
    for (int i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}
void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy) {
    for (int i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}
void cblas_sscal(int n, float alpha, float *x, int incx) {
    for (int i = 0; i < n; ++i) x[(size_t)i * incx] *= alpha;
}
void cblas_dscal(int n, double alpha, double *x, int incx) {
    for (int i = 0; i < n; ++i) x[(size_t)i * incx] *= alpha;
}
