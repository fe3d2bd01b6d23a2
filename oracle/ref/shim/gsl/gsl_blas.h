/*
 * Stand-in for GSL's <gsl/gsl_blas.h>, used only to compile the reference
 * projection from its own sources for the oracle. GSL and a system BLAS are
 * not installed here; the reference's BLAS wrappers
 * (src/math/blas_wrapper.h, local/include/pcgsolver/blas_wrapper.h) only need
 * these level-1 routines with unit stride. They are implemented naively, in
 * index order, in cblas_naive.c next to this directory.
 *
 * Test infrastructure: nothing in the shipped library includes this file.
 */
#ifndef ORACLE_SHIM_GSL_BLAS_H
#define ORACLE_SHIM_GSL_BLAS_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
float  cblas_sdot(int n, const float *x, int incx, const float *y, int incy);
double cblas_dsdot(int n, const float *x, int incx, const float *y, int incy);
double cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
float  cblas_snrm2(int n, const float *x, int incx);
double cblas_dnrm2(int n, const double *x, int incx);
float  cblas_sasum(int n, const float *x, int incx);
double cblas_dasum(int n, const double *x, int incx);
size_t cblas_isamax(int n, const float *x, int incx);
size_t cblas_idamax(int n, const double *x, int incx);
void   cblas_saxpy(int n, float alpha, const float *x, int incx, float *y, int incy);
void   cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
void   cblas_sscal(int n, float alpha, float *x, int incx);
void   cblas_dscal(int n, double alpha, double *x, int incx);
#ifdef __cplusplus
}
#endif
#endif
