// Stand-in for the four CBLAS level-1 routines Puck calls. The bodies live in
// oracle/ref/shim_blas.c, compiled without fast-math or FMA contraction so the
// summation order is fixed: sequential over the index, each product and each
// sum rounded to float. Test infrastructure only.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
typedef int MKL_INT;
float cblas_sdot(const MKL_INT n, const float* x, const MKL_INT incx, const float* y,
                 const MKL_INT incy);
void cblas_saxpy(const MKL_INT n, const float a, const float* x, const MKL_INT incx, float* y,
                 const MKL_INT incy);
float cblas_snrm2(const MKL_INT n, const float* x, const MKL_INT incx);
void cblas_sscal(const MKL_INT n, const float a, float* x, const MKL_INT incx);
#ifdef __cplusplus
}
#endif
