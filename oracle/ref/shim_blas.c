/*
 * Deterministic BLAS for the oracle build of the reference (test
 * infrastructure only). Puck calls sgemm_ ("TN" only), cblas_sdot,
 * cblas_saxpy, cblas_snrm2 and cblas_sscal. MKL/OpenBLAS sum in a blocked,
 * library-specific order; this file fixes the order so that the CUDA path can
 * reproduce every float bit:
 *   dot(x, y)  = (((0 + x0*y0) + x1*y1) + ...)  each product and sum rounded
 *   nrm2(x)    = sqrtf(dot(x, x))
 *   sgemm TN   : C[i + j*ldc] = dot(A[:, i], B[:, j])  (alpha = 1, beta = 0)
 * Compile with -O2 -ffp-contract=off and without -ffast-math.
 */
#include <math.h>
#include <stddef.h>

typedef int MKL_INT;

float cblas_sdot(const MKL_INT n, const float* x, const MKL_INT incx, const float* y,
                 const MKL_INT incy) {
    float s = 0.0f;
    for (MKL_INT i = 0; i < n; ++i) {
        float p = x[(ptrdiff_t)i * incx] * y[(ptrdiff_t)i * incy];
        s = s + p;
    }
    return s;
}

void cblas_saxpy(const MKL_INT n, const float a, const float* x, const MKL_INT incx, float* y,
                 const MKL_INT incy) {
    for (MKL_INT i = 0; i < n; ++i) {
        float p = a * x[(ptrdiff_t)i * incx];
        y[(ptrdiff_t)i * incy] = y[(ptrdiff_t)i * incy] + p;
    }
}

float cblas_snrm2(const MKL_INT n, const float* x, const MKL_INT incx) {
    return sqrtf(cblas_sdot(n, x, incx, x, incx));
}

void cblas_sscal(const MKL_INT n, const float a, float* x, const MKL_INT incx) {
    for (MKL_INT i = 0; i < n; ++i) {
        x[(ptrdiff_t)i * incx] = a * x[(ptrdiff_t)i * incx];
    }
}

/* Column-major sgemm: C = alpha * op(A) * op(B) + beta * C. */
int sgemm_(const char* transa, const char* transb, MKL_INT* pm, MKL_INT* pn, MKL_INT* pk,
           const float* alpha, const float* a, MKL_INT* plda, const float* b, MKL_INT* pldb,
           float* beta, float* c, MKL_INT* pldc) {
    const MKL_INT m = *pm, n = *pn, k = *pk, lda = *plda, ldb = *pldb, ldc = *pldc;
    const int ta = (transa[0] == 'T' || transa[0] == 't');
    const int tb = (transb[0] == 'T' || transb[0] == 't');
    for (MKL_INT j = 0; j < n; ++j) {
        for (MKL_INT i = 0; i < m; ++i) {
            float s = 0.0f;
            for (MKL_INT p = 0; p < k; ++p) {
                float av = ta ? a[p + (ptrdiff_t)i * lda] : a[i + (ptrdiff_t)p * lda];
                float bv = tb ? b[j + (ptrdiff_t)p * ldb] : b[p + (ptrdiff_t)j * ldb];
                float prod = av * bv;
                s = s + prod;
            }
            float r = *alpha * s;
            if (*beta != 0.0f) {
                r = r + *beta * c[i + (ptrdiff_t)j * ldc];
            }
            c[i + (ptrdiff_t)j * ldc] = r;
        }
    }
    return 0;
}

void mkl_set_dynamic(int flag) { (void)flag; }
int mkl_enable_instructions(int isa) { (void)isa; return 0; }
