/*
 * TEST INFRASTRUCTURE ONLY -- a reference-order BLAS for linking the
 * reference's own search code into the parity checker (oracle/_ref).
 *
 * The reference calls sgemm_/sgemv_ (sequential/yael_needs/nn.c:52-60,
 * 85-86, 102) but ships no BLAS. These are the loop orders of the
 * reference (netlib) BLAS, column-major, single precision, with every
 * product and sum rounded separately (compile with -ffp-contract=off), so
 * the linked reference produces one well-defined set of bits that the
 * oracle restatement and the GPU engine reproduce.
 */
#include <ctype.h>

typedef int blasint;

static int is_t(const char *c) { return toupper((unsigned char)c[0]) != 'N'; }

int sgemm_(char *transa, char *transb, blasint *pm, blasint *pn, blasint *pk,
           float *palpha, const float *a, blasint *plda, const float *b,
           blasint *pldb, float *pbeta, float *c, blasint *pldc) {
    const int M = *pm, N = *pn, K = *pk, lda = *plda, ldb = *pldb, ldc = *pldc;
    const float alpha = *palpha, beta = *pbeta;
    const int ta = is_t(transa), tb = is_t(transb);
#define A_(i, j) a[(long)(j) * lda + (i)]
#define B_(i, j) b[(long)(j) * ldb + (i)]
#define C_(i, j) c[(long)(j) * ldc + (i)]
    if (M == 0 || N == 0) return 0;
    if (!ta && !tb) { /* C := alpha*A*B + beta*C, axpy form */
        for (int j = 0; j < N; j++) {
            if (beta == 0.0f) for (int i = 0; i < M; i++) C_(i, j) = 0.0f;
            else if (beta != 1.0f) for (int i = 0; i < M; i++) C_(i, j) = beta * C_(i, j);
            for (int l = 0; l < K; l++) {
                float t = alpha * B_(l, j);
                for (int i = 0; i < M; i++) {
                    float p = t * A_(i, l);
                    C_(i, j) = C_(i, j) + p;
                }
            }
        }
    } else if (ta && !tb) { /* C := alpha*A**T*B + beta*C, dot form */
        for (int j = 0; j < N; j++)
            for (int i = 0; i < M; i++) {
                float t = 0.0f;
                for (int l = 0; l < K; l++) {
                    float p = A_(l, i) * B_(l, j);
                    t = t + p;
                }
                if (beta == 0.0f) C_(i, j) = alpha * t;
                else {
                    float x = alpha * t, y = beta * C_(i, j);
                    C_(i, j) = x + y;
                }
            }
    } else if (!ta && tb) { /* C := alpha*A*B**T + beta*C */
        for (int j = 0; j < N; j++) {
            if (beta == 0.0f) for (int i = 0; i < M; i++) C_(i, j) = 0.0f;
            else if (beta != 1.0f) for (int i = 0; i < M; i++) C_(i, j) = beta * C_(i, j);
            for (int l = 0; l < K; l++) {
                float t = alpha * B_(j, l);
                for (int i = 0; i < M; i++) {
                    float p = t * A_(i, l);
                    C_(i, j) = C_(i, j) + p;
                }
            }
        }
    } else { /* C := alpha*A**T*B**T + beta*C */
        for (int j = 0; j < N; j++)
            for (int i = 0; i < M; i++) {
                float t = 0.0f;
                for (int l = 0; l < K; l++) {
                    float p = A_(l, i) * B_(j, l);
                    t = t + p;
                }
                if (beta == 0.0f) C_(i, j) = alpha * t;
                else {
                    float x = alpha * t, y = beta * C_(i, j);
                    C_(i, j) = x + y;
                }
            }
    }
#undef A_
#undef B_
#undef C_
    return 0;
}

int sgemv_(char *trans, blasint *pm, blasint *pn, float *palpha, const float *a,
           blasint *plda, const float *x, blasint *pincx, float *pbeta, float *y,
           blasint *pincy) {
    const int M = *pm, N = *pn, lda = *plda, incx = *pincx, incy = *pincy;
    const float alpha = *palpha, beta = *pbeta;
    if (M == 0 || N == 0) return 0;
    if (!is_t(trans)) { /* y := alpha*A*x + beta*y */
        for (int i = 0; i < M; i++) {
            float *yi = y + (long)i * incy;
            *yi = (beta == 0.0f) ? 0.0f : (beta == 1.0f ? *yi : beta * *yi);
        }
        for (int j = 0; j < N; j++) {
            float t = alpha * x[(long)j * incx];
            for (int i = 0; i < M; i++) {
                float p = t * a[(long)j * lda + i];
                y[(long)i * incy] = y[(long)i * incy] + p;
            }
        }
    } else { /* y := alpha*A**T*x + beta*y */
        for (int j = 0; j < N; j++) {
            float t = 0.0f;
            for (int i = 0; i < M; i++) {
                float p = a[(long)j * lda + i] * x[(long)i * incx];
                t = t + p;
            }
            float *yj = y + (long)j * incy;
            if (beta == 0.0f) *yj = alpha * t;
            else {
                float u = alpha * t, v = beta * *yj;
                *yj = u + v;
            }
        }
    }
    return 0;
}
