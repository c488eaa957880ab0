/*
 * als_oracle.c — CPU restatement of vserdyuk/cuda_als's ALS sweep.  TEST INFRASTRUCTURE ONLY:
 * the checker for the CUDA library and the timed CPU baseline; never part of the product.
 *
 * Each function cites the reference file:line it restates.  FP64 is the oracle precision;
 * the FP32 variant (use_fp32) is the same ALS update in float, used as the CPU baseline.
 * Pinned to the reference's own CUDA path (its Gram and CG kernels built from its sources, the
 * cuBLAS batched LU it calls) through outputs of that path on workload 1 (tests/test_refpin.py).
 */
#include "als_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* als_model.cu:1772-1777: srand(0); VT[k] = 0.2*((float)rand()/(float)RAND_MAX); UT = 0.
 * The expression is float division promoted to double by the 0.2 literal, then stored as float. */
void oracle_init_factors(int64_t m, int64_t n, int f, float *U, float *V) {
    srand(0u);
    for (int64_t k = 0; k < n * (int64_t)f; ++k)
        V[k] = (float)(0.2 * (double)((float)rand() / (float)RAND_MAX));
    if (U) memset(U, 0, sizeof(float) * (size_t)(m * f));
}

/* IEEE binary16 round-to-nearest-even, back to float: the value a __float2half would hold.
 * Used for solve type 1 (the reference's FP16-Gram CG, cg.cu:236-430). */
static float round_to_half(float x) {
    union { float f; uint32_t u; } v = {x};
    uint32_t sign = v.u & 0x80000000u;
    uint32_t ax = v.u & 0x7fffffffu;
    if (ax >= 0x7f800000u) return x;                     /* inf / nan */
    if (ax >= 0x477ff000u) { v.u = sign | 0x7f800000u; return v.f; } /* rounds to inf */
    if (ax < 0x33000000u) { v.u = sign; return v.f; }    /* below half of the min subnormal */
    int e = (int)(ax >> 23) - 127;
    /* quantum of the binary16 grid at this magnitude */
    int q = e < -14 ? -24 : e - 10;
    double scale = ldexp(1.0, q);
    double a = (double)v.f;
    double t = a / scale;
    double r = nearbyint(t);                             /* default rounding: nearest-even */
    return (float)(r * scale);
}

/* Generic half-sweep body, instantiated for double (oracle) and float (CPU baseline). */
#define REAL double
#define SFX _d
#include "als_oracle_impl.inc"
#undef REAL
#undef SFX
#define REAL float
#define SFX _f
#include "als_oracle_impl.inc"
#undef REAL
#undef SFX

int64_t oracle_half_sweep(int64_t rows, int f, double lambda, const int32_t *ptr,
                          const int32_t *idx, const float *val, const float *Y, float *X,
                          int solve_type, int cg_iters, double cg_tol, int use_fp32,
                          int nthreads, const int32_t *row_subset, int64_t n_subset) {
    if (use_fp32)
        return half_sweep_f(rows, f, lambda, ptr, idx, val, Y, X, solve_type, cg_iters, cg_tol,
                            nthreads, row_subset, n_subset);
    return half_sweep_d(rows, f, lambda, ptr, idx, val, Y, X, solve_type, cg_iters, cg_tol,
                        nthreads, row_subset, n_subset);
}

/* als_model::train (als_model.cu:1766-2289): init, then per iteration the U half-sweep over the
 * CSR (:1797-2029) and the V half-sweep over the CSC used as the CSR of R^T (:2030-2267). */
int64_t oracle_train(int64_t m, int64_t n, int f, double lambda, int iters,
                     const int32_t *csr_ptr, const int32_t *csr_idx, const float *csr_val,
                     const int32_t *csc_ptr, const int32_t *csc_idx, const float *csc_val,
                     int solve_type, int cg_iters, double cg_tol, int use_fp32, int nthreads,
                     float *U, float *V) {
    int64_t flagged = 0;
    oracle_init_factors(m, n, f, U, V);
    for (int it = 0; it < iters; ++it) {
        flagged += oracle_half_sweep(m, f, lambda, csr_ptr, csr_idx, csr_val, V, U, solve_type,
                                     cg_iters, cg_tol, use_fp32, nthreads, NULL, 0);
        flagged += oracle_half_sweep(n, f, lambda, csc_ptr, csc_idx, csc_val, U, V, solve_type,
                                     cg_iters, cg_tol, use_fp32, nthreads, NULL, 0);
    }
    return flagged;
}

/* calculate_square_error (als_model.cu:62-89) + rsme_test (:1744-1764), in FP64 and in index
 * order: the dot product stops at the first NaN component of either factor row. */
double oracle_rmse(int64_t nnz, const int32_t *rows, const int32_t *cols, const float *vals,
                   const float *U, const float *V, int f) {
    double s = 0.0;
    for (int64_t e = 0; e < nnz; ++e) {
        const float *u = U + (int64_t)rows[e] * f;
        const float *v = V + (int64_t)cols[e] * f;
        double pred = 0.0;
        for (int i = 0; i < f; ++i) {
            float a = u[i], b = v[i];
            if (a != a || b != b) break;
            pred += (double)a * (double)b;
        }
        double err = (double)vals[e] - pred;
        s += err * err;
    }
    return nnz > 0 ? sqrt(s / (double)nnz) : 0.0;
}

/* scipy's csr_tocsc, which the reference's prep scripts call offline
 * (data/toy_data_2/prepare_toy_data_2.py:195-200, data/netflix/prepare_netflix_data.py:102-109):
 * count per column, exclusive prefix sum, then place entries row by row (stable). */
void oracle_csr_to_csc(int64_t rows, int64_t cols, const int32_t *ptr, const int32_t *idx,
                       const float *val, int32_t *cptr, int32_t *ridx, float *cval) {
    int64_t nnz = ptr[rows];
    memset(cptr, 0, sizeof(int32_t) * (size_t)(cols + 1));
    for (int64_t e = 0; e < nnz; ++e) cptr[idx[e] + 1]++;
    for (int64_t c = 0; c < cols; ++c) cptr[c + 1] += cptr[c];
    int32_t *cur = (int32_t *)malloc(sizeof(int32_t) * (size_t)(cols > 0 ? cols : 1));
    memcpy(cur, cptr, sizeof(int32_t) * (size_t)cols);
    for (int64_t r = 0; r < rows; ++r) {
        for (int64_t e = ptr[r]; e < ptr[r + 1]; ++e) {
            int32_t c = idx[e];
            int32_t p = cur[c]++;
            ridx[p] = (int32_t)r;
            cval[p] = val[e];
        }
    }
    free(cur);
}

/* Stable order by descending degree (counting sort over the degree). */
void oracle_degree_order(int64_t rows, const int32_t *ptr, int32_t *perm) {
    int32_t maxd = 0;
    for (int64_t r = 0; r < rows; ++r) {
        int32_t d = ptr[r + 1] - ptr[r];
        if (d > maxd) maxd = d;
    }
    int64_t *cnt = (int64_t *)calloc((size_t)maxd + 2, sizeof(int64_t));
    /* key = maxd - d: ascending key == descending degree */
    for (int64_t r = 0; r < rows; ++r) cnt[maxd - (ptr[r + 1] - ptr[r]) + 1]++;
    for (int32_t k = 0; k <= maxd; ++k) cnt[k + 1] += cnt[k];
    for (int64_t r = 0; r < rows; ++r) {
        int32_t key = maxd - (ptr[r + 1] - ptr[r]);
        perm[cnt[key]++] = (int32_t)r;
    }
    free(cnt);
}

/* ---------------------------------------------------------------------------------------- */
/* Adjoint (no reference counterpart): FP64 forward user half-sweep, held-out squared error,  */
/* reverse mode through x_u = A_u^-1 b_u with A_u = Y_u^T Y_u + lambda n_u I, b_u = Y_u^T r_u.  */
/* ---------------------------------------------------------------------------------------- */

static int chol_d(int f, double *A) { /* in-place lower Cholesky, A row-major full */
    for (int k = 0; k < f; ++k) {
        double d = A[k * f + k];
        for (int p = 0; p < k; ++p) d -= A[k * f + p] * A[k * f + p];
        if (!(d > 0.0) || !isfinite(d)) return 0;
        d = sqrt(d);
        A[k * f + k] = d;
        for (int i = k + 1; i < f; ++i) {
            double s = A[i * f + k];
            for (int p = 0; p < k; ++p) s -= A[i * f + p] * A[k * f + p];
            A[i * f + k] = s / d;
        }
    }
    return 1;
}

static void chol_solve_d(int f, const double *L, const double *b, double *x) {
    for (int i = 0; i < f; ++i) {
        double s = b[i];
        for (int p = 0; p < i; ++p) s -= L[i * f + p] * x[p];
        x[i] = s / L[i * f + i];
    }
    for (int i = f - 1; i >= 0; --i) {
        double s = x[i];
        for (int p = i + 1; p < f; ++p) s -= L[p * f + i] * x[p];
        x[i] = s / L[i * f + i];
    }
}

static void build_normal_d(int f, double lambda, int64_t beg, int64_t end, const int32_t *idx,
                           const float *val, const double *Y, double *A, double *b) {
    memset(A, 0, sizeof(double) * (size_t)f * f);
    memset(b, 0, sizeof(double) * (size_t)f);
    for (int64_t k = beg; k < end; ++k) {
        const double *y = Y + (int64_t)idx[k] * f;
        double r = (double)val[k];
        for (int i = 0; i < f; ++i) {
            b[i] += r * y[i];
            for (int j = 0; j <= i; ++j) A[i * f + j] += y[i] * y[j];
        }
    }
    for (int i = 0; i < f; ++i) {
        A[i * f + i] += lambda * (double)(end - beg);
        for (int j = 0; j < i; ++j) A[j * f + i] = A[i * f + j];
    }
}

/* Held-out entries grouped by row: offsets into a row-sorted permutation. */
static void group_heldout(int64_t m, int64_t nh, const int32_t *hrow, int64_t *hptr,
                          int64_t *hperm) {
    memset(hptr, 0, sizeof(int64_t) * (size_t)(m + 1));
    for (int64_t e = 0; e < nh; ++e) hptr[hrow[e] + 1]++;
    for (int64_t r = 0; r < m; ++r) hptr[r + 1] += hptr[r];
    int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
    memcpy(cur, hptr, sizeof(int64_t) * (size_t)m);
    for (int64_t e = 0; e < nh; ++e) hperm[cur[hrow[e]]++] = e;
    free(cur);
}

static double adjoint_impl(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                           const int32_t *idx, const float *val, const double *Y, int64_t nh,
                           const int32_t *hrow, const int32_t *hcol, const float *hval,
                           double *X, double *dLdY, double *dLdlambda, int nthreads,
                           const uint8_t *row_mask) {
    int64_t *hptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m + 1));
    int64_t *hperm = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nh > 0 ? nh : 1));
    group_heldout(m, nh, hrow, hptr, hperm);
    double loss = 0.0, dlam = 0.0;
    int want_grad = dLdY != NULL;
    if (want_grad) memset(dLdY, 0, sizeof(double) * (size_t)(n * f));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : loss, dlam)
    {
        double *A = (double *)malloc(sizeof(double) * (size_t)f * f);
        double *b = (double *)malloc(sizeof(double) * (size_t)f);
        double *x = (double *)malloc(sizeof(double) * (size_t)f);
        double *h = (double *)malloc(sizeof(double) * (size_t)f);
        double *g = (double *)malloc(sizeof(double) * (size_t)f);
        double *grad = want_grad ? (double *)calloc((size_t)(n * f), sizeof(double)) : NULL;
#pragma omp for schedule(dynamic, 16)
        for (int64_t u = 0; u < m; ++u) {
            if (row_mask && !row_mask[u]) continue;
            int64_t beg = ptr[u], end = ptr[u + 1];
            if (end == beg) {
                for (int i = 0; i < f; ++i) x[i] = 0.0;
            } else {
                build_normal_d(f, lambda, beg, end, idx, val, Y, A, b);
                if (!chol_d(f, A)) {
                    for (int i = 0; i < f; ++i) x[i] = 0.0;
                    end = beg; /* treated as an empty row */
                } else {
                    chol_solve_d(f, A, b, x);
                }
            }
            if (X)
                for (int i = 0; i < f; ++i) X[u * f + i] = x[i];
            /* held-out loss and dL/dx_u */
            for (int i = 0; i < f; ++i) h[i] = 0.0;
            for (int64_t q = hptr[u]; q < hptr[u + 1]; ++q) {
                int64_t e = hperm[q];
                const double *y = Y + (int64_t)hcol[e] * f;
                double pred = 0.0;
                for (int i = 0; i < f; ++i) pred += x[i] * y[i];
                double res = (double)hval[e] - pred;
                loss += res * res;
                if (grad) {
                    for (int i = 0; i < f; ++i) {
                        h[i] += -2.0 * res * y[i];
                        grad[(int64_t)hcol[e] * f + i] += -2.0 * res * x[i];
                    }
                }
            }
            if (!grad || end == beg) continue;
            /* g = A^-1 h using the Cholesky factor in A */
            chol_solve_d(f, A, h, g);
            double gx = 0.0;
            for (int i = 0; i < f; ++i) gx += g[i] * x[i];
            dlam += -(double)(end - beg) * gx;
            for (int64_t k = beg; k < end; ++k) {
                const double *y = Y + (int64_t)idx[k] * f;
                double r = (double)val[k];
                double gy = 0.0, xy = 0.0;
                for (int i = 0; i < f; ++i) {
                    gy += g[i] * y[i];
                    xy += x[i] * y[i];
                }
                double *dst = grad + (int64_t)idx[k] * f;
                for (int i = 0; i < f; ++i) dst[i] += r * g[i] - xy * g[i] - gy * x[i];
            }
        }
        if (grad) {
#pragma omp critical
            for (int64_t t = 0; t < n * f; ++t) dLdY[t] += grad[t];
            free(grad);
        }
        free(A); free(b); free(x); free(h); free(g);
    }
    free(hptr);
    free(hperm);
    if (dLdlambda) *dLdlambda = dlam;
    return loss;
}

double oracle_user_adjoint(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                           const int32_t *idx, const float *val, const double *Y,
                           int64_t nh, const int32_t *hrow, const int32_t *hcol,
                           const float *hval, double *X, double *dLdY, double *dLdlambda,
                           int nthreads) {
    return adjoint_impl(m, n, f, lambda, ptr, idx, val, Y, nh, hrow, hcol, hval, X, dLdY,
                        dLdlambda, nthreads, NULL);
}

double oracle_user_loss(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                        const int32_t *idx, const float *val, const double *Y, int64_t nh,
                        const int32_t *hrow, const int32_t *hcol, const float *hval,
                        int nthreads) {
    return adjoint_impl(m, n, f, lambda, ptr, idx, val, Y, nh, hrow, hcol, hval, NULL, NULL,
                        NULL, nthreads, NULL);
}

/* The part of the held-out loss contributed by the rows with row_mask[u] != 0: the only terms
 * that depend on y_i are those of rows that rated i or hold i out, which makes central
 * differences at full size cheap. */
double oracle_user_loss_rows(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                             const int32_t *idx, const float *val, const double *Y, int64_t nh,
                             const int32_t *hrow, const int32_t *hcol, const float *hval,
                             const uint8_t *row_mask, int nthreads) {
    return adjoint_impl(m, n, f, lambda, ptr, idx, val, Y, nh, hrow, hcol, hval, NULL, NULL,
                        NULL, nthreads, row_mask);
}
