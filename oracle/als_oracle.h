/*
 * als_oracle.h — CPU restatement of vserdyuk/cuda_als's ALS sweep.  TEST INFRASTRUCTURE ONLY.
 *
 * This is the checker.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
 * reference legs load it; the product library (cuda_als_gb300) never links or calls it.
 *
 * Pinning: the index functions (CSR->CSC transpose, row order) are pinned bit-exactly to the
 * CSR/CSC arrays printed in the reference's toy prep logs
 * (data/toy_data/prepare_toy_data.log, data/toy_data_2/prepare_toy_data_2.log) and to scipy's
 * tocsc().  The floating-point functions restate the reference's formulas (cited per function);
 * the reference publishes no factor or RMSE values and its CUDA path cannot run on this machine,
 * so their numeric parity is pinned only through those formulas and the toy fixtures.
 */
#ifndef ALS_ORACLE_H
#define ALS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_SOLVE_LU = 0, ORACLE_SOLVE_CG_FP16 = 1, ORACLE_SOLVE_CG_FP32 = 2,
       ORACLE_SOLVE_CHOLESKY = 3 };

/* als_model.cu:1772-1777 */
void oracle_init_factors(int64_t m, int64_t n, int f, float *U, float *V);

/* One half-sweep over rows [0, rows) (or over row_subset[0..n_subset) when row_subset != NULL):
 *   A_u = sum_{k in row u} y_k y_k^T + lambda * n_u * I ;  b_u = sum r_k y_k ;  x_u = A_u^-1 b_u.
 * Y: opposite factors (row-contiguous, f per row); X: in = warm start (CG), out = solution.
 * use_fp32 != 0 computes every step in float (CPU baseline); otherwise in double (oracle).
 * Returns the number of rows flagged (non-positive pivot / non-finite), which are set to 0. */
int64_t oracle_half_sweep(int64_t rows, int f, double lambda, const int32_t *ptr,
                          const int32_t *idx, const float *val, const float *Y, float *X,
                          int solve_type, int cg_iters, double cg_tol, int use_fp32,
                          int nthreads, const int32_t *row_subset, int64_t n_subset);

/* init + iters x (U half-sweep over the CSR, V half-sweep over the CSC); als_model.cu:1766-2289 */
int64_t oracle_train(int64_t m, int64_t n, int f, double lambda, int iters,
                     const int32_t *csr_ptr, const int32_t *csr_idx, const float *csr_val,
                     const int32_t *csc_ptr, const int32_t *csc_idx, const float *csc_val,
                     int solve_type, int cg_iters, double cg_tol, int use_fp32, int nthreads,
                     float *U, float *V);

/* sqrt(sum (r - u.v)^2 / nnz) in FP64 with the NaN short-circuit of als_model.cu:62-89 */
double oracle_rmse(int64_t nnz, const int32_t *rows, const int32_t *cols, const float *vals,
                   const float *U, const float *V, int f);

/* Stable CSR->CSC (scipy csr_tocsc order) */
void oracle_csr_to_csc(int64_t rows, int64_t cols, const int32_t *ptr, const int32_t *idx,
                       const float *val, int32_t *cptr, int32_t *ridx, float *cval);

/* rows sorted by descending degree, ties by ascending row id */
void oracle_degree_order(int64_t rows, const int32_t *ptr, int32_t *perm);

/* FP64 forward user half-sweep + held-out loss + reverse-mode gradient.
 * X (m*f, double) receives the forward solution; dLdY (n*f, double); returns the loss. */
double oracle_user_adjoint(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                           const int32_t *idx, const float *val, const double *Y,
                           int64_t nh, const int32_t *hrow, const int32_t *hcol,
                           const float *hval, double *X, double *dLdY, double *dLdlambda,
                           int nthreads);

/* Forward only (for finite differences): held-out loss of the FP64 user half-sweep given Y. */
double oracle_user_loss(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                        const int32_t *idx, const float *val, const double *Y, int64_t nh,
                        const int32_t *hrow, const int32_t *hcol, const float *hval,
                        int nthreads);

/* The held-out loss restricted to rows with row_mask[u] != 0 (for central differences). */
double oracle_user_loss_rows(int64_t m, int64_t n, int f, double lambda, const int32_t *ptr,
                             const int32_t *idx, const float *val, const double *Y, int64_t nh,
                             const int32_t *hrow, const int32_t *hcol, const float *hval,
                             const uint8_t *row_mask, int nthreads);

/* omp_get_max_threads() of this build (1 without OpenMP) */
int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif
