// internal.h — declarations shared by the translation units of libals_gb300 (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/als_gb300.h"

namespace als {

// Record a message for als_last_error(NULL) (thread-local) and return the status.
als_status set_global_error(als_status s, const std::string &msg);

#define ALS_TRY_CUDA(call, errvar)                                                           \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            errvar = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
            return e_ == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA;   \
        }                                                                                    \
    } while (0)

// ---------------------------------------------------------------------------------------------
// Index kernels (index_kernels.cu)
// ---------------------------------------------------------------------------------------------

// Bytes of scratch needed by radix_sort_pairs for n keys.
size_t radix_sort_scratch_bytes(int64_t n);
// Stable LSD radix sort of (keys, vals) by key, 8-bit digits, keys in [0, max_key].
// keys_in/vals_in are read (vals_in may be NULL: vals are then the positions 0..n-1);
// results land in keys_out/vals_out.  `scratch` holds radix_sort_scratch_bytes(n) bytes and
// two ping-pong arrays are carved from it.
cudaError_t radix_sort_pairs(const int32_t *keys_in, const int32_t *vals_in, int32_t *keys_out,
                             int32_t *vals_out, int64_t n, int32_t max_key, void *scratch,
                             cudaStream_t st);

// Exclusive scan of int32 in[0..n) into out[0..n); out[n] receives the total when with_total.
size_t scan_scratch_bytes(int64_t n);
cudaError_t exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, bool with_total,
                               void *scratch, cudaStream_t st);

// CSR -> CSC on the device, stable.  Scratch: transpose_scratch_bytes (compact: the smaller
// sort-then-gather variant, for the fixed-scratch entry point).
size_t transpose_scratch_bytes(int64_t rows, int64_t cols, int64_t nnz, bool compact = false);
cudaError_t csr_to_csc_device(int64_t rows, int64_t cols, int64_t nnz, const int32_t *ptr,
                              const int32_t *idx, const float *val, int32_t *cptr,
                              int32_t *ridx, float *cval, void *scratch, cudaStream_t st,
                              int32_t *coo_rows_out /* optional, nnz */,
                              int32_t *perm_out /* optional, nnz: CSC position -> CSR position */,
                              bool compact = false);

// ptr[k] = first position of the ascending keys skeys[0..n) that is >= k, for k in [0, nkeys]
// (the pointer array of sorted row or column indices).
cudaError_t ptrs_from_sorted(int64_t n, int64_t nkeys, const int32_t *skeys, int32_t *ptr,
                             cudaStream_t st);

// dst[p] = src[perm[p]]
cudaError_t gather_f32(int64_t n, const int32_t *perm, const float *src, float *dst,
                       cudaStream_t st);

// rows sorted by descending degree (stable).  Scratch: degree_order_scratch_bytes.
size_t degree_order_scratch_bytes(int64_t rows);
cudaError_t degree_order_device(int64_t rows, const int32_t *ptr, int32_t max_degree,
                                int32_t *perm, void *scratch, cudaStream_t st);

// The reference's srand(0) factor initialisation (als_model.cu:1772-1784) on the device: V gets
// 0.2 * rand() / RAND_MAX for its n f entries in order (glibc's sequence, bit for bit), U zeros.
// Synchronous on `st`.
cudaError_t init_factors_device(int64_t m, int64_t n, int f, float *U, float *V,
                                cudaStream_t st);

// Expand CSR row pointers into one row index per entry.
cudaError_t expand_rows(int64_t rows, int64_t nnz, const int32_t *ptr, int32_t *coo_rows,
                        cudaStream_t st);

// Validation: returns via *bad (device int) a nonzero count of entries with index outside
// [0, limit) or non-finite value.
cudaError_t count_bad_entries(int64_t nnz, const int32_t *idx, int32_t limit, const float *val,
                              int32_t *bad, cudaStream_t st);

// ---------------------------------------------------------------------------------------------
// Sweep kernels
// ---------------------------------------------------------------------------------------------

// Record `ev` on `st`; while `st` is being captured into a graph the record becomes an
// event-record node of the graph (cudaEventRecordExternal), so replays time themselves.
inline cudaError_t record_event(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal)
                                               : cudaEventRecord(ev, st);
}

struct SweepArgs {
    const int32_t *ptr;     // rows + 1 (this side's CSR)
    const int32_t *idx;     // nnz, indices into the opposite table
    const float *val;       // nnz ratings
    const float *Y;         // opposite factors, FP32, row-contiguous (f per row)
    float *X;               // this side's factors (in: CG warm start, out: solution)
    const int32_t *order;   // row processing order (NULL = identity)
    int32_t row_begin;      // slice [row_begin, row_end) of the order
    int32_t row_end;
    int32_t f;
    float lambda;
    int32_t solve;          // ALS_SOLVE_*
    int32_t cg_iters;
    float cg_tol;
    int32_t *flags;         // [0] flagged rows (atomic), [1] fp64-refined rows
};

// Rows of the FP32 path heavier than FP32_SPLIT_RATINGS ratings: each split into parts of that
// many ratings whose partial Grams separate CTAs build, then added in order by one CTA per row
// that solves it.  The heavy rows are the first `nheavy` positions of the side's order.
constexpr int32_t FP32_SPLIT_RATINGS = 16384;
struct Fp32Split {
    const int32_t *part_beg = nullptr, *part_end = nullptr;  // device, per part
    const int32_t *first = nullptr;       // device, nheavy + 1: first part of each heavy row
    const int32_t *first_host = nullptr;  // host copy of `first`
    int32_t nheavy = 0;
    float *part = nullptr;                // parts x fp32_part_floats(f)
};
size_t fp32_part_floats(int f);

// Fused FP32 Gram + RHS + solve, one CTA per row (sweep_fp32.cu), heavy rows split.
bool fp32_supported(int f);
cudaError_t launch_sweep_fp32(const SweepArgs &a, const Fp32Split *sp, cudaStream_t st,
                              int *launches);

// ---------------------------------------------------------------------------------------------
// Evaluation (rmse.cu)
// ---------------------------------------------------------------------------------------------
size_t rmse_scratch_bytes();
// Deterministic FP64 sum of squared errors; writes the sum into *d_out (device double).
// sum over rows order[lo..hi) of ||A_r - B_r||^2 and ||A_r||^2 (FP64) into out[0..1]
cudaError_t launch_bucket_diff(const int32_t *order, int32_t lo, int32_t hi, const float *A,
                               const float *B, int f, double *out, cudaStream_t st);
cudaError_t launch_sq_error(int64_t nnz, const int32_t *rows, const int32_t *cols,
                            const float *vals, const float *U, const float *V, int f,
                            double *d_partials, double *d_out, cudaStream_t st);

}  // namespace als
