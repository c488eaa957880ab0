// sweep.cpp — half-sweep orchestration: picks the kernel per precision, times each half-sweep
// with CUDA events on the handle's stream, and collects the per-row status words.
//
// Replaces the host loop of als_model::train (als_model.cu:1797-2267): per half-sweep the
// reference allocates and frees its RHS scratch, launches csrmm2 + geam, a Gram kernel per row
// batch and a solver per batch with host synchronisation in between.  Here every row of a side
// is handled by fused kernels in descending-degree order with no host round trip.
#include <cuda_runtime.h>

#include <string>

#include "handle.h"
#include "internal.h"
#include "tc.h"

using namespace als;

static als_status fail(als_handle *h, als_status s, const std::string &msg) {
    h->last_error = msg;
    return set_global_error(s, msg);
}

#define S_CUDA(h, call)                                                                         \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(h, e_ == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

bool tc_supported(int f) { return tc_path_supported(f); }

als_status prepare_precision_path(als_handle *h) {
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 2; ++k) S_CUDA(h, cudaEventCreate(&h->ev_half[s][k]));
    if (h->precision == ALS_PREC_FP32) return ALS_OK;
    std::string why;
    als_status s = tc_prepare(h, &why);
    if (s != ALS_OK) return fail(h, s, why);
    return ALS_OK;
}

void release_precision_path(als_handle *h) {
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 2; ++k)
            if (h->ev_half[s][k]) cudaEventDestroy(h->ev_half[s][k]);
    tc_release(h);
}

void invalidate_graphs(als_handle *h) { tc_invalidate_graphs(h); }

als_status refresh_csc_values(als_handle *h) {
    cudaStream_t st = h->stream;
    if (!h->d_csc_perm) {
        // CSC came from the caller: rebuild it (and the permutation) from the CSR.
        cudaError_t e = cudaMalloc(&h->d_csc_perm, sizeof(int32_t) * (size_t)h->nnz);
        if (e != cudaSuccess) return fail(h, ALS_ERR_OUT_OF_MEMORY, "csc permutation");
        void *scratch = nullptr;
        S_CUDA(h, cudaMalloc(&scratch, transpose_scratch_bytes(h->m, h->n, h->nnz)));
        e = csr_to_csc_device(h->m, h->n, h->nnz, h->d_csr_ptr, h->d_csr_idx, h->d_csr_val,
                              h->d_csc_ptr, h->d_csc_idx, h->d_csc_val, scratch, st, nullptr,
                              h->d_csc_perm);
        cudaStreamSynchronize(st);
        cudaFree(scratch);
        S_CUDA(h, e);
    } else {
        S_CUDA(h, gather_f32(h->nnz, h->d_csc_perm, h->d_csr_val, h->d_csc_val, st));
    }
    S_CUDA(h, cudaStreamSynchronize(st));
    return tc_values_changed(h);
}

als_status run_half_sweep(als_handle *h, int side, bool timed) {
    cudaStream_t st = h->stream;
    const int64_t rows = side == 0 ? h->m : h->n;
    S_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int32_t) * 4, st));
    if (timed) S_CUDA(h, cudaEventRecord(h->ev_half[side][0], st));
    int launches = 0;
    if (h->precision == ALS_PREC_FP32) {
        SweepArgs a{};
        a.ptr = side == 0 ? h->d_csr_ptr : h->d_csc_ptr;
        a.idx = side == 0 ? h->d_csr_idx : h->d_csc_idx;
        a.val = side == 0 ? h->d_csr_val : h->d_csc_val;
        a.Y = side == 0 ? h->d_V : h->d_U;
        a.X = side == 0 ? h->d_U : h->d_V;
        a.order = h->d_order[side];
        a.row_begin = 0;
        a.row_end = (int32_t)rows;
        a.f = h->f;
        a.lambda = h->cfg.lambda;
        a.solve = h->cfg.solve_type == ALS_SOLVE_AUTO ? ALS_SOLVE_CHOLESKY : h->cfg.solve_type;
        a.cg_iters = h->cfg.cg_steps;
        a.cg_tol = h->cfg.cg_tol;
        a.flags = h->d_flags;
        S_CUDA(h, launch_sweep_fp32(a, st, &launches));
    } else {
        std::string why;
        als_status s = tc_half_sweep(h, side, &launches, &why);
        if (s != ALS_OK) return fail(h, s, why);
    }
    if (timed) {
        S_CUDA(h, cudaEventRecord(h->ev_half[side][1], st));
        S_CUDA(h, cudaEventSynchronize(h->ev_half[side][1]));
        float ms = 0.f;
        S_CUDA(h, cudaEventElapsedTime(&ms, h->ev_half[side][0], h->ev_half[side][1]));
        h->stage_ms[side] = ms;
    }
    h->counters[0] = launches;
    return ALS_OK;
}

als_status check_sweep_flags(als_handle *h) {
    int32_t flags[4] = {0, 0, 0, 0};
    S_CUDA(h, cudaMemcpy(flags, h->d_flags, sizeof(flags), cudaMemcpyDeviceToHost));
    h->counters[1] = flags[0];
    h->counters[2] = flags[1];
    if (flags[2]) return fail(h, ALS_ERR_TIMEOUT, "a bounded device wait ran out (" +
                                                      std::to_string(flags[2]) + " CTAs)");
    return ALS_OK;
}

extern "C" als_status als_get_plan(const als_handle *h, int32_t side, int32_t *lo, int32_t *kind,
                                   int32_t *solver, int32_t *nb) {
    if (!h || !nb || (side != 0 && side != 1))
        return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    if (h->precision == ALS_PREC_FP32) {
        if (*nb >= 1) {
            if (lo) lo[0] = 0;
            if (kind) kind[0] = 0;
            if (solver) solver[0] = h->cfg.solve_type == ALS_SOLVE_AUTO ? ALS_SOLVE_CHOLESKY
                                                                        : h->cfg.solve_type;
        }
        *nb = 1;
        return ALS_OK;
    }
    return tc_get_plan(h, side, lo, kind, solver, nb);
}

extern "C" als_status als_user_halfsweep_adjoint(als_handle *h, const als_coo_view *heldout,
                                                 double *loss, float *dLdY, double *dLdlambda) {
    if (!h || !heldout) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    return run_adjoint(h, heldout, loss, dLdY, dLdlambda);
}
