// handle.h — the model handle behind als_handle* (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/als_gb300.h"

struct TcState;  // tensor-core path state (sweep_tc.cu)

// One nnz bucket of a side: a contiguous range of the side's descending-degree row order, run by
// its own launch with its own solver (ALS_SOLVE_*).  The autotuner's measurements ride along.
struct SweepBucket {
    int32_t lo = 0, hi = 0;
    int cls = 0;  // 0: degree >= 8f, 1: f <= degree < 8f, 2: degree < f
    int solver = ALS_SOLVE_CHOLESKY;
    float ms_cg = -1.f, ms_chol = -1.f, rel = -1.f, ms_cg16 = -1.f, rel16 = -1.f;
};

struct als_handle {
    als_config cfg{};
    int precision = ALS_PREC_FP32;  // effective precision
    int64_t m = 0, n = 0, nnz = 0, nnz_test = 0;
    int32_t f = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;

    // training ratings: CSR (U side) and CSC (V side), row of each CSR entry
    int32_t *d_csr_ptr = nullptr, *d_csr_idx = nullptr;
    float *d_csr_val = nullptr;
    int32_t *d_csc_ptr = nullptr, *d_csc_idx = nullptr;
    float *d_csc_val = nullptr;
    int32_t *d_coo_row = nullptr;
    int32_t *d_csc_perm = nullptr;  // CSC position -> CSR position (built on demand)
    // test ratings (COO)
    int32_t *d_test_row = nullptr, *d_test_col = nullptr;
    float *d_test_val = nullptr;
    // factors, FP32 row-contiguous (the reference's d_UT / d_VT)
    float *d_U = nullptr, *d_V = nullptr;
    // rows of each side in descending-degree order, and the host copy of the pointer arrays
    int32_t *d_order[2] = {nullptr, nullptr};
    std::vector<int32_t> host_ptr[2];
    int32_t maxdeg[2] = {0, 0};
    // status words and reduction scratch
    int32_t *d_flags = nullptr;
    double *d_partials = nullptr, *d_scalar = nullptr;

    void *d_scratch = nullptr;  // transpose / degree-order scratch, allocated once
    cudaEvent_t ev_transpose[2] = {nullptr, nullptr};
    std::vector<float> h_U, h_V;  // host mirror written by als_train (h_UT / h_VT)
    std::string last_error;
    double stage_ms[4] = {-1.0, -1.0, -1.0, -1.0};
    int64_t counters[3] = {0, 0, 0};
    uint64_t wait_ns = 0;  // bound of the sweep kernels' device waits (0: the default, 10 s)
    std::vector<cudaEvent_t> events;
    cudaEvent_t ev_half[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    // one ALS epoch (U then V half-sweep) captured once the kernel plan is final, replayed by
    // als_iterate; dropped whenever a pointer, the data or the plan changes
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int64_t eager_epochs = 0;  // epochs run without a graph since the last invalidation
                               // (capture waits for the first one)
    // kernel plan per side: buckets (rebuilt when the ratings change), half-sweeps since the
    // rebuild, and the autotuner's decision per degree class (kept across rating changes)
    std::vector<SweepBucket> plan[2];
    int sweeps[2] = {0, 0};
    bool tuned[2] = {false, false};
    int cls_solver[2][3] = {{ALS_SOLVE_CHOLESKY, ALS_SOLVE_CHOLESKY, ALS_SOLVE_CHOLESKY},
                            {ALS_SOLVE_CHOLESKY, ALS_SOLVE_CHOLESKY, ALS_SOLVE_CHOLESKY}};

    TcState *tc = nullptr;

    // FP32 path: the heavy rows' parts per side (built on the side's first FP32 sweep, dropped
    // when the ratings change): device tables part_beg, part_end, first (one block), the host
    // copy of `first`, and the partial-Gram scratch
    struct Split {
        bool built = false;
        int32_t nheavy = 0, nparts = 0;
        int32_t *d_tab = nullptr;
        std::vector<int32_t> first;
        float *d_part = nullptr;
    } split[2];

    // event log attached by als_set_log (not owned): training lines, per-iteration test RMSE
    als_log *log = nullptr;
    bool log_iter_rmse = false, log_cout = false;

    ~als_handle();
};

// sweep.cpp
als_status prepare_precision_path(als_handle *h);
void release_precision_path(als_handle *h);
void invalidate_graphs(als_handle *h);
als_status refresh_csc_values(als_handle *h);
als_status run_half_sweep(als_handle *h, int side);
als_status run_epochs(als_handle *h, int32_t iters);
void data_changed(als_handle *h);
void reset_tuning(als_handle *h);
als_status read_stage_ms(als_handle *h, int side);
als_status check_sweep_flags(als_handle *h);
bool tc_supported(int f);

// eventlog.cpp
namespace als {
void log_text(als_log *lg, const std::string &text, bool write_cout);
void log_event(als_log *lg, int32_t event, bool finished, bool write_cout);
void log_set_als_iter(als_log *lg, int64_t als_iter);
}  // namespace als
