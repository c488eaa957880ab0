// sweep.cpp — half-sweep orchestration: picks the kernel per precision, times each half-sweep
// with CUDA events on the handle's stream, and collects the per-row status words.
//
// Replaces the host loop of als_model::train (als_model.cu:1797-2267): per half-sweep the
// reference allocates and frees its RHS scratch, launches csrmm2 + geam, a Gram kernel per row
// batch and a solver per batch with host synchronisation in between.  Here every row of a side
// is handled by fused kernels in descending-degree order with no host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

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

void release_split(als_handle *h);

void release_precision_path(als_handle *h) {
    release_split(h);
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 2; ++k)
            if (h->ev_half[s][k]) cudaEventDestroy(h->ev_half[s][k]);
    tc_release(h);
}

void invalidate_graphs(als_handle *h) {
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->graph_exec = nullptr;
    h->graph = nullptr;
    // the next capture waits for one eager epoch on the new state, so a reload followed by a
    // single epoch (the e2e pattern) pays for no capture and instantiation
    h->eager_epochs = 0;
    tc_invalidate_graphs(h);
}


als_status refresh_csc_values(als_handle *h) {
    cudaStream_t st = h->stream;
    if (!h->d_csc_perm) {
        // no permutation yet (the CSC came from the caller, or was built without it): rebuild
        // the CSC and the permutation from the CSR, in the handle's transpose scratch
        cudaError_t e = cudaMalloc(&h->d_csc_perm, sizeof(int32_t) * (size_t)h->nnz);
        if (e != cudaSuccess) return fail(h, ALS_ERR_OUT_OF_MEMORY, "csc permutation");
        e = csr_to_csc_device(h->m, h->n, h->nnz, h->d_csr_ptr, h->d_csr_idx, h->d_csr_val,
                              h->d_csc_ptr, h->d_csc_idx, h->d_csc_val, h->d_scratch, st,
                              nullptr, h->d_csc_perm);
        S_CUDA(h, e);
    } else {
        S_CUDA(h, gather_f32(h->nnz, h->d_csc_perm, h->d_csr_val, h->d_csc_val, st));
    }
    S_CUDA(h, cudaStreamSynchronize(st));
    return tc_values_changed(h);
}

// ---------------------------------------------------------------------------- kernel plan

// Relative agreement the autotuner asks of CG against Cholesky on a bucket's rows (Frobenius norm
// of the difference over the norm of the Cholesky solution) at the tuning sweep.  The tuning
// sweep is the first warm start, where six CG steps are furthest from converged; on rows lighter
// than f (rank-deficient Grams) they land 2-3e-2 from Cholesky there (MovieLens-latest-shaped
// items) and keep the test RMSE within 5e-5 of plain FP32 Cholesky after training, as the
// reference's own configurations run CG on every row.
constexpr double AUTO_TOL = 5e-2;
// The tuning sweep runs on the first warm start, where CG takes all its steps; later epochs exit
// earlier, which favours the solver with the smaller fixed cost per row.  The tensor-core CG pays
// a scale reduction and a packing pass per row, so it must beat the best other solver by this
// factor on the tuning sweep (measured on the Netflix-shaped workload: its 2-9% leads on the
// mid / light U buckets at the tuning sweep are 3-5% losses in steady state, its 29-33% leads on
// the heavy buckets stay wins).
constexpr float CG16_MARGIN = 0.85f;

static bool autotuned(const als_handle *h) { return h->cfg.solve_type == ALS_SOLVE_AUTO; }

// Buckets of a side from the host copy of its pointer array: rows of degree >= 8f (the Gram
// dominates), f <= degree < 8f, and degree < f (rank-deficient Gram, the solve dominates).  The
// order array is sorted by descending degree, so each bucket is a contiguous range of it.  A fixed
// solver makes one bucket of every row.
static void build_plan(als_handle *h, int side) {
    const std::vector<int32_t> &ptr = h->host_ptr[side];
    const int64_t rows = side == 0 ? h->m : h->n;
    std::vector<SweepBucket> &plan = h->plan[side];
    plan.clear();
    h->sweeps[side] = 0;
    if (!autotuned(h) || (int64_t)ptr.size() != rows + 1) {
        SweepBucket b;
        b.hi = (int32_t)rows;
        b.solver = autotuned(h) ? ALS_SOLVE_CHOLESKY : h->cfg.solve_type;
        plan.push_back(b);
        h->tuned[side] = true;
        return;
    }
    int64_t heavy = 0, mid = 0;
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t d = ptr[r + 1] - ptr[r];
        if (d >= 8 * (int64_t)h->f) ++heavy;
        else if (d >= h->f) ++mid;
    }
    const int64_t cuts[4] = {0, heavy, heavy + mid, rows};
    for (int k = 0; k < 3; ++k) {
        if (cuts[k + 1] == cuts[k]) continue;
        SweepBucket b;
        b.lo = (int32_t)cuts[k];
        b.hi = (int32_t)cuts[k + 1];
        b.cls = k;
        b.solver = h->tuned[side] ? h->cls_solver[side][k] : ALS_SOLVE_CHOLESKY;
        plan.push_back(b);
    }
}

// The ratings changed (creation, reload): drop the graph and the buckets; an autotuned side keeps
// its per-class solver choice and applies it to the new buckets.
void data_changed(als_handle *h) {
    invalidate_graphs(h);
    for (auto &pl : h->plan) pl.clear();
    release_split(h);
}

// Forget the autotuner's decisions (als_init_factors with autotune = 1).
void reset_tuning(als_handle *h) {
    if (!autotuned(h)) return;
    invalidate_graphs(h);
    for (int s = 0; s < 2; ++s) {
        h->plan[s].clear();
        h->tuned[s] = false;
        for (int &c : h->cls_solver[s]) c = ALS_SOLVE_CHOLESKY;
    }
}

static bool plan_final(const als_handle *h) {
    for (int s = 0; s < 2; ++s)
        if (h->plan[s].empty() || !h->tuned[s]) return false;
    return true;
}

void release_split(als_handle *h) {
    for (auto &sp : h->split) {
        if (sp.d_tab) cudaFree(sp.d_tab);
        if (sp.d_part) cudaFree(sp.d_part);
        sp = als_handle::Split();
    }
}

// The FP32 path's heavy rows of a side (degree > FP32_SPLIT_RATINGS): the first positions of the
// side's descending-degree order (ties by ascending row id, the order the device sort makes),
// each cut into parts of FP32_SPLIT_RATINGS ratings.
static cudaError_t build_split(als_handle *h, int side) {
    als_handle::Split &sp = h->split[side];
    if (sp.built) return cudaSuccess;
    const std::vector<int32_t> &ptr = h->host_ptr[side];
    const int64_t rows = (int64_t)ptr.size() - 1;
    std::vector<int32_t> heavy;
    for (int64_t r = 0; r < rows; ++r)
        if (ptr[r + 1] - ptr[r] > FP32_SPLIT_RATINGS) heavy.push_back((int32_t)r);
    std::stable_sort(heavy.begin(), heavy.end(), [&](int32_t x, int32_t y) {
        return ptr[x + 1] - ptr[x] > ptr[y + 1] - ptr[y];
    });
    std::vector<int32_t> pbeg, pend;
    sp.first.assign(1, 0);
    for (int32_t r : heavy) {
        for (int32_t b = ptr[r]; b < ptr[r + 1]; b += FP32_SPLIT_RATINGS) {
            pbeg.push_back(b);
            pend.push_back(std::min(ptr[r + 1], b + FP32_SPLIT_RATINGS));
        }
        sp.first.push_back((int32_t)pbeg.size());
    }
    sp.nheavy = (int32_t)heavy.size();
    sp.nparts = (int32_t)pbeg.size();
    if (sp.nparts > 0) {
        const size_t np = (size_t)sp.nparts;
        cudaError_t e = cudaMalloc(&sp.d_tab, sizeof(int32_t) * (2 * np + sp.first.size()));
        if (e == cudaSuccess)
            e = cudaMalloc(&sp.d_part, sizeof(float) * np * fp32_part_floats(h->f));
        if (e == cudaSuccess)
            e = cudaMemcpy(sp.d_tab, pbeg.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(sp.d_tab + np, pend.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(sp.d_tab + 2 * np, sp.first.data(), sizeof(int32_t) * sp.first.size(),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    sp.built = true;
    return cudaSuccess;
}

static cudaError_t launch_bucket(als_handle *h, int side, const SweepBucket &b, int solve, int slot,
                                 int *launches) {
    if (h->precision != ALS_PREC_FP32)
        return tc_launch_bucket(h, side, b.lo, b.hi, solve, slot, launches);
    cudaError_t e = build_split(h, side);
    if (e != cudaSuccess) return e;
    SweepArgs a{};
    a.ptr = side == 0 ? h->d_csr_ptr : h->d_csc_ptr;
    a.idx = side == 0 ? h->d_csr_idx : h->d_csc_idx;
    a.val = side == 0 ? h->d_csr_val : h->d_csc_val;
    a.Y = side == 0 ? h->d_V : h->d_U;
    a.X = side == 0 ? h->d_U : h->d_V;
    a.order = h->d_order[side];
    a.row_begin = b.lo;
    a.row_end = b.hi;
    a.f = h->f;
    a.lambda = h->cfg.lambda;
    a.solve = solve;
    a.cg_iters = h->cfg.cg_steps;
    a.cg_tol = h->cfg.cg_tol;
    a.flags = h->d_flags;
    const als_handle::Split &sp = h->split[side];
    Fp32Split fs;
    if (sp.nparts > 0) {
        const size_t np = (size_t)sp.nparts;
        fs.part_beg = sp.d_tab;
        fs.part_end = sp.d_tab + np;
        fs.first = sp.d_tab + 2 * np;
        fs.first_host = sp.first.data();
        fs.nheavy = sp.nheavy;
        fs.part = sp.d_part;
    }
    return launch_sweep_fp32(a, sp.nparts > 0 ? &fs : nullptr, h->stream, launches);
}

// The tuning sweep of a side (ALS_SOLVE_AUTO, the side's second half-sweep: the first leaves the
// warm start CG needs).  Every bucket runs the FP32 CG, on the tensor-core path also the
// FP16-Gram CG (its products on the tensor core), and then Cholesky, all from the same warm
// start and each timed with CUDA events; the bucket keeps the fastest of Cholesky and the CGs
// that agree with it within AUTO_TOL (the tensor-core CG only with a CG16_MARGIN lead).  The
// factors keep the Cholesky solution and the status words count the Cholesky run only.
// Synchronous (the host reads the timings): never graph-captured.
static als_status tune_side(als_handle *h, int side, int *launches) {
    cudaStream_t st = h->stream;
    const int64_t rows = side == 0 ? h->m : h->n;
    float *X = side == 0 ? h->d_U : h->d_V;
    const size_t xbytes = sizeof(float) * (size_t)rows * h->f;
    float *x_prev = nullptr, *x_cg = nullptr, *x_cg16 = nullptr;
    double *d_diff = nullptr;
    int32_t *flags_save = nullptr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const bool with_cg16 = h->precision != ALS_PREC_FP32;
    auto cleanup = [&]() {
        if (x_prev) cudaFree(x_prev);
        if (x_cg) cudaFree(x_cg);
        if (x_cg16) cudaFree(x_cg16);
        if (d_diff) cudaFree(d_diff);
        if (flags_save) cudaFree(flags_save);
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    };
    if (cudaMalloc(&x_prev, xbytes) != cudaSuccess || cudaMalloc(&x_cg, xbytes) != cudaSuccess ||
        (with_cg16 && cudaMalloc(&x_cg16, xbytes) != cudaSuccess) ||
        cudaMalloc(&d_diff, 4 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&flags_save, 4 * sizeof(int32_t)) != cudaSuccess) {
        cleanup();
        return fail(h, ALS_ERR_OUT_OF_MEMORY, "out of memory for the autotuner's factor copies");
    }
    for (auto &e : ev) cudaEventCreate(&e);
    cudaError_t e = cudaSuccess;
    bool timed_out = false;
    for (size_t k = 0; k < h->plan[side].size() && e == cudaSuccess && !timed_out; ++k) {
        SweepBucket &b = h->plan[side][k];
        cudaMemcpyAsync(x_prev, X, xbytes, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(flags_save, h->d_flags, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
        cudaEventRecord(ev[0], st);
        e = launch_bucket(h, side, b, ALS_SOLVE_CG_FP32, (int)k, launches);
        cudaEventRecord(ev[1], st);
        if (e != cudaSuccess) break;
        cudaMemcpyAsync(x_cg, X, xbytes, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(X, x_prev, xbytes, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(h->d_flags, flags_save, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
        if (with_cg16) {
            cudaEventRecord(ev[4], st);
            e = launch_bucket(h, side, b, ALS_SOLVE_CG_FP16, (int)k, launches);
            cudaEventRecord(ev[5], st);
            if (e != cudaSuccess) break;
            cudaMemcpyAsync(x_cg16, X, xbytes, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(X, x_prev, xbytes, cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(h->d_flags, flags_save, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                            st);
        }
        cudaEventRecord(ev[2], st);
        e = launch_bucket(h, side, b, ALS_SOLVE_CHOLESKY, (int)k, launches);
        cudaEventRecord(ev[3], st);
        if (e != cudaSuccess) break;
        e = launch_bucket_diff(h->d_order[side], b.lo, b.hi, X, x_cg, h->f, d_diff, st);
        ++*launches;
        if (e == cudaSuccess && with_cg16) {
            e = launch_bucket_diff(h->d_order[side], b.lo, b.hi, X, x_cg16, h->f, d_diff + 2, st);
            ++*launches;
        }
        double diff[4] = {0.0, 0.0, 0.0, 0.0};
        int32_t fl[4] = {0, 0, 0, 0};
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(diff, d_diff, sizeof(double) * (with_cg16 ? 4 : 2),
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fl, h->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        if (fl[2]) {  // a bounded wait ran out: stop; check_sweep_flags reports the timeout
            timed_out = true;
            break;
        }
        cudaEventElapsedTime(&b.ms_cg, ev[0], ev[1]);
        cudaEventElapsedTime(&b.ms_chol, ev[2], ev[3]);
        b.rel = diff[1] > 0.0 ? (float)std::sqrt(diff[0] / diff[1]) : 0.f;
        if (with_cg16) {
            cudaEventElapsedTime(&b.ms_cg16, ev[4], ev[5]);
            b.rel16 = diff[3] > 0.0 ? (float)std::sqrt(diff[2] / diff[3]) : 0.f;
        }
        b.solver = ALS_SOLVE_CHOLESKY;
        float best = b.ms_chol;
        if (b.rel <= AUTO_TOL && b.ms_cg < best) {
            b.solver = ALS_SOLVE_CG_FP32;
            best = b.ms_cg;
        }
        if (with_cg16 && b.rel16 <= AUTO_TOL && b.ms_cg16 >= 0.f && b.ms_cg16 < CG16_MARGIN * best) {
            b.solver = ALS_SOLVE_CG_FP16;
            best = b.ms_cg16;
        }
        h->cls_solver[side][b.cls] = b.solver;
    }
    cleanup();
    if (e != cudaSuccess) return fail(h, ALS_ERR_CUDA, std::string("autotuner: ") + cudaGetErrorString(e));
    if (!timed_out) h->tuned[side] = true;
    return ALS_OK;
}

// Enqueue one half-sweep on the handle's stream, bracketed by the side's timing events: the BF16
// table for the tensor-core path, then one launch per bucket of the side's plan.  No host
// synchronisation (except the autotuner's one tuning sweep), so an epoch can be graph-captured.
// The status words are zeroed by the caller once per call, so a timeout on either side survives
// until check_sweep_flags reads them.
als_status run_half_sweep(als_handle *h, int side) {
    cudaStream_t st = h->stream;
    if (h->plan[side].empty()) build_plan(h, side);
    S_CUDA(h, record_event(h->ev_half[side][0], st));
    int launches = 0;
    if (h->precision != ALS_PREC_FP32) {
        std::string why;
        als_status s = tc_quantise(h, side, &launches, &why);
        if (s != ALS_OK) return fail(h, s, why);
    }
    const bool tuning = !h->tuned[side] && h->sweeps[side] >= 1;
    ++h->sweeps[side];
    if (tuning) {
        als_status s = tune_side(h, side, &launches);
        if (s != ALS_OK) return s;
    } else {
        // adjacent buckets that settled on the same solver are contiguous ranges of the order:
        // one launch covers them (no tail between them, one launch fewer)
        const auto &plan = h->plan[side];
        for (size_t k = 0; k < plan.size();) {
            size_t last = k;
            while (last + 1 < plan.size() && plan[last + 1].solver == plan[k].solver) ++last;
            SweepBucket run = plan[k];
            run.hi = plan[last].hi;
            S_CUDA(h, launch_bucket(h, side, run, run.solver, (int)k, &launches));
            k = last + 1;
        }
    }
    S_CUDA(h, record_event(h->ev_half[side][1], st));
    h->counters[0] = launches;
    return ALS_OK;
}

// After the stream has been synchronised: the side's last half-sweep time.
als_status read_stage_ms(als_handle *h, int side) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev_half[side][0], h->ev_half[side][1]) == cudaSuccess) {
        h->stage_ms[side] = ms;
    } else {
        h->stage_ms[side] = -1.0;  // not measurable: reported as negative, not as a failure
        cudaGetLastError();
    }
    return ALS_OK;
}

// `iters` epochs.  Once the kernel plan is final (first epoch run; under ALS_SOLVE_AUTO the
// tuning sweeps done) and use_graph is set, an epoch is captured into a CUDA graph once and
// replayed: one launch call per epoch instead of one per kernel and memset.
als_status run_epochs(als_handle *h, int32_t iters) {
    cudaStream_t st = h->stream;
    int epoch_launches = 0;
    for (int32_t it = 0; it < iters; ++it) {
        const bool graphable = h->cfg.use_graph && h->eager_epochs > 0 &&
                               plan_final(h);
        if (graphable && !h->graph_exec) {
            S_CUDA(h, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            als_status s = run_half_sweep(h, 0);
            epoch_launches = (int)h->counters[0];
            if (s == ALS_OK) s = run_half_sweep(h, 1);
            epoch_launches += (int)h->counters[0];
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(st, &g);
            if (s != ALS_OK) {
                if (g) cudaGraphDestroy(g);
                return s;
            }
            S_CUDA(h, e);
            h->graph = g;
            S_CUDA(h, cudaGraphInstantiate(&h->graph_exec, g, 0));
            h->counters[0] = epoch_launches;
        }
        if (graphable) {
            S_CUDA(h, cudaGraphLaunch(h->graph_exec, st));
        } else {
            als_status s = run_half_sweep(h, 0);
            if (s != ALS_OK) return s;
            int launches = (int)h->counters[0];
            s = run_half_sweep(h, 1);
            if (s != ALS_OK) return s;
            h->counters[0] += launches;
            ++h->eager_epochs;
        }
    }
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

extern "C" als_status als_set_wait_limit_ns(als_handle *h, uint64_t ns) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    h->wait_ns = ns;
    invalidate_graphs(h);  // the limit is a kernel argument captured in the epoch graph
    return ALS_OK;
}

extern "C" als_status als_get_plan(const als_handle *h, int32_t side, int32_t *lo, int32_t *kind,
                                   int32_t *solver, int32_t *nb) {
    if (!h || !nb || (side != 0 && side != 1))
        return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    const int32_t fkind = h->precision == ALS_PREC_FP32 ? 0 : h->precision == ALS_PREC_FP8 ? 2 : 1;
    const std::vector<SweepBucket> &plan = h->plan[side];
    if (plan.empty()) {  // no sweep yet: the plan the next sweep starts from
        if (*nb >= 1) {
            if (lo) lo[0] = 0;
            if (kind) kind[0] = fkind;
            if (solver) solver[0] = autotuned(h) ? ALS_SOLVE_CHOLESKY : h->cfg.solve_type;
        }
        *nb = 1;
        return ALS_OK;
    }
    for (int32_t k = 0; k < (int32_t)plan.size() && k < *nb; ++k) {
        if (lo) lo[k] = plan[k].lo;
        if (kind) kind[k] = fkind;
        if (solver) solver[k] = plan[k].solver;
    }
    *nb = (int32_t)plan.size();
    return ALS_OK;
}

extern "C" als_status als_get_tuning(const als_handle *h, int32_t side, float *ms_cg,
                                     float *ms_chol, float *rel, float *ms_cg16, float *rel16,
                                     int32_t *nb) {
    if (!h || !nb || (side != 0 && side != 1))
        return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    const std::vector<SweepBucket> &plan = h->plan[side];
    for (int32_t k = 0; k < (int32_t)plan.size() && k < *nb; ++k) {
        if (ms_cg) ms_cg[k] = plan[k].ms_cg;
        if (ms_chol) ms_chol[k] = plan[k].ms_chol;
        if (rel) rel[k] = plan[k].rel;
        if (ms_cg16) ms_cg16[k] = plan[k].ms_cg16;
        if (rel16) rel16[k] = plan[k].rel16;
    }
    *nb = (int32_t)plan.size();
    return ALS_OK;
}

extern "C" als_status als_user_halfsweep_adjoint(als_handle *h, const als_coo_view *heldout,
                                                 double *loss, float *dLdY, double *dLdlambda) {
    if (!h || !heldout) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    return run_adjoint(h, heldout, loss, dLdY, dLdlambda);
}

extern "C" als_status als_user_halfsweep_adjoint_f64(als_handle *h, const als_coo_view *heldout,
                                                     const double *Y, double lambda, double *loss,
                                                     double *dLdY, double *dLdlambda) {
    if (!h || !heldout) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    return run_adjoint_f64(h, heldout, Y, lambda, loss, dLdY, dLdlambda);
}
