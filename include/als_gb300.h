/*
 * als_gb300.h — C ABI of the GB300-native ALS (weighted-lambda alternating least squares) sweep.
 *
 * Drop-in boundary for vserdyuk/cuda_als.  Every entry point below names the reference interface it
 * replaces (file:line inside that project).  The ABI is plain C: integers, floats, raw pointers and
 * sizes.  No C++ types, no torch types, no exceptions cross it; every call returns an als_status.
 *
 * Conventions
 *   - Indices are 0-based int32, values are float32, exactly as the reference's raw .bin arrays
 *     (cuda_sparse_matrix.h:8-38, cuda_sparse_matrix.cpp:6-27).
 *   - Factor tables are row-contiguous float32: U[row * f + k], V[col * f + k]
 *     (the reference's h_UT / h_VT, als_model.h:58-66).
 *   - A handle owns all of its device memory; views passed to als_create are copied.
 *   - One handle = one CUDA stream.  A handle is not thread-safe; distinct handles are.
 *   - Calls are synchronous (they return after the device work finished) unless named *_async.
 */
#ifndef ALS_GB300_H
#define ALS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Replaces the reference's exit(1) inside CUDA_CHECK/CUBLAS_CHECK/CUSPARSE_CHECK
 * (cuda_common.h:13-91) and std::runtime_error for file/config problems
 * (cuda_sparse_matrix.cpp:9-27, als_model.cu:1910-1975). */
typedef enum als_status {
    ALS_OK = 0,
    ALS_ERR_INVALID_ARG = 1,  /* bad size, null pointer, index out of range, non-finite rating   */
    ALS_ERR_IO = 2,           /* missing file, file size not equal to the expected buffer size    */
    ALS_ERR_CUDA = 3,         /* a CUDA runtime/driver call failed                                */
    ALS_ERR_NUMERIC = 4,      /* non-positive pivot / non-finite solution flagged by a kernel     */
    ALS_ERR_TIMEOUT = 5,      /* a bounded device-side wait ran out                               */
    ALS_ERR_UNSUPPORTED = 6,  /* configuration outside what this build implements                 */
    ALS_ERR_OUT_OF_MEMORY = 7,
    ALS_ERR_NO_DEVICE = 8     /* no CUDA device visible                                           */
} als_status;

/* als_model::CALCULATE_VTVS_TYPE (als_model.h:12-21), same integer values as the INI key
 * als_calculate_vtvs_type.  Types 0-4 select the FP32 Gram path, 5-7 the BF16 tensor-core path
 * (tcgen05), unless als_config.precision overrides it.  Type 3 (the reference's load-only
 * microbenchmark) is accepted and runs the FP32 path. */
enum {
    ALS_VTVS_SIMPLE = 0,
    ALS_VTVS_SMEM_ROW_MAJOR = 1,
    ALS_VTVS_SMEM_COL_MAJOR = 2,
    ALS_VTVS_SMEM_ROW_MAJOR_NO_CALC = 3,
    ALS_VTVS_SMEM_COL_MAJOR_TWO_THREADS = 4,
    ALS_VTVS_SMEM_ROW_MAJOR_TENSOR = 5,
    ALS_VTVS_SMEM_ROW_MAJOR_TENSOR_SYMMETRIC = 6,
    ALS_VTVS_SMEM_ROW_MAJOR_TENSOR_SYMMETRIC_MULT_FRAG = 7
};

/* als_model::SOLVE_TYPE (als_model.h:23-27), same integer values as the INI key als_solve_type,
 * plus two solvers of this build. */
enum {
    ALS_SOLVE_LU = 0,          /* LU without pivoting (cublasSgetrfBatched with PivotArray=NULL)  */
    ALS_SOLVE_CG_FP16 = 1,     /* warm-started CG on an FP16-rounded Gram (cg.cu:236-430)          */
    ALS_SOLVE_CG_FP32 = 2,     /* warm-started CG, FP32 (cg.cu:37-232)                             */
    ALS_SOLVE_CHOLESKY = 3,    /* batched Cholesky + triangular solves (this build)                */
    ALS_SOLVE_AUTO = 4         /* per-bucket choice made by the autotuner (this build)             */
};

/* Arithmetic type of the Gram/RHS contraction. */
enum {
    ALS_PREC_FROM_VTVS = -1,   /* derive from calculate_vtvs_type (0-4 -> FP32, 5-7 -> BF16)       */
    ALS_PREC_FP32 = 0,
    ALS_PREC_BF16 = 1,
    ALS_PREC_FP8 = 2           /* e4m3 operands, one power-of-two scale per feature (per row and
                                  column of every Gram: exact), ratings in e4m3; f <= 128     */
};

/* Model configuration.  The first block holds the reference's INI keys and als_model ctor
 * arguments (main.cpp:28-47, als_model.h:29-32) with the same meaning; the second block holds the
 * [als_gb300] keys of this build.  Fill with als_config_default() first. */
typedef struct als_config {
    int32_t f;                    /* [als] f                                                    */
    float lambda;                 /* [als] lambda (weighted by the row's rating count)           */
    int32_t iters;                /* [als] als_iters                                            */
    int32_t calculate_vtvs_type;  /* [als] als_calculate_vtvs_type                              */
    int32_t solve_type;           /* [als] als_solve_type                                       */
    int32_t smem_col_cnt;         /* kept for the ctor signature; hard-coded 32 in main.cpp:43  */
    int32_t m_batches;            /* [als] m_batches: accepted; rows are bucketed, not batched  */
    int32_t n_batches;            /* [als] n_batches: accepted; see m_batches                   */
    /* ---- [als_gb300] ---- */
    int32_t precision;            /* ALS_PREC_*                                                 */
    int32_t refine_steps;         /* iterative-refinement steps after a Cholesky solve          */
    float cond_threshold;         /* diag-ratio estimate above which the residual is FP64       */
    int32_t cg_steps;             /* CG iterations (reference CG_ITER = 6, als_model.cu:16)     */
    float cg_tol;                 /* CG exit when r'r < cg_tol (reference CG_ERROR, cg.cu:32)   */
    int32_t use_graph;            /* replay each epoch from a CUDA graph once the plan is final */
    int32_t autotune;             /* ALS_SOLVE_AUTO: 0 tune once per handle, 1 at every init    */
    int32_t device;               /* CUDA device ordinal                                        */
} als_config;

/* Non-owning views of host (or, for *_device entry points, device) arrays.
 * host_sparse_matrix's CSR / CSC / COO members (cuda_sparse_matrix.h:27-37). */
typedef struct als_csr_view {
    int64_t rows, cols, nnz;
    const int32_t *row_ptrs;   /* rows + 1 */
    const int32_t *col_idxs;   /* nnz      */
    const float *vals;         /* nnz      */
} als_csr_view;

typedef struct als_csc_view {
    int64_t rows, cols, nnz;
    const int32_t *col_ptrs;   /* cols + 1 */
    const int32_t *row_idxs;   /* nnz      */
    const float *vals;         /* nnz      */
} als_csc_view;

typedef struct als_coo_view {
    int64_t rows, cols, nnz;
    const int32_t *row_idxs;   /* nnz */
    const int32_t *col_idxs;   /* nnz */
    const float *vals;         /* nnz */
} als_coo_view;

typedef struct als_handle als_handle;

/* ------------------------------------------------------------------------------------------ */
/* Library / configuration                                                                    */
/* ------------------------------------------------------------------------------------------ */

/* Version string of this build. */
const char *als_version(void);

/* Human-readable name of a status code. */
const char *als_status_string(als_status s);

/* Defaults: f=100, lambda=0.05, iters=10, type 1, solve 0 (LU), smem_col_cnt=32, batches 1,
 * precision from the vtvs type, refine 1, cond 1e4, CG 6 steps / 1e-4, graph on, autotune off. */
void als_config_default(als_config *cfg);

/* Parse the reference's INI file (keys of main.cpp:28-47 plus an optional [als_gb300] section)
 * into cfg, and the [data] section into the out-parameters.  data_folder receives at most
 * data_folder_len bytes (NUL-terminated).  Replaces INIReader usage in main.cpp:21-47. */
als_status als_config_from_ini(const char *path, als_config *cfg, int64_t *m, int64_t *n,
                               int64_t *nnz_train, int64_t *nnz_test, int32_t *als_runs,
                               char *data_folder, size_t data_folder_len);

/* Page-locked host memory for the views (cudaMallocHost / cudaFreeHost), as host_sparse_matrix
 * holds its arrays (cuda_sparse_matrix.cpp:23, :33-41); H2D copies from it run at full link speed. */
als_status als_host_alloc(size_t bytes, void **out);
als_status als_host_free(void *p);

/* Read a raw little-endian .bin array into caller memory; the file size must equal `bytes`.
 * Replaces host_sparse_matrix::malloc_load_file (cuda_sparse_matrix.cpp:6-27). */
als_status als_load_bin(const char *path, void *dst, size_t bytes);

/* ------------------------------------------------------------------------------------------ */
/* Model (als_model, als_model.h:11-80)                                                        */
/* ------------------------------------------------------------------------------------------ */

/* Construct: copy train CSR (required), train CSC (optional: built on the GPU by a stable
 * transpose when NULL), test COO (optional) to the device and allocate factors and scratch.
 * Replaces als_model::als_model (als_model.cu:1517-1552) + device_sparse_matrix ctor
 * (cuda_sparse_matrix.cpp:76-110).  Views hold HOST pointers. */
als_status als_create(const als_config *cfg, const als_csr_view *train_csr,
                      const als_csc_view *train_csc, const als_coo_view *test_coo,
                      als_handle **out);

/* Same, but the views hold DEVICE pointers (on cfg->device); they are copied device-to-device. */
als_status als_create_device(const als_config *cfg, const als_csr_view *train_csr,
                             const als_csc_view *train_csc, const als_coo_view *test_coo,
                             als_handle **out);

/* Free everything the handle owns.  Replaces als_model::~als_model (als_model.cu:1554-1568). */
als_status als_destroy(als_handle *h);

/* Last error message recorded on the handle (empty string if none). */
const char *als_last_error(const als_handle *h);

/* Replace the handle's stream (cudaStream_t passed as void*).  NULL = the handle's own stream. */
als_status als_set_stream(als_handle *h, void *stream);

/* Upload new ratings of the same sizes (m, n, nnz, nnz_test) into an existing handle, from HOST
 * views: the CSR (and CSC when given, else the GPU transpose rebuilds it) and the test COO are
 * copied, validated and re-ordered; the factors are kept.  What a caller with a new rating
 * snapshot of the same shape does instead of rebuilding als_model (als_model.cu:1517-1552). */
als_status als_reload(als_handle *h, const als_csr_view *train_csr, const als_csc_view *train_csc,
                      const als_coo_view *test_coo);

/* Replace the training ratings' VALUES in place (same sparsity pattern), from host memory,
 * ordered as the CSR given at creation.  The CSC copy is refreshed on the GPU. */
als_status als_update_values(als_handle *h, const float *csr_vals_host);

/* srand(0); V = 0.2*rand()/RAND_MAX for n*f entries in order; U = 0; upload.
 * The reference's init (als_model.cu:1772-1784). */
als_status als_init_factors(als_handle *h);

/* Run `iters` ALS iterations (U half-sweep then V half-sweep each) from the current factors. */
als_status als_iterate(als_handle *h, int32_t iters);

/* One half-sweep: side 0 solves U given V (rows of the CSR), side 1 solves V given U (CSC).
 * The U block of als_model::train (als_model.cu:1797-2029) / the V block (:2030-2267). */
als_status als_half_sweep(als_handle *h, int32_t side);

/* init + cfg.iters iterations + copy factors to the handle's host mirror.
 * Replaces als_model::train (als_model.cu:1766-2289). */
als_status als_train(als_handle *h);

/* sqrt(sum((r - u.v)^2) / nnz) over the test / train ratings, accumulated in FP64 in a fixed
 * order (deterministic).  A factor component that is NaN ends that rating's dot product, as
 * calculate_square_error does (als_model.cu:62-89).  Replaces rsme_test / rsme_train
 * (als_model.cu:1722-1764; the reference's spelling "rsme" is kept by the host wrappers). */
als_status als_rmse_test(als_handle *h, double *out);
als_status als_rmse_train(als_handle *h, double *out);

/* Copy the factor tables out to / in from host memory (m*f and n*f floats; either may be NULL).
 * Replaces the public h_UT/h_VT/d_UT/d_VT members (als_model.h:58-66). */
als_status als_get_factors(als_handle *h, float *U, float *V);
als_status als_set_factors(als_handle *h, const float *U, const float *V);

/* Raw device pointers of the factor tables (for zero-copy callers). */
als_status als_get_device_factors(als_handle *h, float **U, float **V);

/* Write the cumf_sgd/libmf binary model: int loss=0, m, n, f, float mean rating, U, V.
 * Replaces als_model::save_libmf (als_model.cu:2294-2312). */
als_status als_save_libmf(als_handle *h, const char *path);

/* Shape of the handle: m, n, f, nnz_train, nnz_test (any pointer may be NULL). */
als_status als_get_shape(const als_handle *h, int64_t *m, int64_t *n, int32_t *f,
                         int64_t *nnz_train, int64_t *nnz_test);

/* Timing of the last half-sweeps measured with CUDA events on the handle's stream:
 * out[0] = U half-sweep ms, out[1] = V half-sweep ms, out[2] = quantise ms (BF16/FP8),
 * out[3] = transpose ms at creation.  Any entry not measured is negative. */
als_status als_get_stage_ms(const als_handle *h, double out[4]);

/* Counters of the last half-sweep: out[0] = kernel launches, out[1] = rows with a
 * non-positive pivot or non-finite solution (solved as x = 0 and flagged), out[2] = rows whose
 * residual was refined in FP64.  */
als_status als_get_counters(const als_handle *h, int64_t out[3]);

/* Bound, in nanoseconds, of every device-side wait of the tensor-core sweep kernels (a stage's
 * gathered rows, a free accumulator, a finished Gram, a product on the tensor core); 0 restores
 * the default of 10 s.  A wait that runs out makes its CTA stop taking rows, let every copy and
 * MMA it issued finish (those drains keep the 10 s bound), free its tensor memory and return; the
 * call then fails with ALS_ERR_TIMEOUT and the handle stays usable (the next call's status words
 * start from zero).  A limit shorter than a healthy wait turns healthy sweeps into timeouts: it
 * is a watchdog for a stuck device, and the way the timeout path is tested. */
als_status als_set_wait_limit_ns(als_handle *h, uint64_t ns);

/* The kernel choice per nnz bucket after autotuning: for bucket b, kind[b] (0 = FP32 SIMT,
 * 1 = BF16 tcgen05, 2 = FP8 tcgen05) and solver[b] (ALS_SOLVE_*).  nb in: capacity, out: count. */
als_status als_get_plan(const als_handle *h, int32_t side, int32_t *lo, int32_t *kind,
                        int32_t *solver, int32_t *nb);

/* The autotuner's measurements per bucket of the plan (ALS_SOLVE_AUTO): ms_cg[b] / ms_chol[b] /
 * ms_cg16[b] = CUDA-event time of the bucket's launch with the FP32 CG, Cholesky and (tensor-core
 * precisions only) the FP16-Gram CG on the tuning sweep (the side's second half-sweep, all from
 * the same warm start); rel[b] / rel16[b] = ||x_cg - x_chol|| / ||x_chol|| over the bucket's
 * rows for each CG.  The bucket keeps the fastest of Cholesky and the CGs with rel <= 5e-2.
 * Negative entries: not measured.  Any output pointer may be NULL.  nb in: capacity, out:
 * count.  Buckets are the rows of degree >= 8f, f <= degree < 8f and degree < f, in order. */
als_status als_get_tuning(const als_handle *h, int32_t side, float *ms_cg, float *ms_chol,
                          float *rel, float *ms_cg16, float *rel16, int32_t *nb);

/* ------------------------------------------------------------------------------------------ */
/* Adjoint of the user half-sweep (no reference counterpart; required by the build's spec)     */
/* ------------------------------------------------------------------------------------------ */

/* Held-out loss L = sum over (u,i,r) in heldout of (r - x_u . y_i)^2 where X = argmin of the
 * user half-sweep given Y = V.  Computes X (written to the handle's U), L, dL/dY (n*f floats,
 * host) and dL/dlambda by solving A_u g_u = dL/dx_u with each row's L D L^T factor, in FP32.
 * dL/dY is summed per item over its ratings in a fixed order (deterministic).
 * `heldout` is a host COO view (rows index U, cols index V). */
als_status als_user_halfsweep_adjoint(als_handle *h, const als_coo_view *heldout, double *loss,
                                      float *dLdY, double *dLdlambda);

/* The same, everything in FP64 on the GPU (Gram, factor, both solves, the reverse pass), from
 * FP64 item factors Y (n*f doubles, host) and an FP64 lambda rather than the handle's FP32 V and
 * lambda; dL/dY is returned in FP64 (n*f doubles, host).  The handle's V receives Y rounded to
 * FP32 and its U the forward solution.  f <= 128.  For gradient checks against finite
 * differences and for the hyper-gradient of lambda at full precision. */
als_status als_user_halfsweep_adjoint_f64(als_handle *h, const als_coo_view *heldout,
                                          const double *Y, double lambda, double *loss,
                                          double *dLdY, double *dLdlambda);

/* ------------------------------------------------------------------------------------------ */
/* Index kernels                                                                              */
/* ------------------------------------------------------------------------------------------ */

/* Stable CSR -> CSC transpose (rows inside each column ascending, i.e. the order scipy's
 * tocsc() produces).  The reference does this offline in scipy
 * (data/netflix/prepare_netflix_data.py:102-109, data/toy_data_2/prepare_toy_data_2.py:195-200).
 * HOST pointers; output arrays must hold cols+1 / nnz / nnz elements. */
als_status als_csr_to_csc(const als_csr_view *csr, int32_t *col_ptrs, int32_t *row_idxs,
                          float *vals);

/* Same, DEVICE pointers, enqueued on `stream` (cudaStream_t as void*); temporary memory is
 * allocated with cudaMallocAsync on that stream and released before return. */
als_status als_csr_to_csc_device(const als_csr_view *csr, int32_t *col_ptrs, int32_t *row_idxs,
                                 float *vals, void *stream);

/* The same stable transpose without allocating anything: for callers that may not allocate
 * device memory (a plug-in inside an engine that owns all device memory, an allocation-free
 * latency-critical loop).  No counterpart in the reference.  Scratch is a fixed 16 MiB device
 * array inside this library; the transpose needs 28 bytes per rating plus 1 KiB per 4,096
 * ratings, each array rounded up to 256 bytes, so at most 593,856 ratings are accepted and larger
 * inputs are rejected with ALS_ERR_INVALID_ARG.  The first call in each CUDA context looks the
 * array up (again after a device reset); all calls share the array, so calls that overlap on the
 * GPU race and must be serialised by the caller.  DEVICE pointers, enqueued on `stream`. */
als_status als_csr_to_csc_device_noalloc(const als_csr_view *csr, int32_t *col_ptrs,
                                         int32_t *row_idxs, float *vals, void *stream);

/* Rating triples -> the CSR, the row of every CSR entry and the CSC, built on the GPU.  Replaces
 * the reference's offline scipy step (data/toy_data/prepare_toy_data.py:108-110, 147-150,
 * 201-208; data/netflix/prepare_netflix_data.py:88-109): coo_matrix((vals, (rows, cols))) then
 * .tocsr().tocoo() (R_train_coo.row.bin and the sorted test COO), .tocsr() (R_train_csr.*.bin)
 * and .tocsc() (R_train_csc.*.bin), values cast to float32.  Entries end in (row, column) order;
 * the triples of one cell (duplicates) are summed in FP64 and rounded once to FP32, which equals
 * scipy's float64 sum + float32 cast whenever that sum is exact (any ratings on a common grid,
 * such as star ratings).  Indices are 0-based; an index outside [0, rows) x [0, cols) fails with
 * ALS_ERR_INVALID_ARG.  HOST pointers.  Output arrays hold coo->nnz entries (the upper bound);
 * *nnz_out receives the count after summing duplicates (the CSR's row_ptrs[rows]).  coo_rows may
 * be NULL; col_ptrs (cols + 1), row_idxs and csc_vals are all three given or all NULL. */
als_status als_coo_to_csr(const als_coo_view *coo, int32_t *row_ptrs, int32_t *col_idxs,
                          float *vals, int32_t *coo_rows, int32_t *col_ptrs, int32_t *row_idxs,
                          float *csc_vals, int64_t *nnz_out);

/* Same, DEVICE pointers, enqueued on `stream` (cudaStream_t as void*), scratch allocated with
 * cudaMallocAsync on it; synchronous (the count after summing duplicates sizes the later
 * launches and is returned in *nnz_out, host memory). */
als_status als_coo_to_csr_device(const als_coo_view *coo, int32_t *row_ptrs, int32_t *col_idxs,
                                 float *vals, int32_t *coo_rows, int32_t *col_ptrs,
                                 int32_t *row_idxs, float *csc_vals, int64_t *nnz_out,
                                 void *stream);

/* Row order used by the persistent sweep: rows sorted by descending rating count, ties by
 * ascending row id (a stable sort).  Replaces contiguous m_batches/n_batches splitting
 * (main.cpp:46-47, als_model.cu:1891-1896).  HOST pointers: row_ptrs (rows+1) in, perm (rows)
 * out. */
als_status als_degree_order(int64_t rows, const int32_t *row_ptrs, int32_t *perm);

/* Contiguous row ranges for nparts ranks, balanced by weight: a row weighs its rating count plus
 * row_weight (the solve's cost in rating-equivalents; 0 = balance ratings only).  Part k gets rows
 * [bounds[k], bounds[k+1]), bounds[0] = 0, bounds[nparts] = rows; boundary k falls where the
 * running weight crosses k/nparts of the total (a row goes to the earlier part when its midpoint
 * lies before that point), so every boundary is within half a row's weight of its target.  Replaces the reference's equal-count m_batches / n_batches split
 * (als_model.cu:1891-1896) for sharding a half-sweep over ranks.  Host work, HOST pointers:
 * row_ptrs (rows + 1) in, bounds (nparts + 1) out. */
als_status als_partition_rows(int64_t rows, const int32_t *row_ptrs, int32_t nparts,
                              double row_weight, int64_t *bounds);

/* ------------------------------------------------------------------------------------------ */
/* Synthetic ratings (seeded, deterministic across machines and thread counts)                */
/* ------------------------------------------------------------------------------------------ */

/* Shapes of the five workload configurations (1..5); see als_synth_generate. */
als_status als_synth_shape(int32_t config, int64_t *m, int64_t *n, int64_t *nnz_total,
                           int32_t *f, float *lambda);

/* Generate workload `config` with `seed` at `scale` (1.0 = full size; smaller values shrink
 * rows, cols and nnz for tests).  Two calls: with NULL arrays to get sizes, then with arrays.
 * Train is CSR sorted by (row, col); test is COO sorted by (row, col).  Every row and column
 * keeps at least one training rating. */
als_status als_synth_generate(int32_t config, uint64_t seed, double scale, int64_t *m, int64_t *n,
                              int64_t *nnz_train, int64_t *nnz_test, int32_t *row_ptrs,
                              int32_t *col_idxs, float *vals, int32_t *test_rows,
                              int32_t *test_cols, float *test_vals);

/* ------------------------------------------------------------------------------------------ */
/* Event log: the reference's timing CSV (logger.h:7-48, logger.cpp)                           */
/* ------------------------------------------------------------------------------------------ */

/* Timed events, same integer values and names as logger::EVENT_TYPE (logger.h:8-13). */
enum {
    ALS_EVENT_UPDATE_U = 0,          /* "ALS_UPDATE_U": one U half-sweep                        */
    ALS_EVENT_UPDATE_V = 1,          /* "ALS_UPDATE_V": one V half-sweep                        */
    ALS_EVENT_ITER = 2,              /* "ALS_ITER": one ALS iteration (U then V)                */
    ALS_EVENT_MF_MODEL_TRAINING = 3  /* "MF_MODEL_TRAINING": model construction + train()       */
};

typedef struct als_log als_log;

/* An in-memory CSV log with the columns
 *   log_name,id,run_iter,als_iter,prev_ts,curr_ts,elapsed,event_elapsed,text
 * (timestamps: wall-clock seconds since the epoch, 6 decimals).  log_name is the UTC creation
 * time "%Y%m%d_%H%M%S" + "_debug=false.csv".  Writes the header and the line "init logger".
 * log_folder may be NULL or empty (save() then writes log_name in the current directory).
 * Replaces logger::init (logger.cpp:56-73). */
als_status als_log_create(const char *log_folder, als_log **out);
als_status als_log_destroy(als_log *lg);

/* A text line: elapsed = time since the previous text line, event_elapsed empty; the prev_ts
 * column holds the new timestamp (as logger::log, logger.cpp:75-87).  write_cout != 0 also prints
 * "run iter: R als iter: A elapsed: E <text>" to stdout.  Thread-safe, as are all log calls. */
als_status als_log_text(als_log *lg, const char *text, int32_t write_cout);

/* Event start / finish (logger.cpp:89-143).  The finish line has text "event <NAME> finished",
 * event_elapsed = now - the event's start, and does not advance prev_ts. */
als_status als_log_event_started(als_log *lg, int32_t event);
als_status als_log_event_finished(als_log *lg, int32_t event, int32_t write_cout);

/* The run_iter / als_iter columns of the following lines (logger.h:43-44, public fields there). */
als_status als_log_set_iters(als_log *lg, int64_t run_iter, int64_t als_iter);
als_status als_log_get_iters(const als_log *lg, int64_t *run_iter, int64_t *als_iter);

/* log_name (owned by the log). */
const char *als_log_name(const als_log *lg);

/* The CSV so far: len in = capacity of buf in bytes, out = bytes needed including the NUL.
 * buf may be NULL to query the size; a short buffer receives nothing and ALS_ERR_INVALID_ARG. */
als_status als_log_contents(const als_log *lg, char *buf, size_t *len);

/* Write the CSV to `path`, or to <log_folder>/<log_name> when path is NULL (logger::save,
 * logger.cpp:145-153).  ALS_ERR_IO when the file cannot be written. */
als_status als_log_save(const als_log *lg, const char *path);

/* Attach a log to a handle (NULL detaches; the handle does not own it, and the log must outlive
 * the attachment).  While attached,
 * als_train and als_iterate write the reference's training lines (als_model.cu:1768-1787,
 * 1792-1801, 2021-2034, 2259-2286): "als model training started", "factors initialization done",
 * per iteration als_iter = 1..iters with ALS_UPDATE_U, ALS_UPDATE_V and ALS_ITER events (the
 * stream is synchronised at the end of each half-sweep, so event_elapsed covers its device work;
 * epochs run without the CUDA graph), "RMSE test: %f" after every iteration but the last when
 * iter_rmse != 0 (the reference's CALC_ITER_RMSE build), als_iter = 0, "als model training done".
 * write_cout != 0 echoes every line to stdout, as the reference's write_cout = true calls. */
als_status als_set_log(als_handle *h, als_log *lg, int32_t iter_rmse, int32_t write_cout);

/* A string value of an INI file ("" when the section or key is absent, as INIReader::Get with
 * an empty default, main.cpp:36, :49).  buf receives at most len bytes (NUL-terminated). */
als_status als_ini_get(const char *path, const char *section, const char *key, char *buf,
                       size_t len);

#ifdef __cplusplus
}
#endif

#endif /* ALS_GB300_H */
