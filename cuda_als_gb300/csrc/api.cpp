// api.cpp — the C ABI (include/als_gb300.h): model handle, construction, sweeps, evaluation,
// factor I/O, INI/.bin readers and the standalone index entry points.
//
// Reference host code replaced: als_model (als_model.h:11-80, als_model.cu:1494-2312),
// host_sparse_matrix / device_sparse_matrix (cuda_sparse_matrix.h:8-68,
// cuda_sparse_matrix.cpp:6-122), the INI handling of main.cpp:21-47 and the error macros of
// cuda_common.h:13-91 (statuses instead of exit(1)).
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "handle.h"
#include "internal.h"
#include "tc.h"

namespace als {

static thread_local std::string g_error;

als_status set_global_error(als_status s, const std::string &msg) {
    g_error = msg;
    return s;
}

}  // namespace als

using namespace als;

// ---------------------------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------------------------

#define H_CUDA(h, call)                                                                         \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            (h)->last_error = std::string(#call) + ": " + cudaGetErrorString(e_);               \
            g_error_copy(h);                                                                    \
            return e_ == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA;      \
        }                                                                                       \
    } while (0)

#define G_CUDA(call)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return set_global_error(e_ == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY     \
                                                                    : ALS_ERR_CUDA,             \
                                    std::string(#call) + ": " + cudaGetErrorString(e_));        \
    } while (0)

static void g_error_copy(const als_handle *h) { set_global_error(ALS_OK, h->last_error); }

static als_status h_fail(als_handle *h, als_status s, const std::string &msg) {
    if (h) h->last_error = msg;
    return set_global_error(s, msg);
}

template <typename T>
static cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

static als_status check_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return set_global_error(ALS_ERR_NO_DEVICE, std::string("no CUDA device: ") +
                                                       (e != cudaSuccess ? cudaGetErrorString(e)
                                                                         : "count 0"));
    return ALS_OK;
}

// Host-side structural checks of a compressed matrix: ptr[0] = 0, non-decreasing, ptr[rows] = nnz.
static bool check_ptrs(const int32_t *ptr, int64_t rows, int64_t nnz, std::string *why) {
    if (!ptr) { *why = "null pointer array"; return false; }
    if (ptr[0] != 0) { *why = "ptr[0] != 0"; return false; }
    for (int64_t r = 0; r < rows; ++r)
        if (ptr[r + 1] < ptr[r]) {
            *why = "pointer array decreases at " + std::to_string(r);
            return false;
        }
    if ((int64_t)ptr[rows] != nnz) {
        *why = "ptr[rows] = " + std::to_string(ptr[rows]) + " != nnz " + std::to_string(nnz);
        return false;
    }
    return true;
}

// ---------------------------------------------------------------------------------------------
// library / config
// ---------------------------------------------------------------------------------------------

extern "C" const char *als_version(void) { return "als_gb300 1.0 (sm_103a)"; }

extern "C" const char *als_status_string(als_status s) {
    switch (s) {
    case ALS_OK: return "ALS_OK";
    case ALS_ERR_INVALID_ARG: return "ALS_ERR_INVALID_ARG";
    case ALS_ERR_IO: return "ALS_ERR_IO";
    case ALS_ERR_CUDA: return "ALS_ERR_CUDA";
    case ALS_ERR_NUMERIC: return "ALS_ERR_NUMERIC";
    case ALS_ERR_TIMEOUT: return "ALS_ERR_TIMEOUT";
    case ALS_ERR_UNSUPPORTED: return "ALS_ERR_UNSUPPORTED";
    case ALS_ERR_OUT_OF_MEMORY: return "ALS_ERR_OUT_OF_MEMORY";
    case ALS_ERR_NO_DEVICE: return "ALS_ERR_NO_DEVICE";
    }
    return "ALS_ERR_UNKNOWN";
}

extern "C" void als_config_default(als_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->f = 100;
    c->lambda = 0.05f;
    c->iters = 10;
    c->calculate_vtvs_type = ALS_VTVS_SMEM_ROW_MAJOR;
    c->solve_type = ALS_SOLVE_LU;
    c->smem_col_cnt = 32;
    c->m_batches = 1;
    c->n_batches = 1;
    c->precision = ALS_PREC_FROM_VTVS;
    c->refine_steps = 1;
    c->cond_threshold = 1e4f;
    c->cg_steps = 6;
    c->cg_tol = 1e-4f;
    c->use_graph = 1;
    c->autotune = 0;
    c->device = 0;
}

// Minimal INI reader for the reference's files (the keys of main.cpp:28-47): [section] headers,
// "key = value" lines, ';' / '#' comment lines and " ;" inline comments; names compare
// case-insensitively as inih does.
static bool parse_ini(const char *path, std::map<std::string, std::string> *kv) {
    std::ifstream in(path);
    if (!in) return false;
    std::string line, section;
    auto trim = [](std::string s) {
        size_t b = s.find_first_not_of(" \t\r\n"), e = s.find_last_not_of(" \t\r\n");
        return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
    };
    auto lower = [](std::string s) {
        for (auto &ch : s) ch = (char)std::tolower((unsigned char)ch);
        return s;
    };
    while (std::getline(in, line)) {
        line = trim(line);
        if (line.empty() || line[0] == ';' || line[0] == '#') continue;
        if (line[0] == '[') {
            size_t e = line.find(']');
            if (e == std::string::npos) return false;
            section = lower(trim(line.substr(1, e - 1)));
            continue;
        }
        size_t eq = line.find_first_of("=:");
        if (eq == std::string::npos) return false;
        std::string key = lower(trim(line.substr(0, eq)));
        std::string val = line.substr(eq + 1);
        size_t sc = val.find(" ;");
        if (sc != std::string::npos) val = val.substr(0, sc);
        (*kv)[section + "." + key] = trim(val);
    }
    return true;
}

extern "C" als_status als_config_from_ini(const char *path, als_config *cfg, int64_t *m,
                                          int64_t *n, int64_t *nnz_train, int64_t *nnz_test,
                                          int32_t *als_runs, char *data_folder,
                                          size_t data_folder_len) {
    if (!path || !cfg) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::map<std::string, std::string> kv;
    if (!parse_ini(path, &kv))
        return set_global_error(ALS_ERR_IO, std::string("Can't load ") + path);
    als_config_default(cfg);
    auto geti = [&](const char *k, long long d) -> long long {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::strtoll(it->second.c_str(), nullptr, 0);
    };
    auto getf = [&](const char *k, double d) -> double {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::strtod(it->second.c_str(), nullptr);
    };
    // main.cpp:28-47 (missing keys default to 0 there, as here)
    if (m) *m = geti("data.m", 0);
    if (n) *n = geti("data.n", 0);
    if (nnz_train) *nnz_train = geti("data.nnz_train", 0);
    if (nnz_test) *nnz_test = geti("data.nnz_test", 0);
    if (als_runs) *als_runs = (int32_t)geti("general.als_runs", 0);
    cfg->f = (int32_t)geti("als.f", 0);
    cfg->lambda = (float)getf("als.lambda", 0.0);
    cfg->iters = (int32_t)geti("als.als_iters", 0);
    cfg->calculate_vtvs_type = (int32_t)geti("als.als_calculate_vtvs_type", 0);
    cfg->solve_type = (int32_t)geti("als.als_solve_type", 0);
    cfg->m_batches = (int32_t)geti("als.m_batches", 0);
    cfg->n_batches = (int32_t)geti("als.n_batches", 0);
    cfg->smem_col_cnt = 32;  // hard-coded in main.cpp:43
    // [als_gb300]
    auto it = kv.find("als_gb300.precision");
    if (it != kv.end()) {
        std::string p = it->second;
        for (auto &ch : p) ch = (char)std::tolower((unsigned char)ch);
        if (p == "fp32") cfg->precision = ALS_PREC_FP32;
        else if (p == "bf16") cfg->precision = ALS_PREC_BF16;
        else if (p == "fp8") cfg->precision = ALS_PREC_FP8;
        else cfg->precision = (int32_t)std::strtol(p.c_str(), nullptr, 0);
    }
    cfg->refine_steps = (int32_t)geti("als_gb300.refine_steps", cfg->refine_steps);
    cfg->cond_threshold = (float)getf("als_gb300.cond_threshold", cfg->cond_threshold);
    cfg->cg_steps = (int32_t)geti("als_gb300.cg_steps", cfg->cg_steps);
    cfg->cg_tol = (float)getf("als_gb300.cg_tol", cfg->cg_tol);
    cfg->use_graph = (int32_t)geti("als_gb300.graph", cfg->use_graph);
    cfg->autotune = (int32_t)geti("als_gb300.autotune", cfg->autotune);
    if (data_folder && data_folder_len) {
        auto d = kv.find("data.data_folder");
        std::string s = d == kv.end() ? std::string() : d->second;
        std::snprintf(data_folder, data_folder_len, "%s", s.c_str());
    }
    return ALS_OK;
}

extern "C" als_status als_ini_get(const char *path, const char *section, const char *key,
                                   char *buf, size_t len) {
    if (!path || !section || !key || !buf || !len)
        return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::map<std::string, std::string> kv;
    if (!parse_ini(path, &kv))
        return set_global_error(ALS_ERR_IO, std::string("Can't load ") + path);
    std::string k = std::string(section) + "." + key;
    for (auto &ch : k) ch = (char)std::tolower((unsigned char)ch);
    auto it = kv.find(k);
    std::snprintf(buf, len, "%s", it == kv.end() ? "" : it->second.c_str());
    return ALS_OK;
}

extern "C" als_status als_host_alloc(size_t bytes, void **out) {
    if (!out) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    als_status s = check_device();
    if (s != ALS_OK) return s;
    G_CUDA(cudaMallocHost(out, bytes ? bytes : 1));
    return ALS_OK;
}

extern "C" als_status als_host_free(void *p) {
    if (p) G_CUDA(cudaFreeHost(p));
    return ALS_OK;
}

extern "C" als_status als_load_bin(const char *path, void *dst, size_t bytes) {
    if (!path || (!dst && bytes))
        return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::ifstream ifs(path, std::ios::binary | std::ios::ate);
    if (!ifs) return set_global_error(ALS_ERR_IO, std::string(path) + ": " + std::strerror(errno));
    size_t size = (size_t)ifs.tellg();
    if (size == 0) return set_global_error(ALS_ERR_IO, std::string(path) + " is empty");
    if (size != bytes)
        return set_global_error(ALS_ERR_IO, std::string(path) +
                                                ": file size does not match buffer size (" +
                                                std::to_string(size) + " != " +
                                                std::to_string(bytes) + ")");
    ifs.seekg(0, std::ios::beg);
    if (!ifs.read((char *)dst, (std::streamsize)bytes))
        return set_global_error(ALS_ERR_IO, std::string(path) + ": short read");
    return ALS_OK;
}

// ---------------------------------------------------------------------------------------------
// model
// ---------------------------------------------------------------------------------------------

static int effective_precision(const als_config &c) {
    if (c.precision != ALS_PREC_FROM_VTVS) return c.precision;
    return c.calculate_vtvs_type >= ALS_VTVS_SMEM_ROW_MAJOR_TENSOR ? ALS_PREC_BF16 : ALS_PREC_FP32;
}

static als_status validate_config(const als_config &c, std::string *why) {
    if (c.f < 1) { *why = "f must be >= 1"; return ALS_ERR_INVALID_ARG; }
    if (!(c.lambda >= 0.f) || !std::isfinite(c.lambda)) {
        *why = "lambda must be finite and >= 0";
        return ALS_ERR_INVALID_ARG;
    }
    if (c.iters < 0) { *why = "als_iters must be >= 0"; return ALS_ERR_INVALID_ARG; }
    if (c.calculate_vtvs_type < 0 || c.calculate_vtvs_type > 7) {
        *why = "als_calculate_vtvs_type must be 0..7";
        return ALS_ERR_INVALID_ARG;
    }
    if (c.solve_type < 0 || c.solve_type > ALS_SOLVE_AUTO) {
        *why = "als_solve_type must be 0..4";
        return ALS_ERR_INVALID_ARG;
    }
    if (c.cg_steps < 0) { *why = "cg_steps must be >= 0"; return ALS_ERR_INVALID_ARG; }
    int p = effective_precision(c);
    if (p < ALS_PREC_FP32 || p > ALS_PREC_FP8) {
        *why = "precision must be fp32, bf16 or fp8";
        return ALS_ERR_INVALID_ARG;
    }
    if (p == ALS_PREC_FP32 && !fp32_supported(c.f)) {
        *why = "f too large for the FP32 path (max 231)";
        return ALS_ERR_UNSUPPORTED;
    }
    if (p != ALS_PREC_FP32 && !tc_supported(c.f)) {
        *why = "f not supported by the tensor-core path (1..128)";
        return ALS_ERR_UNSUPPORTED;
    }
    return ALS_OK;
}

// Shape checks shared by als_create and als_reload.
static als_status check_views(const als_csr_view *csr, const als_csc_view *csc,
                              const als_coo_view *test) {
    if (!csr) return set_global_error(ALS_ERR_INVALID_ARG, "null train CSR");
    if (csr->rows < 1 || csr->cols < 1 || csr->nnz < 0 || csr->nnz > INT32_MAX ||
        csr->rows >= INT32_MAX || csr->cols >= INT32_MAX)
        return set_global_error(ALS_ERR_INVALID_ARG, "train shape out of range");
    if (!csr->row_ptrs || (csr->nnz > 0 && (!csr->col_idxs || !csr->vals)))
        return set_global_error(ALS_ERR_INVALID_ARG, "train CSR has null arrays");
    if (csc && (csc->rows != csr->rows || csc->cols != csr->cols || csc->nnz != csr->nnz ||
                !csc->col_ptrs || (csc->nnz > 0 && (!csc->row_idxs || !csc->vals))))
        return set_global_error(ALS_ERR_INVALID_ARG, "train CSC shape differs from CSR");
    if (test && (test->rows != csr->rows || test->cols != csr->cols || test->nnz < 0 ||
                 test->nnz > INT32_MAX ||
                 (test->nnz > 0 && (!test->row_idxs || !test->col_idxs || !test->vals))))
        return set_global_error(ALS_ERR_INVALID_ARG, "test COO shape differs from train");
    return ALS_OK;
}

// Copy the ratings into the handle's device arrays, validate them, build (or take) the CSC and
// the degree orders.  The device arrays and the scratch are allocated by create_impl.
static als_status upload_inputs(als_handle *h, const als_csr_view *csr, const als_csc_view *csc,
                                const als_coo_view *test, bool on_device) {
    std::string why;
    const int64_t m = h->m, n = h->n, nnz = h->nnz;
    cudaStream_t st = h->stream;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;

    // host-side structure checks (pointer arrays must be readable here)
    std::vector<int32_t> ptr_host;
    const int32_t *ptr_h = csr->row_ptrs;
    if (on_device) {
        ptr_host.resize((size_t)m + 1);
        H_CUDA(h, cudaMemcpy(ptr_host.data(), csr->row_ptrs, sizeof(int32_t) * (m + 1),
                             cudaMemcpyDeviceToHost));
        ptr_h = ptr_host.data();
    }
    if (!check_ptrs(ptr_h, m, nnz, &why)) return h_fail(h, ALS_ERR_INVALID_ARG, "train CSR: " + why);
    int32_t maxdeg_rows = 0;
    for (int64_t r = 0; r < m; ++r) maxdeg_rows = std::max(maxdeg_rows, ptr_h[r + 1] - ptr_h[r]);
    if (csc) {
        std::vector<int32_t> cptr_host;
        const int32_t *cptr_h = csc->col_ptrs;
        if (on_device) {
            cptr_host.resize((size_t)n + 1);
            H_CUDA(h, cudaMemcpy(cptr_host.data(), csc->col_ptrs, sizeof(int32_t) * (n + 1),
                                 cudaMemcpyDeviceToHost));
            cptr_h = cptr_host.data();
        }
        if (!check_ptrs(cptr_h, n, nnz, &why))
            return h_fail(h, ALS_ERR_INVALID_ARG, "train CSC: " + why);
    }

    // uploads
    H_CUDA(h, cudaMemcpyAsync(h->d_csr_ptr, csr->row_ptrs, sizeof(int32_t) * (m + 1), kind, st));
    if (nnz > 0) {
        H_CUDA(h, cudaMemcpyAsync(h->d_csr_idx, csr->col_idxs, sizeof(int32_t) * nnz, kind, st));
        H_CUDA(h, cudaMemcpyAsync(h->d_csr_val, csr->vals, sizeof(float) * nnz, kind, st));
    }
    if (h->nnz_test > 0) {
        H_CUDA(h, cudaMemcpyAsync(h->d_test_row, test->row_idxs, sizeof(int32_t) * h->nnz_test, kind, st));
        H_CUDA(h, cudaMemcpyAsync(h->d_test_col, test->col_idxs, sizeof(int32_t) * h->nnz_test, kind, st));
        H_CUDA(h, cudaMemcpyAsync(h->d_test_val, test->vals, sizeof(float) * h->nnz_test, kind, st));
    }
    // device-side validation of indices and values (no trap: counted and reported)
    H_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int32_t) * 8, st));
    H_CUDA(h, count_bad_entries(nnz, h->d_csr_idx, (int32_t)n, h->d_csr_val, h->d_flags, st));
    if (h->nnz_test > 0) {
        H_CUDA(h, count_bad_entries(h->nnz_test, h->d_test_row, (int32_t)m, h->d_test_val,
                                    h->d_flags + 1, st));
        H_CUDA(h, count_bad_entries(h->nnz_test, h->d_test_col, (int32_t)n, nullptr,
                                    h->d_flags + 1, st));
    }
    // CSC: uploaded, or built by the GPU transpose
    H_CUDA(h, cudaEventRecord(h->ev_transpose[0], st));
    if (csc) {
        H_CUDA(h, cudaMemcpyAsync(h->d_csc_ptr, csc->col_ptrs, sizeof(int32_t) * (n + 1), kind, st));
        if (nnz > 0) {
            H_CUDA(h, cudaMemcpyAsync(h->d_csc_idx, csc->row_idxs, sizeof(int32_t) * nnz, kind, st));
            H_CUDA(h, cudaMemcpyAsync(h->d_csc_val, csc->vals, sizeof(float) * nnz, kind, st));
        }
        H_CUDA(h, expand_rows(m, nnz, h->d_csr_ptr, h->d_coo_row, st));
        H_CUDA(h, count_bad_entries(nnz, h->d_csc_idx, (int32_t)m, h->d_csc_val, h->d_flags + 2, st));
        if (h->d_csc_perm) {  // a caller-given CSC invalidates the cached permutation
            cudaFree(h->d_csc_perm);
            h->d_csc_perm = nullptr;
        }
    } else {
        // the CSC -> CSR permutation is built on demand (als_update_values) from this pattern
        if (h->d_csc_perm) {
            cudaFree(h->d_csc_perm);
            h->d_csc_perm = nullptr;
        }
        H_CUDA(h, csr_to_csc_device(m, n, nnz, h->d_csr_ptr, h->d_csr_idx, h->d_csr_val,
                                    h->d_csc_ptr, h->d_csc_idx, h->d_csc_val, h->d_scratch, st,
                                    h->d_coo_row, nullptr));
    }
    H_CUDA(h, cudaEventRecord(h->ev_transpose[1], st));
    std::vector<int32_t> cptr((size_t)n + 1);
    int32_t bad[3] = {0, 0, 0};
    H_CUDA(h, cudaMemcpyAsync(cptr.data(), h->d_csc_ptr, sizeof(int32_t) * (n + 1),
                              cudaMemcpyDeviceToHost, st));
    H_CUDA(h, cudaMemcpyAsync(bad, h->d_flags, sizeof(bad), cudaMemcpyDeviceToHost, st));
    H_CUDA(h, cudaStreamSynchronize(st));
    if (bad[0]) return h_fail(h, ALS_ERR_INVALID_ARG,
                              "train CSR: " + std::to_string(bad[0]) +
                                  " entries with a column index out of range or a non-finite rating");
    if (bad[1]) return h_fail(h, ALS_ERR_INVALID_ARG,
                              "test COO: " + std::to_string(bad[1]) +
                                  " entries with an index out of range or a non-finite rating");
    if (bad[2]) return h_fail(h, ALS_ERR_INVALID_ARG, "train CSC: entries out of range");
    float tms = 0.f;
    H_CUDA(h, cudaEventElapsedTime(&tms, h->ev_transpose[0], h->ev_transpose[1]));
    h->stage_ms[3] = tms;
    int32_t maxdeg_cols = 0;
    for (int64_t c = 0; c < n; ++c) maxdeg_cols = std::max(maxdeg_cols, cptr[c + 1] - cptr[c]);
    h->maxdeg[0] = maxdeg_rows;
    h->maxdeg[1] = maxdeg_cols;
    h->host_ptr[0].assign(ptr_h, ptr_h + m + 1);
    h->host_ptr[1] = std::move(cptr);
    H_CUDA(h, degree_order_device(m, h->d_csr_ptr, maxdeg_rows, h->d_order[0], h->d_scratch, st));
    H_CUDA(h, degree_order_device(n, h->d_csc_ptr, maxdeg_cols, h->d_order[1], h->d_scratch, st));
    H_CUDA(h, cudaStreamSynchronize(st));
    data_changed(h);
    return tc_values_changed(h);
}

static als_status create_impl(const als_config *cfg, const als_csr_view *csr,
                              const als_csc_view *csc, const als_coo_view *test, bool on_device,
                              als_handle **out) {
    if (!cfg || !csr || !out) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    std::string why;
    als_status s = validate_config(*cfg, &why);
    if (s != ALS_OK) return set_global_error(s, why);
    s = check_views(csr, csc, test);
    if (s != ALS_OK) return s;
    s = check_device();
    if (s != ALS_OK) return s;
    G_CUDA(cudaSetDevice(cfg->device));

    std::unique_ptr<als_handle> h(new als_handle());
    h->cfg = *cfg;
    h->precision = effective_precision(*cfg);
    h->m = csr->rows;
    h->n = csr->cols;
    h->nnz = csr->nnz;
    h->nnz_test = test ? test->nnz : 0;
    h->f = cfg->f;
    G_CUDA(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;

    // device allocations (all of them up front: nothing allocates inside a sweep)
    const int64_t m = h->m, n = h->n, nnz = h->nnz, f = h->f;
    H_CUDA(h.get(), dalloc(&h->d_csr_ptr, m + 1));
    H_CUDA(h.get(), dalloc(&h->d_csr_idx, nnz));
    H_CUDA(h.get(), dalloc(&h->d_csr_val, nnz));
    H_CUDA(h.get(), dalloc(&h->d_csc_ptr, n + 1));
    H_CUDA(h.get(), dalloc(&h->d_csc_idx, nnz));
    H_CUDA(h.get(), dalloc(&h->d_csc_val, nnz));
    H_CUDA(h.get(), dalloc(&h->d_coo_row, nnz));
    H_CUDA(h.get(), dalloc(&h->d_U, m * f));
    H_CUDA(h.get(), dalloc(&h->d_V, n * f));
    H_CUDA(h.get(), dalloc(&h->d_order[0], m));
    H_CUDA(h.get(), dalloc(&h->d_order[1], n));
    H_CUDA(h.get(), dalloc(&h->d_flags, 8));
    H_CUDA(h.get(), dalloc(&h->d_partials, rmse_scratch_bytes() / sizeof(double) + 1));
    H_CUDA(h.get(), dalloc(&h->d_scalar, 4));
    if (h->nnz_test > 0) {
        H_CUDA(h.get(), dalloc(&h->d_test_row, h->nnz_test));
        H_CUDA(h.get(), dalloc(&h->d_test_col, h->nnz_test));
        H_CUDA(h.get(), dalloc(&h->d_test_val, h->nnz_test));
    }
    const size_t scratch_bytes = std::max(transpose_scratch_bytes(m, n, nnz),
                                          std::max(degree_order_scratch_bytes(m),
                                                   degree_order_scratch_bytes(n)));
    H_CUDA(h.get(), cudaMalloc(&h->d_scratch, scratch_bytes));
    for (int k = 0; k < 2; ++k) H_CUDA(h.get(), cudaEventCreate(&h->ev_transpose[k]));
    als_status ps = prepare_precision_path(h.get());
    if (ps != ALS_OK) return ps;
    s = upload_inputs(h.get(), csr, csc, test, on_device);
    if (s != ALS_OK) return s;
    h->h_U.assign((size_t)(m * f), 0.f);
    h->h_V.assign((size_t)(n * f), 0.f);
    *out = h.release();
    return ALS_OK;
}

extern "C" als_status als_reload(als_handle *h, const als_csr_view *csr, const als_csc_view *csc,
                                 const als_coo_view *test) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    als_status s = check_views(csr, csc, test);
    if (s != ALS_OK) return s;
    if (csr->rows != h->m || csr->cols != h->n || csr->nnz != h->nnz ||
        (test ? test->nnz : 0) != h->nnz_test)
        return h_fail(h, ALS_ERR_INVALID_ARG, "reload: sizes differ from the handle's");
    cudaSetDevice(h->cfg.device);
    return upload_inputs(h, csr, csc, test, false);
}

extern "C" als_status als_create(const als_config *cfg, const als_csr_view *csr,
                                 const als_csc_view *csc, const als_coo_view *test,
                                 als_handle **out) {
    return create_impl(cfg, csr, csc, test, false, out);
}

extern "C" als_status als_create_device(const als_config *cfg, const als_csr_view *csr,
                                        const als_csc_view *csc, const als_coo_view *test,
                                        als_handle **out) {
    return create_impl(cfg, csr, csc, test, true, out);
}

als_handle::~als_handle() {
    release_precision_path(this);
    void *ptrs[] = {d_csr_ptr, d_csr_idx, d_csr_val, d_csc_ptr, d_csc_idx, d_csc_val,
                    d_coo_row, d_csc_perm, d_U, d_V, d_order[0], d_order[1], d_flags,
                    d_partials, d_scalar, d_test_row, d_test_col, d_test_val, d_scratch};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto e : events) cudaEventDestroy(e);
    for (auto e : ev_transpose)
        if (e) cudaEventDestroy(e);
    if (own_stream) cudaStreamDestroy(own_stream);
}

extern "C" als_status als_destroy(als_handle *h) {
    if (!h) return ALS_OK;
    cudaSetDevice(h->cfg.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
    return ALS_OK;
}

extern "C" const char *als_last_error(const als_handle *h) {
    if (h) return h->last_error.c_str();
    return g_error.c_str();
}

extern "C" als_status als_set_stream(als_handle *h, void *stream) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    invalidate_graphs(h);
    return ALS_OK;
}

extern "C" als_status als_update_values(als_handle *h, const float *vals) {
    if (!h || (!vals && h->nnz)) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    cudaSetDevice(h->cfg.device);
    if (h->nnz == 0) return ALS_OK;
    cudaStream_t st = h->stream;
    H_CUDA(h, cudaMemcpyAsync(h->d_csr_val, vals, sizeof(float) * h->nnz,
                              cudaMemcpyHostToDevice, st));
    return refresh_csc_values(h);
}

extern "C" als_status als_init_factors(als_handle *h) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    cudaSetDevice(h->cfg.device);
    if (h->cfg.autotune) reset_tuning(h);  // a new run re-tunes the ALS_SOLVE_AUTO plan
    // als_model.cu:1772-1777: srand(0), VT[k] = 0.2*((float)rand()/(float)RAND_MAX), UT = 0,
    // generated on the GPU bit for bit (init.cu: glibc's rand() sequence by jump-ahead)
    H_CUDA(h, init_factors_device(h->m, h->n, h->f, h->d_U, h->d_V, h->stream));
    return ALS_OK;
}

extern "C" als_status als_half_sweep(als_handle *h, int32_t side) {
    if (!h || (side != 0 && side != 1)) return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    cudaSetDevice(h->cfg.device);
    H_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int32_t) * 4, h->stream));
    als_status s = run_half_sweep(h, side);
    if (s != ALS_OK) return s;
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    s = read_stage_ms(h, side);
    if (s != ALS_OK) return s;
    return check_sweep_flags(h);
}

static als_status rmse_impl(als_handle *h, bool test, double *out);

// Epochs with an event log attached: als_iter = 1..iters, the ALS_ITER / ALS_UPDATE_U /
// ALS_UPDATE_V events of als_model.cu:1792-1801, :2021-2034, :2259-2261 (each half-sweep is
// waited for before its event finishes, so the event times its device work; no CUDA graph), the
// optional "RMSE test" line of :2269-2274, and als_iter = 0 afterwards (:2277-2279).
static als_status iterate_logged(als_handle *h, int32_t iters) {
    als_log *lg = h->log;
    const bool cout = h->log_cout;
    for (int32_t it = 0; it < iters; ++it) {
        als::log_set_als_iter(lg, it + 1);
        als::log_event(lg, ALS_EVENT_ITER, false, false);
        int64_t launches = 0;
        for (int side = 0; side < 2; ++side) {
            const int32_t ev = side == 0 ? ALS_EVENT_UPDATE_U : ALS_EVENT_UPDATE_V;
            als::log_event(lg, ev, false, false);
            als_status s = run_half_sweep(h, side);
            if (s != ALS_OK) return s;
            H_CUDA(h, cudaStreamSynchronize(h->stream));
            launches += h->counters[0];
            s = read_stage_ms(h, side);
            if (s != ALS_OK) return s;
            als::log_event(lg, ev, true, cout);
        }
        h->counters[0] = launches;
        ++h->eager_epochs;
        als::log_event(lg, ALS_EVENT_ITER, true, cout);
        if (h->log_iter_rmse && it < iters - 1) {
            double r = 0.0;
            als_status s = rmse_impl(h, true, &r);
            if (s != ALS_OK) return s;
            char buf[64];
            std::snprintf(buf, sizeof(buf), "%f", (double)(float)r);  // std::to_string(float)
            als::log_text(lg, std::string("RMSE test: ") + buf, cout);
        }
    }
    als::log_set_als_iter(lg, 0);
    return ALS_OK;
}

extern "C" als_status als_iterate(als_handle *h, int32_t iters) {
    if (!h || iters < 0) return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    cudaSetDevice(h->cfg.device);
    H_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(int32_t) * 4, h->stream));
    if (h->log) {
        als_status s = iterate_logged(h, iters);
        if (s != ALS_OK) return s;
        return check_sweep_flags(h);
    }
    als_status s = run_epochs(h, iters);
    if (s != ALS_OK) return s;
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    for (int side = 0; side < 2 && iters > 0; ++side) {
        s = read_stage_ms(h, side);
        if (s != ALS_OK) return s;
    }
    return check_sweep_flags(h);
}

extern "C" als_status als_train(als_handle *h) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    if (h->log) als::log_text(h->log, "als model training started", h->log_cout);  // :1768-1770
    als_status s = als_init_factors(h);
    if (s != ALS_OK) return s;
    if (h->log) als::log_text(h->log, "factors initialization done", h->log_cout);  // :1786-1788
    s = als_iterate(h, h->cfg.iters);
    if (s != ALS_OK) return s;
    // final result from device to host (als_model.cu:2283-2284)
    H_CUDA(h, cudaMemcpyAsync(h->h_V.data(), h->d_V, sizeof(float) * h->n * h->f,
                              cudaMemcpyDeviceToHost, h->stream));
    H_CUDA(h, cudaMemcpyAsync(h->h_U.data(), h->d_U, sizeof(float) * h->m * h->f,
                              cudaMemcpyDeviceToHost, h->stream));
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->log) als::log_text(h->log, "als model training done", h->log_cout);  // :2286-2288
    return ALS_OK;
}

static als_status rmse_impl(als_handle *h, bool test, double *out) {
    if (!h || !out) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    cudaSetDevice(h->cfg.device);
    const int64_t nnz = test ? h->nnz_test : h->nnz;
    if (nnz == 0) { *out = 0.0; return ALS_OK; }
    const int32_t *rows = test ? h->d_test_row : h->d_coo_row;
    const int32_t *cols = test ? h->d_test_col : h->d_csr_idx;
    const float *vals = test ? h->d_test_val : h->d_csr_val;
    H_CUDA(h, launch_sq_error(nnz, rows, cols, vals, h->d_U, h->d_V, h->f, h->d_partials,
                              h->d_scalar, h->stream));
    double sum = 0.0;
    H_CUDA(h, cudaMemcpyAsync(&sum, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    *out = std::sqrt(sum / (double)nnz);
    return ALS_OK;
}

extern "C" als_status als_rmse_test(als_handle *h, double *out) { return rmse_impl(h, true, out); }
extern "C" als_status als_rmse_train(als_handle *h, double *out) { return rmse_impl(h, false, out); }

extern "C" als_status als_get_factors(als_handle *h, float *U, float *V) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    cudaSetDevice(h->cfg.device);
    if (U) H_CUDA(h, cudaMemcpyAsync(U, h->d_U, sizeof(float) * h->m * h->f, cudaMemcpyDeviceToHost, h->stream));
    if (V) H_CUDA(h, cudaMemcpyAsync(V, h->d_V, sizeof(float) * h->n * h->f, cudaMemcpyDeviceToHost, h->stream));
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    return ALS_OK;
}

extern "C" als_status als_set_factors(als_handle *h, const float *U, const float *V) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    cudaSetDevice(h->cfg.device);
    if (U) H_CUDA(h, cudaMemcpyAsync(h->d_U, U, sizeof(float) * h->m * h->f, cudaMemcpyHostToDevice, h->stream));
    if (V) H_CUDA(h, cudaMemcpyAsync(h->d_V, V, sizeof(float) * h->n * h->f, cudaMemcpyHostToDevice, h->stream));
    H_CUDA(h, cudaStreamSynchronize(h->stream));
    return ALS_OK;
}

extern "C" als_status als_get_device_factors(als_handle *h, float **U, float **V) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    if (U) *U = h->d_U;
    if (V) *V = h->d_V;
    return ALS_OK;
}

extern "C" als_status als_save_libmf(als_handle *h, const char *path) {
    if (!h || !path) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::vector<float> U((size_t)(h->m * h->f)), V((size_t)(h->n * h->f));
    als_status s = als_get_factors(h, U.data(), V.data());
    if (s != ALS_OK) return s;
    // mean of the training ratings (the reference: cublasSasum / nnz, als_model.cu:2295-2297)
    float mean_rating = 0.f;
    if (h->nnz > 0) {
        std::vector<float> vals((size_t)h->nnz);
        H_CUDA(h, cudaMemcpy(vals.data(), h->d_csr_val, sizeof(float) * h->nnz,
                             cudaMemcpyDeviceToHost));
        double sum = 0.0;
        for (float v : vals) sum += std::fabs((double)v);
        mean_rating = (float)(sum / (double)h->nnz);
    }
    std::ofstream out(path, std::ios::binary);
    if (!out) return h_fail(h, ALS_ERR_IO, std::string(path) + ": cannot open for writing");
    // als_model.cu:2294-2312: int loss=0, int m, int n, int f, float mean, U, V
    int32_t hdr[4] = {0, (int32_t)h->m, (int32_t)h->n, h->f};
    out.write((const char *)hdr, sizeof(hdr));
    out.write((const char *)&mean_rating, sizeof(float));
    out.write((const char *)U.data(), (std::streamsize)(sizeof(float) * U.size()));
    out.write((const char *)V.data(), (std::streamsize)(sizeof(float) * V.size()));
    if (!out) return h_fail(h, ALS_ERR_IO, std::string(path) + ": write failed");
    return ALS_OK;
}

extern "C" als_status als_get_shape(const als_handle *h, int64_t *m, int64_t *n, int32_t *f,
                                    int64_t *nnz_train, int64_t *nnz_test) {
    if (!h) return set_global_error(ALS_ERR_INVALID_ARG, "null handle");
    if (m) *m = h->m;
    if (n) *n = h->n;
    if (f) *f = h->f;
    if (nnz_train) *nnz_train = h->nnz;
    if (nnz_test) *nnz_test = h->nnz_test;
    return ALS_OK;
}

extern "C" als_status als_get_stage_ms(const als_handle *h, double out[4]) {
    if (!h || !out) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    for (int i = 0; i < 4; ++i) out[i] = h->stage_ms[i];
    return ALS_OK;
}

extern "C" als_status als_get_counters(const als_handle *h, int64_t out[3]) {
    if (!h || !out) return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    for (int i = 0; i < 3; ++i) out[i] = h->counters[i];
    return ALS_OK;
}

// ---------------------------------------------------------------------------------------------
// standalone index entry points
// ---------------------------------------------------------------------------------------------

extern "C" als_status als_csr_to_csc_device(const als_csr_view *csr, int32_t *col_ptrs,
                                            int32_t *row_idxs, float *vals, void *stream) {
    if (!csr || !col_ptrs || (csr->nnz > 0 && (!row_idxs || !vals)))
        return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    if (csr->rows < 0 || csr->cols < 0 || csr->nnz < 0 || csr->nnz > INT32_MAX)
        return set_global_error(ALS_ERR_INVALID_ARG, "shape out of range");
    cudaStream_t st = (cudaStream_t)stream;
    void *scratch = nullptr;
    G_CUDA(cudaMallocAsync(&scratch, transpose_scratch_bytes(csr->rows, csr->cols, csr->nnz), st));
    cudaError_t e = csr_to_csc_device(csr->rows, csr->cols, csr->nnz, csr->row_ptrs,
                                      csr->col_idxs, csr->vals, col_ptrs, row_idxs, vals, scratch,
                                      st, nullptr, nullptr);
    cudaFreeAsync(scratch, st);
    if (e != cudaSuccess)
        return set_global_error(ALS_ERR_CUDA, std::string("csr_to_csc: ") + cudaGetErrorString(e));
    return ALS_OK;
}

extern "C" als_status als_csr_to_csc(const als_csr_view *csr, int32_t *col_ptrs,
                                     int32_t *row_idxs, float *vals) {
    if (!csr || !col_ptrs || (csr->nnz > 0 && (!row_idxs || !vals || !csr->col_idxs || !csr->vals)))
        return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    std::string why;
    if (csr->rows < 0 || csr->cols < 0 || csr->nnz < 0 || csr->nnz > INT32_MAX)
        return set_global_error(ALS_ERR_INVALID_ARG, "shape out of range");
    if (!check_ptrs(csr->row_ptrs, csr->rows, csr->nnz, &why))
        return set_global_error(ALS_ERR_INVALID_ARG, why);
    for (int64_t k = 0; k < csr->nnz; ++k)
        if (csr->col_idxs[k] < 0 || csr->col_idxs[k] >= csr->cols)
            return set_global_error(ALS_ERR_INVALID_ARG,
                                    "column index out of range at " + std::to_string(k));
    als_status s = check_device();
    if (s != ALS_OK) return s;
    const int64_t rows = csr->rows, cols = csr->cols, nnz = csr->nnz;
    cudaStream_t st;
    G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int32_t *d_ptr = nullptr, *d_idx = nullptr, *d_cptr = nullptr, *d_ridx = nullptr;
    float *d_val = nullptr, *d_cval = nullptr;
    void *scratch = nullptr;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    step(dalloc(&d_ptr, rows + 1));
    step(dalloc(&d_idx, nnz));
    step(dalloc(&d_val, nnz));
    step(dalloc(&d_cptr, cols + 1));
    step(dalloc(&d_ridx, nnz));
    step(dalloc(&d_cval, nnz));
    if (e == cudaSuccess) step(cudaMalloc(&scratch, transpose_scratch_bytes(rows, cols, nnz)));
    if (e == cudaSuccess) {
        step(cudaMemcpyAsync(d_ptr, csr->row_ptrs, sizeof(int32_t) * (rows + 1), cudaMemcpyHostToDevice, st));
        if (nnz > 0) {
            step(cudaMemcpyAsync(d_idx, csr->col_idxs, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, st));
            step(cudaMemcpyAsync(d_val, csr->vals, sizeof(float) * nnz, cudaMemcpyHostToDevice, st));
        }
        step(csr_to_csc_device(rows, cols, nnz, d_ptr, d_idx, d_val, d_cptr, d_ridx, d_cval, scratch, st, nullptr, nullptr));
        step(cudaMemcpyAsync(col_ptrs, d_cptr, sizeof(int32_t) * (cols + 1), cudaMemcpyDeviceToHost, st));
        if (nnz > 0) {
            step(cudaMemcpyAsync(row_idxs, d_ridx, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, st));
            step(cudaMemcpyAsync(vals, d_cval, sizeof(float) * nnz, cudaMemcpyDeviceToHost, st));
        }
        step(cudaStreamSynchronize(st));
    }
    void *all[] = {d_ptr, d_idx, d_val, d_cptr, d_ridx, d_cval, scratch};
    for (void *p : all)
        if (p) cudaFree(p);
    cudaStreamDestroy(st);
    if (e != cudaSuccess)
        return set_global_error(e == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA,
                                std::string("csr_to_csc: ") + cudaGetErrorString(e));
    return ALS_OK;
}

extern "C" als_status als_partition_rows(int64_t rows, const int32_t *row_ptrs, int32_t nparts,
                                         double row_weight, int64_t *bounds) {
    if (rows < 0 || nparts < 1 || !bounds || (rows > 0 && !row_ptrs) || !(row_weight >= 0.0) ||
        !std::isfinite(row_weight))
        return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    std::string why;
    if (rows > 0 && !check_ptrs(row_ptrs, rows, row_ptrs[rows], &why))
        return set_global_error(ALS_ERR_INVALID_ARG, why);
    const double total = rows > 0 ? (double)row_ptrs[rows] - row_ptrs[0] + row_weight * rows : 0.0;
    bounds[0] = 0;
    int64_t r = 0;
    double before = 0.0;  // weight of rows [0, r)
    for (int32_t k = 1; k < nparts; ++k) {
        const double target = total * k / nparts;
        // a row joins the earlier part while its midpoint lies before the target
        while (r < rows) {
            const double w = (double)(row_ptrs[r + 1] - row_ptrs[r]) + row_weight;
            if (before + 0.5 * w >= target) break;
            before += w;
            ++r;
        }
        bounds[k] = r;
    }
    bounds[nparts] = rows;
    return ALS_OK;
}

extern "C" als_status als_degree_order(int64_t rows, const int32_t *row_ptrs, int32_t *perm) {
    if (rows < 0 || (rows > 0 && (!row_ptrs || !perm)) || rows >= INT32_MAX)
        return set_global_error(ALS_ERR_INVALID_ARG, "bad argument");
    if (rows == 0) return ALS_OK;
    std::string why;
    if (!check_ptrs(row_ptrs, rows, row_ptrs[rows], &why))
        return set_global_error(ALS_ERR_INVALID_ARG, why);
    als_status s = check_device();
    if (s != ALS_OK) return s;
    int32_t maxd = 0;
    for (int64_t r = 0; r < rows; ++r) maxd = std::max(maxd, row_ptrs[r + 1] - row_ptrs[r]);
    cudaStream_t st;
    G_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int32_t *d_ptr = nullptr, *d_perm = nullptr;
    void *scratch = nullptr;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    step(dalloc(&d_ptr, rows + 1));
    step(dalloc(&d_perm, rows));
    if (e == cudaSuccess) step(cudaMalloc(&scratch, degree_order_scratch_bytes(rows)));
    if (e == cudaSuccess) {
        step(cudaMemcpyAsync(d_ptr, row_ptrs, sizeof(int32_t) * (rows + 1), cudaMemcpyHostToDevice, st));
        step(degree_order_device(rows, d_ptr, maxd, d_perm, scratch, st));
        step(cudaMemcpyAsync(perm, d_perm, sizeof(int32_t) * rows, cudaMemcpyDeviceToHost, st));
        step(cudaStreamSynchronize(st));
    }
    void *all[] = {d_ptr, d_perm, scratch};
    for (void *p : all)
        if (p) cudaFree(p);
    cudaStreamDestroy(st);
    if (e != cudaSuccess)
        return set_global_error(ALS_ERR_CUDA, std::string("degree_order: ") + cudaGetErrorString(e));
    return ALS_OK;
}
