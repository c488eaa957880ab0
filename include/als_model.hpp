// als_model.hpp — header-only C++ face of the C ABI with the reference's types and names, so a
// caller written against vserdyuk/cuda_als (its main.cpp) compiles unchanged against this library:
//
//   host_sparse_matrix train(m, n, nnz_train);                 // cuda_sparse_matrix.h:8-38
//   train.load_csc(...); train.load_csr(...); train.load_coo(...);
//   host_sparse_matrix test(m, n, nnz_test); test.load_coo(...);
//   als_model model(train, test, f, lambda, iters, vtvs, solve, smem_col_cnt,
//                   m_batches, n_batches);                     // als_model.h:29-32
//   model.train(); model.rsme_test(); model.save_libmf(path);
//   model.set_logger(g_logger);   // the lines its train() writes into the global g_logger
//
// Differences a caller can see: errors throw als_gb300_error (the reference exit(1)s inside
// CUDA_CHECK, cuda_common.h:13-91); SOLVE_TYPE has two more values (CHOLESKY, AUTO); h_UT / h_VT
// are the row-contiguous m x f / n x f factor tables the reference keeps under those names,
// filled by train(); d_UT / d_VT point at the library's device tables.  Link with
// -lals_gb300 (cuda_als_gb300/libals_gb300.so).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "als_error.hpp"
#include "als_gb300.h"
#include "als_logger.hpp"

// Host ratings of one matrix in page-locked memory (cudaMallocHost, as the reference), loaded
// from the reference's raw .bin files (cuda_sparse_matrix.cpp:6-69).  CSR and COO share the
// values and column indices; whichever of load_csr / load_coo runs first reads them.
struct host_sparse_matrix {
    host_sparse_matrix(size_t row_cnt_, size_t col_cnt_, size_t val_cnt_)
        : row_cnt(row_cnt_), col_cnt(col_cnt_), val_cnt(val_cnt_) {}
    ~host_sparse_matrix() {
        for (void *p : {(void *)h_csr_coo_vals, (void *)h_csr_row_ptrs, (void *)h_csr_coo_col_idxs,
                        (void *)h_coo_row_idxs, (void *)h_csc_vals, (void *)h_csc_row_idxs,
                        (void *)h_csc_col_ptrs})
            if (p) als_host_free(p);
    }
    host_sparse_matrix(const host_sparse_matrix &) = delete;
    host_sparse_matrix &operator=(const host_sparse_matrix &) = delete;

    void load_csr(std::string vals_path, std::string row_ptrs_path, std::string col_idxs_path) {
        if (!has_coo) {
            malloc_load_file(vals_path, (void **)&h_csr_coo_vals, val_cnt * sizeof(float));
            malloc_load_file(col_idxs_path, (void **)&h_csr_coo_col_idxs, val_cnt * sizeof(int));
        }
        malloc_load_file(row_ptrs_path, (void **)&h_csr_row_ptrs, (row_cnt + 1) * sizeof(int));
        has_csr = true;
    }
    void load_csc(std::string vals_path, std::string row_idxs_path, std::string col_ptrs_path) {
        malloc_load_file(vals_path, (void **)&h_csc_vals, val_cnt * sizeof(float));
        malloc_load_file(row_idxs_path, (void **)&h_csc_row_idxs, val_cnt * sizeof(int));
        malloc_load_file(col_ptrs_path, (void **)&h_csc_col_ptrs, (col_cnt + 1) * sizeof(int));
        has_csc = true;
    }
    void load_coo(std::string vals_path, std::string row_idxs_path, std::string col_idxs_path) {
        if (!has_csr) {
            malloc_load_file(vals_path, (void **)&h_csr_coo_vals, val_cnt * sizeof(float));
            malloc_load_file(col_idxs_path, (void **)&h_csr_coo_col_idxs, val_cnt * sizeof(int));
        }
        malloc_load_file(row_idxs_path, (void **)&h_coo_row_idxs, val_cnt * sizeof(int));
        has_coo = true;
    }
    // Pinned allocation of buf_size bytes filled from `path` (whose size must be buf_size).
    static void malloc_load_file(std::string path, void **host_ptr, size_t buf_size) {
        void *p = nullptr;
        als_gb300_detail::check(als_host_alloc(buf_size ? buf_size : 1, &p));
        const als_status s = als_load_bin(path.c_str(), p, buf_size);
        if (s != ALS_OK) {
            als_host_free(p);
            als_gb300_detail::check(s);
        }
        if (*host_ptr) als_host_free(*host_ptr);
        *host_ptr = p;
    }

    bool has_coo = false;
    bool has_csr = false;
    bool has_csc = false;

    size_t row_cnt = 0;
    size_t col_cnt = 0;
    size_t val_cnt = 0;

    float *h_csr_coo_vals = nullptr;
    int *h_csr_row_ptrs = nullptr;
    int *h_csr_coo_col_idxs = nullptr;

    int *h_coo_row_idxs = nullptr;

    float *h_csc_vals = nullptr;
    int *h_csc_row_idxs = nullptr;
    int *h_csc_col_ptrs = nullptr;
};

struct als_model {
    enum class CALCULATE_VTVS_TYPE {
        SIMPLE = 0,
        SMEM_ROW_MAJOR,
        SMEM_COL_MAJOR,
        SMEM_ROW_MAJOR_NO_CALC,
        SMEM_COL_MAJOR_TWO_THREADS,
        SMEM_ROW_MAJOR_TENSOR,
        SMEM_ROW_MAJOR_TENSOR_SYMMETRIC,
        SMEM_ROW_MAJOR_TENSOR_SYMMETRIC_MULT_FRAG
    };
    enum class SOLVE_TYPE { LU = 0, CUMF_ALS_CG_FP16, CUMF_ALS_CG_FP32, CHOLESKY, AUTO };

    // Uploads both matrices (train: CSR required, CSC optional — built on the GPU when absent —
    // and its COO rows; test: COO) and allocates the factors.  The [als_gb300] options keep their
    // defaults (als_config_default); use the C ABI on handle() for anything else.
    als_model(host_sparse_matrix &host_train_ratings, host_sparse_matrix &host_test_ratings,
              int f_, float lambda_, int iters_, CALCULATE_VTVS_TYPE calculate_vtvs_type_,
              SOLVE_TYPE solve_type_, int smem_col_cnt_, int m_batches_, int n_batches_)
        : als_model(host_train_ratings, host_test_ratings,
                    make_config(f_, lambda_, iters_, calculate_vtvs_type_, solve_type_,
                                smem_col_cnt_, m_batches_, n_batches_)) {}

    // The same from a full configuration (e.g. als_config_from_ini, [als_gb300] options included).
    als_model(host_sparse_matrix &host_train_ratings, host_sparse_matrix &host_test_ratings,
              const als_config &cfg)
        : m((int)host_train_ratings.row_cnt), n((int)host_train_ratings.col_cnt),
          m_batches(cfg.m_batches), n_batches(cfg.n_batches), f(cfg.f), lambda(cfg.lambda),
          iters(cfg.iters), calculate_vtvs_type((CALCULATE_VTVS_TYPE)cfg.calculate_vtvs_type),
          solve_type((SOLVE_TYPE)cfg.solve_type), smem_col_cnt(cfg.smem_col_cnt) {
        const host_sparse_matrix &tr = host_train_ratings, &te = host_test_ratings;
        if (!tr.has_csr) throw als_gb300_error(ALS_ERR_INVALID_ARG, "train ratings need CSR");
        als_csr_view csr{(int64_t)tr.row_cnt, (int64_t)tr.col_cnt, (int64_t)tr.val_cnt,
                         tr.h_csr_row_ptrs, tr.h_csr_coo_col_idxs, tr.h_csr_coo_vals};
        als_csc_view csc{(int64_t)tr.row_cnt, (int64_t)tr.col_cnt, (int64_t)tr.val_cnt,
                         tr.h_csc_col_ptrs, tr.h_csc_row_idxs, tr.h_csc_vals};
        als_coo_view coo{(int64_t)te.row_cnt, (int64_t)te.col_cnt, (int64_t)te.val_cnt,
                         te.h_coo_row_idxs, te.h_csr_coo_col_idxs, te.h_csr_coo_vals};
        als_gb300_detail::check(als_create(&cfg, &csr, tr.has_csc ? &csc : nullptr,
                                           te.has_coo ? &coo : nullptr, &h_));
        als_gb300_detail::check(als_get_device_factors(h_, &d_UT, &d_VT), h_);
        hu_.assign((size_t)m * f, 0.f);
        hv_.assign((size_t)n * f, 0.f);
        h_UT = hu_.data();
        h_VT = hv_.data();
    }
    ~als_model() {
        if (h_) als_destroy(h_);
    }
    als_model(const als_model &) = delete;
    als_model &operator=(const als_model &) = delete;

    // als_model.cu:1766-2289: srand(0) init, iters x (U, V) half-sweeps, factors copied to host.
    void train() {
        if (logger_) als_gb300_detail::check(als_set_log(h_, logger_->handle(), iter_rmse_, cout_), h_);
        const als_status s = als_train(h_);
        if (logger_) logger_->pull();  // train() leaves als_iter = 0, as the reference's
        als_gb300_detail::check(s, h_);
        als_gb300_detail::check(als_get_factors(h_, h_UT, h_VT), h_);
    }
    // Write train()'s lines into `lg` (the reference writes them into its global g_logger):
    // per-iteration ALS_UPDATE_U / ALS_UPDATE_V / ALS_ITER events, with iter_rmse the test RMSE
    // after every iteration but the last (its CALC_ITER_RMSE build); write_cout echoes them.
    void set_logger(logger &lg, bool iter_rmse = false, bool write_cout = true) {
        logger_ = &lg;
        iter_rmse_ = iter_rmse ? 1 : 0;
        cout_ = write_cout ? 1 : 0;
    }
    float rsme_train() { return (float)rmse(false); }
    float rsme_test() { return (float)rmse(true); }
    void save_libmf(const char *path) { als_gb300_detail::check(als_save_libmf(h_, path), h_); }

    static std::string to_string(CALCULATE_VTVS_TYPE t) {
        static const char *names[] = {"SIMPLE",
                                      "SMEM_ROW_MAJOR",
                                      "SMEM_COL_MAJOR",
                                      "SMEM_ROW_MAJOR_NO_CALC",
                                      "SMEM_COL_MAJOR_TWO_THREADS",
                                      "SMEM_ROW_MAJOR_TENSOR",
                                      "SMEM_ROW_MAJOR_TENSOR_SYMMETRIC",
                                      "SMEM_ROW_MAJOR_TENSOR_SYMMETRIC_MULT_FRAG"};
        const int k = (int)t;
        return k >= 0 && k < 8 ? names[k] : "UNKNOWN";
    }
    static std::string to_string(SOLVE_TYPE t) {
        static const char *names[] = {"LU", "CUMF_ALS_CG_FP16", "CUMF_ALS_CG_FP32", "CHOLESKY",
                                      "AUTO"};
        const int k = (int)t;
        return k >= 0 && k < 5 ? names[k] : "UNKNOWN";
    }

    // The C handle, for the calls the reference does not have (streams, half-sweeps, timing,
    // the adjoint, re-uploads).
    als_handle *handle() { return h_; }

    int m;  // number of users
    int n;  // number of items
    int m_batches;
    int n_batches;
    int f;  // number of factors
    float lambda;
    int iters;

    float *h_VT = nullptr;  // host item factors, n x f row-contiguous (filled by train())
    float *d_VT = nullptr;  // device item factors (owned by the library)
    float *h_UT = nullptr;  // host user factors, m x f row-contiguous (filled by train())
    float *d_UT = nullptr;  // device user factors (owned by the library)

    CALCULATE_VTVS_TYPE calculate_vtvs_type;
    SOLVE_TYPE solve_type;
    int smem_col_cnt;

private:
    static als_config make_config(int f_, float lambda_, int iters_, CALCULATE_VTVS_TYPE vtvs,
                                  SOLVE_TYPE solve, int smem_col_cnt_, int m_batches_,
                                  int n_batches_) {
        als_config cfg;
        als_config_default(&cfg);
        cfg.f = f_;
        cfg.lambda = lambda_;
        cfg.iters = iters_;
        cfg.calculate_vtvs_type = (int32_t)vtvs;
        cfg.solve_type = (int32_t)solve;
        cfg.smem_col_cnt = smem_col_cnt_;
        cfg.m_batches = m_batches_;
        cfg.n_batches = n_batches_;
        return cfg;
    }
    double rmse(bool test) {
        double out = 0.0;
        als_gb300_detail::check(test ? als_rmse_test(h_, &out) : als_rmse_train(h_, &out), h_);
        return out;
    }
    als_handle *h_ = nullptr;
    std::vector<float> hu_, hv_;
    logger *logger_ = nullptr;
    int32_t iter_rmse_ = 0, cout_ = 1;
};
