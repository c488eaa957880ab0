// coo_build.cu — rating triples -> CSR (+ the row of every CSR entry) and CSC, on the GPU.
//
// The reference builds its input files offline with scipy: the raw (user, item, rating) triples
// of a split become coo_matrix((r, (u - 1, i - 1))), then .tocsr().tocoo() (entries in row-major
// order, duplicates summed), .tocsr() and .tocsc() (data/toy_data/prepare_toy_data.py:108-110,
// 147-150, 201-208; data/netflix/prepare_netflix_data.py:88-109), written as float32
// (.astype(np.float32)).  This is that step on the device:
//
//   1. stable LSD radix sort of the entries by column, then by row, carrying input positions:
//      entries end in (row, column) order, duplicates of a cell in input order;
//   2. head flags (a cell's first entry) and their exclusive scan: each cell's output slot and
//      the count after summing duplicates;
//   3. each head sums its cell's values in FP64, in input order, and rounds once to FP32.  scipy
//      sums the float64 (or integer) ratings before the float32 cast; an FP64 sum of float32
//      values on a common grid (star ratings) is exact, hence independent of order, so the
//      result is bit-identical to scipy's whenever that sum is exact (scipy's own per-row sort
//      is not stable, so no fixed order would do better);
//   4. the row pointers from the sorted rows, and the CSC by the library's stable transpose
//      (rows ascending within a column: scipy's tocsc order).
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "internal.h"

namespace als {

namespace {

inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }
inline int grid_of(int64_t work, int threads) {
    const int64_t g = (work + threads - 1) / threads;
    return (int)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

__global__ void coo_bad_kernel(int64_t nnz, const int32_t *__restrict__ r,
                               const int32_t *__restrict__ c, int32_t rows, int32_t cols,
                               int32_t *bad) {
    int local = 0;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x)
        if (r[p] < 0 || r[p] >= rows || c[p] < 0 || c[p] >= cols) ++local;
    local = __reduce_add_sync(0xffffffffu, local);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(bad, local);
}

// dst[p] = src[perm[p]]
__global__ void gather_i32_kernel(int64_t n, const int32_t *__restrict__ perm,
                                  const int32_t *__restrict__ src, int32_t *__restrict__ dst) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x)
        dst[p] = src[perm[p]];
}

// pos[p] = perm1[perm2[p]] (input position of sorted entry p); col_s[p] = col[pos[p]];
// head[p] = 1 where (row, col) differs from entry p - 1
__global__ void heads_kernel(int64_t n, const int32_t *__restrict__ perm1,
                             const int32_t *__restrict__ perm2, const int32_t *__restrict__ col,
                             const int32_t *__restrict__ row_s, int32_t *__restrict__ pos,
                             int32_t *__restrict__ col_s, int32_t *__restrict__ head) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t q = perm1[perm2[p]];
        const int32_t c = col[q];
        pos[p] = q;
        col_s[p] = c;
        int h = 1;
        if (p > 0) {
            const int32_t cp = col[perm1[perm2[p - 1]]];
            h = (row_s[p] != row_s[p - 1] || c != cp) ? 1 : 0;
        }
        head[p] = h;
    }
}

// Each cell's head writes the cell: its row, column and the FP64 sum of its values in input
// order, rounded once to FP32.
__global__ void emit_kernel(int64_t n, const int32_t *__restrict__ head,
                            const int32_t *__restrict__ slot, const int32_t *__restrict__ row_s,
                            const int32_t *__restrict__ col_s, const int32_t *__restrict__ pos,
                            const float *__restrict__ val, int32_t *__restrict__ out_row,
                            int32_t *__restrict__ out_col, float *__restrict__ out_val) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        if (!head[p]) continue;
        double s = (double)val[pos[p]];
        for (int64_t q = p + 1; q < n && !head[q]; ++q) s += (double)val[pos[q]];
        const int32_t k = slot[p];
        out_row[k] = row_s[p];
        out_col[k] = col_s[p];
        out_val[k] = (float)s;
    }
}

}  // namespace

size_t coo_build_scratch_bytes(int64_t rows, int64_t cols, int64_t nnz) {
    const size_t arr = a256(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    const size_t sort = radix_sort_scratch_bytes(nnz);
    const size_t scan = scan_scratch_bytes(nnz + 1);
    const size_t tr = transpose_scratch_bytes(rows, cols, nnz);
    // perm1, row gathered, sorted rows, perm2, positions, sorted columns, heads, slots (n + 1),
    // the output rows when the caller wants none, then the sort / scan / transpose scratch
    // (used one after another)
    const size_t tail = sort > scan ? (sort > tr ? sort : tr) : (scan > tr ? scan : tr);
    return 9 * arr + a256(sizeof(int32_t)) + a256(sizeof(int32_t)) + tail;
}

// Device core.  `*nnz_out` (host) receives the cell count; the stream is synchronised to read the
// validation count and the cell count (every later launch depends on them).  *bad_out receives
// the number of triples with an index outside [0, rows) x [0, cols); then nothing is built.
cudaError_t coo_to_csr_device(int64_t rows, int64_t cols, int64_t nnz, const int32_t *ridx,
                              const int32_t *cidx, const float *val, int32_t *row_ptrs,
                              int32_t *col_idxs, float *vals, int32_t *coo_rows,
                              int32_t *col_ptrs, int32_t *csc_rows, float *csc_vals,
                              void *scratch, cudaStream_t st, int64_t *nnz_out, int *bad_out) {
    *nnz_out = 0;
    *bad_out = 0;
    if (nnz <= 0) {
        cudaError_t e = cudaMemsetAsync(row_ptrs, 0, sizeof(int32_t) * (size_t)(rows + 1), st);
        if (e == cudaSuccess && col_ptrs)
            e = cudaMemsetAsync(col_ptrs, 0, sizeof(int32_t) * (size_t)(cols + 1), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e;
    }
    const size_t arr = a256(sizeof(int32_t) * (size_t)nnz);
    char *s = (char *)scratch;
    int32_t *perm1 = (int32_t *)s; s += arr;
    int32_t *rows1 = (int32_t *)s; s += arr;
    int32_t *row_s = (int32_t *)s; s += arr;
    int32_t *perm2 = (int32_t *)s; s += arr;
    int32_t *pos = (int32_t *)s; s += arr;
    int32_t *col_s = (int32_t *)s; s += arr;
    int32_t *head = (int32_t *)s; s += arr;
    int32_t *slot = (int32_t *)s; s += a256(sizeof(int32_t) * (size_t)(nnz + 1));
    int32_t *own_rows = (int32_t *)s; s += arr;
    int32_t *d_bad = (int32_t *)s; s += a256(sizeof(int32_t));
    void *tail = s;
    int32_t *out_rows = coo_rows ? coo_rows : own_rows;

    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    coo_bad_kernel<<<grid_of(nnz, 256), 256, 0, st>>>(nnz, ridx, cidx, (int32_t)rows,
                                                      (int32_t)cols, d_bad);
    int32_t bad = 0;
    e = cudaMemcpyAsync(&bad, d_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (bad) {
        *bad_out = bad;
        return cudaSuccess;
    }
    // 1. by column (positions carried), then stably by row
    e = radix_sort_pairs(cidx, nullptr, col_s, perm1, nnz, (int32_t)(cols > 0 ? cols - 1 : 0),
                         tail, st);
    if (e != cudaSuccess) return e;
    gather_i32_kernel<<<grid_of(nnz, 256), 256, 0, st>>>(nnz, perm1, ridx, rows1);
    e = radix_sort_pairs(rows1, nullptr, row_s, perm2, nnz, (int32_t)(rows > 0 ? rows - 1 : 0),
                         tail, st);
    if (e != cudaSuccess) return e;
    // 2. cells and their slots
    heads_kernel<<<grid_of(nnz, 256), 256, 0, st>>>(nnz, perm1, perm2, cidx, row_s, pos, col_s,
                                                    head);
    e = exclusive_scan_i32(head, slot, nnz, true, tail, st);
    if (e != cudaSuccess) return e;
    int32_t cells = 0;
    e = cudaMemcpyAsync(&cells, slot + nnz, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    // 3. one entry per cell, duplicates summed
    emit_kernel<<<grid_of(nnz, 256), 256, 0, st>>>(nnz, head, slot, row_s, col_s, pos, val,
                                                   out_rows, col_idxs, vals);
    // 4. row pointers, then the CSC
    e = ptrs_from_sorted(cells, rows, out_rows, row_ptrs, st);
    if (e != cudaSuccess) return e;
    if (col_ptrs)
        e = csr_to_csc_device(rows, cols, cells, row_ptrs, col_idxs, vals, col_ptrs, csc_rows,
                              csc_vals, tail, st, nullptr, nullptr);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    *nnz_out = cells;
    return e;
}

}  // namespace als

using namespace als;

static als_status coo_args(const als_coo_view *coo, const int32_t *row_ptrs,
                           const int32_t *col_idxs, const float *vals, const int32_t *col_ptrs,
                           const int32_t *csc_rows, const float *csc_vals,
                           const int64_t *nnz_out) {
    if (!coo || !row_ptrs || !nnz_out)
        return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    if (coo->nnz > 0 && (!coo->row_idxs || !coo->col_idxs || !coo->vals || !col_idxs || !vals))
        return set_global_error(ALS_ERR_INVALID_ARG, "null array");
    if (!!col_ptrs != !!csc_rows || !!col_ptrs != !!csc_vals)
        return set_global_error(ALS_ERR_INVALID_ARG,
                                "col_ptrs, row_idxs and csc_vals: all three or none");
    if (coo->rows < 0 || coo->cols < 0 || coo->nnz < 0 || coo->nnz > INT32_MAX ||
        coo->rows >= INT32_MAX || coo->cols >= INT32_MAX)
        return set_global_error(ALS_ERR_INVALID_ARG, "shape out of range");
    return ALS_OK;
}

static als_status cuda_fail(const char *what, cudaError_t e) {
    return set_global_error(e == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA,
                            std::string(what) + ": " + cudaGetErrorString(e));
}

static als_status bad_index(int bad) {
    return set_global_error(ALS_ERR_INVALID_ARG,
                            std::to_string(bad) + " triples with a row or column index out of range");
}

extern "C" als_status als_coo_to_csr_device(const als_coo_view *coo, int32_t *row_ptrs,
                                            int32_t *col_idxs, float *vals, int32_t *coo_rows,
                                            int32_t *col_ptrs, int32_t *row_idxs,
                                            float *csc_vals, int64_t *nnz_out, void *stream) {
    als_status s = coo_args(coo, row_ptrs, col_idxs, vals, col_ptrs, row_idxs, csc_vals, nnz_out);
    if (s != ALS_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    void *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, coo_build_scratch_bytes(coo->rows, coo->cols,
                                                                      coo->nnz), st);
    if (e != cudaSuccess) return cuda_fail("cudaMallocAsync", e);
    int bad = 0;
    e = coo_to_csr_device(coo->rows, coo->cols, coo->nnz, coo->row_idxs, coo->col_idxs,
                          coo->vals, row_ptrs, col_idxs, vals, coo_rows, col_ptrs, row_idxs,
                          csc_vals, scratch, st, nnz_out, &bad);
    cudaFreeAsync(scratch, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail("coo_to_csr", e);
    if (bad) return bad_index(bad);
    return ALS_OK;
}

extern "C" als_status als_coo_to_csr(const als_coo_view *coo, int32_t *row_ptrs,
                                     int32_t *col_idxs, float *vals, int32_t *coo_rows,
                                     int32_t *col_ptrs, int32_t *row_idxs, float *csc_vals,
                                     int64_t *nnz_out) {
    als_status s = coo_args(coo, row_ptrs, col_idxs, vals, col_ptrs, row_idxs, csc_vals, nnz_out);
    if (s != ALS_OK) return s;
    *nnz_out = 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_global_error(ALS_ERR_NO_DEVICE, "no CUDA device");
    const int64_t rows = coo->rows, cols = coo->cols, nnz = coo->nnz;
    const size_t n4 = sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1);
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail("cudaStreamCreate", e);
    char *buf = nullptr;
    // inputs (3 nnz), CSR (rows + 1, 2 nnz), COO rows (nnz), CSC (cols + 1, 2 nnz), scratch
    const size_t a_in = 3 * a256(n4), a_csr = a256(sizeof(int32_t) * (rows + 1)) + 2 * a256(n4);
    const size_t a_rows = a256(n4), a_csc = a256(sizeof(int32_t) * (cols + 1)) + 2 * a256(n4);
    const size_t a_scr = coo_build_scratch_bytes(rows, cols, nnz);
    e = cudaMalloc(&buf, a_in + a_csr + a_rows + a_csc + a_scr);
    if (e != cudaSuccess) {
        cudaStreamDestroy(st);
        return cuda_fail("cudaMalloc", e);
    }
    char *q = buf;
    int32_t *d_r = (int32_t *)q; q += a256(n4);
    int32_t *d_c = (int32_t *)q; q += a256(n4);
    float *d_v = (float *)q; q += a256(n4);
    int32_t *d_ptr = (int32_t *)q; q += a256(sizeof(int32_t) * (rows + 1));
    int32_t *d_idx = (int32_t *)q; q += a256(n4);
    float *d_val = (float *)q; q += a256(n4);
    int32_t *d_rows = (int32_t *)q; q += a256(n4);
    int32_t *d_cptr = (int32_t *)q; q += a256(sizeof(int32_t) * (cols + 1));
    int32_t *d_ridx = (int32_t *)q; q += a256(n4);
    float *d_cval = (float *)q; q += a256(n4);
    void *d_scr = q;
    auto step = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    if (nnz > 0) {
        step(cudaMemcpyAsync(d_r, coo->row_idxs, n4, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_c, coo->col_idxs, n4, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_v, coo->vals, n4, cudaMemcpyHostToDevice, st));
    }
    int bad = 0;
    if (e == cudaSuccess)
        e = coo_to_csr_device(rows, cols, nnz, d_r, d_c, d_v, d_ptr, d_idx, d_val,
                              coo_rows ? d_rows : nullptr, col_ptrs ? d_cptr : nullptr,
                              col_ptrs ? d_ridx : nullptr, col_ptrs ? d_cval : nullptr, d_scr, st,
                              nnz_out, &bad);
    const size_t k4 = sizeof(int32_t) * (size_t)*nnz_out;
    if (e == cudaSuccess && !bad) {
        step(cudaMemcpyAsync(row_ptrs, d_ptr, sizeof(int32_t) * (rows + 1), cudaMemcpyDeviceToHost, st));
        if (k4) {
            step(cudaMemcpyAsync(col_idxs, d_idx, k4, cudaMemcpyDeviceToHost, st));
            step(cudaMemcpyAsync(vals, d_val, k4, cudaMemcpyDeviceToHost, st));
            if (coo_rows) step(cudaMemcpyAsync(coo_rows, d_rows, k4, cudaMemcpyDeviceToHost, st));
        }
        if (col_ptrs) {
            step(cudaMemcpyAsync(col_ptrs, d_cptr, sizeof(int32_t) * (cols + 1), cudaMemcpyDeviceToHost, st));
            if (k4) {
                step(cudaMemcpyAsync(row_idxs, d_ridx, k4, cudaMemcpyDeviceToHost, st));
                step(cudaMemcpyAsync(csc_vals, d_cval, k4, cudaMemcpyDeviceToHost, st));
            }
        }
        step(cudaStreamSynchronize(st));
    }
    cudaStreamSynchronize(st);
    cudaFree(buf);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return cuda_fail("coo_to_csr", e);
    if (bad) return bad_index(bad);
    return ALS_OK;
}
