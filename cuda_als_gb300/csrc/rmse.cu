// rmse.cu — squared error of a rating set against the factors, summed in FP64 in a fixed order.
//
// Replaces calculate_square_error + rsme_test/rsme_train (als_model.cu:62-89, 1722-1764): the
// reference adds FP32 squares into 1000 buckets with atomicAdd (non-deterministic order) and
// sums them with cublasSasum.  Here each thread accumulates its ratings in FP64, CTAs reduce in
// a fixed tree, and one CTA adds the CTA partials in index order, so the result is bit-for-bit
// repeatable.  The dot product keeps the reference's NaN rule: it stops at the first factor
// component that is NaN (als_model.cu:78-79).  HBM/L2-bound: 12 B per rating plus two gathered
// factor rows.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdint.h>

#include "internal.h"

namespace als {

namespace {

constexpr int RMSE_THREADS = 256;
constexpr int RMSE_BLOCKS = 152 * 8;  // fixed grid: the summation order never depends on size

__device__ double block_sum_d(double v, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < RMSE_THREADS / 32; ++w) s += sh[w];
    return s;  // valid in thread 0
}

__global__ void __launch_bounds__(RMSE_THREADS)
sq_error_partials_kernel(int64_t nnz, const int32_t *__restrict__ rows,
                         const int32_t *__restrict__ cols, const float *__restrict__ vals,
                         const float *__restrict__ U, const float *__restrict__ V, int f,
                         double *__restrict__ partials) {
    __shared__ double sh[RMSE_THREADS / 32];
    double acc = 0.0;
    for (int64_t e = (int64_t)blockIdx.x * RMSE_THREADS + threadIdx.x; e < nnz;
         e += (int64_t)RMSE_BLOCKS * RMSE_THREADS) {
        const float *u = U + (int64_t)rows[e] * f;
        const float *v = V + (int64_t)cols[e] * f;
        double pred = 0.0;
        for (int i = 0; i < f; ++i) {
            const float a = __ldg(u + i), b = __ldg(v + i);
            if (a != a || b != b) break;
            pred = fma((double)a, (double)b, pred);
        }
        const double err = (double)vals[e] - pred;
        acc = fma(err, err, acc);
    }
    double s = block_sum_d(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(RMSE_THREADS)
sum_partials_kernel(const double *__restrict__ partials, int n, double *__restrict__ out) {
    __shared__ double sh[RMSE_THREADS / 32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += RMSE_THREADS) acc += partials[i];
    double s = block_sum_d(acc, sh);
    if (threadIdx.x == 0) *out = s;
}

}  // namespace

size_t rmse_scratch_bytes() { return sizeof(double) * (RMSE_BLOCKS + 32); }

cudaError_t launch_sq_error(int64_t nnz, const int32_t *rows, const int32_t *cols,
                            const float *vals, const float *U, const float *V, int f,
                            double *d_partials, double *d_out, cudaStream_t st) {
    sq_error_partials_kernel<<<RMSE_BLOCKS, RMSE_THREADS, 0, st>>>(nnz, rows, cols, vals, U, V,
                                                                   f, d_partials);
    sum_partials_kernel<<<1, RMSE_THREADS, 0, st>>>(d_partials, RMSE_BLOCKS, d_out);
    return cudaGetLastError();
}

// Relative difference of two factor tables over the rows order[lo..hi): sum (a - b)^2 and
// sum a^2 in FP64 (the autotuner's agreement check between two solvers).
static __global__ void bucket_diff_kernel(const int32_t *__restrict__ order, int32_t lo, int32_t hi,
                                   const float *__restrict__ A, const float *__restrict__ Bm, int f,
                                   double *__restrict__ out) {
    __shared__ double sd[32], sa[32];
    double d2 = 0.0, a2 = 0.0;
    const int64_t total = (int64_t)(hi - lo) * f;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = order[lo + e / f];
        const int j = (int)(e % f);
        const double a = A[r * f + j], b = Bm[r * f + j];
        d2 += (a - b) * (a - b);
        a2 += a * a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sd[threadIdx.x >> 5] = d2;
        sa[threadIdx.x >> 5] = a2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double td = 0.0, ta = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            td += sd[w];
            ta += sa[w];
        }
        atomicAdd(&out[0], td);
        atomicAdd(&out[1], ta);
    }
}

cudaError_t launch_bucket_diff(const int32_t *order, int32_t lo, int32_t hi, const float *A,
                               const float *B, int f, double *out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
    if (e != cudaSuccess || hi <= lo) return e;
    const int64_t total = (int64_t)(hi - lo) * f;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, 1216);
    bucket_diff_kernel<<<grid, 256, 0, st>>>(order, lo, hi, A, B, f, out);
    return cudaGetLastError();
}

}  // namespace als
