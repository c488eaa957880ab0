// adjoint.cu — reverse mode of the user half-sweep (no counterpart in the reference).
//
// Forward: x_u = A_u^-1 b_u with A_u = Y_u^T Y_u + lambda n_u I, b_u = Y_u^T r_u (the U block of
// als_model::train, als_model.cu:1797-2029).  Loss on held-out ratings H:
//   L = sum_{(u,i,r) in H} (r - x_u . y_i)^2,  dL/dx_u = h_u = -2 sum_{(u,i) in H} (r - x_u.y_i) y_i.
// Reverse: g_u = A_u^-1 h_u, solved with the same L D L^T factor as the forward solve; then
//   dL/dy_i += r_ui g_u - (y_i . x_u) g_u - (g_u . y_i) x_u     for every training rating (u, i)
//   dL/dy_i += -2 (r - x_u . y_i) x_u                          for every held-out rating (u, i)
//   dL/dlambda = -sum_u n_u g_u . x_u                          (FP64, fixed-order reduction)
// One CTA per user row: the FP32 Gram of [Y | r] in registers (as in sweep_fp32.cu), the factor
// in shared memory, the held-out terms, the second solve, and an atomic scatter of the row's
// contributions into dL/dY (FP32).  The held-out loss itself is summed in FP64 per CTA.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <vector>

#include "handle.h"
#include "internal.h"
#include "solvers.cuh"
#include "tc.h"

namespace als {
namespace {

constexpr int KC = 32;
constexpr int MAX_FP = 232;

__host__ __device__ inline int fp_of(int f) { return ((f + 1 + 7) / 8) * 8; }
__host__ __device__ inline int nt_of(int fp) {
    int nb = fp / 8;
    int t = nb * (nb + 1);
    t = (t + 31) / 32 * 32;
    return t < 64 ? 64 : t;
}
__host__ __device__ inline size_t zsize_of(int fp) {
    size_t z = (size_t)KC * fp, g = (size_t)fp * (fp + 1);
    return z > g ? z : g;
}
inline size_t smem_of(int fp) {
    return sizeof(float) * (zsize_of(fp) + 2 * KC + 5 * (size_t)fp + 64);
}

struct AdjArgs {
    const int32_t *ptr, *idx;  // training CSR of the user side
    const float *val;
    const int32_t *hptr, *hidx;  // held-out ratings grouped by user (CSR)
    const float *hval;
    const float *Y;   // item factors (FP32, row-contiguous)
    float *X;         // user factors out
    float *dY;        // n x f, accumulated atomically (zeroed by the caller)
    double *loss_part, *dlam_part;  // one per CTA
    int32_t *flags;
    int f;
    float lambda;
};

__device__ double block_sum_d(double v, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nwarps; ++w) s += sh[w];
    __syncthreads();
    return s;  // valid in thread 0
}

__global__ void __launch_bounds__(1024) adjoint_user_kernel(const AdjArgs a, const int FP) {
    extern __shared__ __align__(16) float smem[];
    __shared__ double dsh[33];
    const int f = a.f, NB = FP / 8, GS = FP + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int nt = blockDim.x;
    float *Z = smem;
    int32_t *scol = (int32_t *)(smem + zsize_of(FP));
    float *sval = (float *)(scol + KC);
    float *vb = sval + KC, *vx = vb + FP, *vh = vx + FP, *vt = vh + FP, *vq = vt + FP;
    float *red = vq + FP;

    const int row = blockIdx.x;
    const int beg = a.ptr[row], end = a.ptr[row + 1], nu = end - beg;
    const int hbeg = a.hptr[row], hend = a.hptr[row + 1];
    float *xo = a.X + (int64_t)row * f;
    double loss = 0.0, dlam = 0.0;

    if (nu == 0) {  // x = 0; held-out residuals are r itself, no gradient through x
        for (int i = tid; i < f; i += nt) xo[i] = 0.f;
        for (int e = hbeg + tid; e < hend; e += nt) loss += (double)a.hval[e] * a.hval[e];
        const double s = block_sum_d(loss, dsh);
        if (tid == 0) {
            a.loss_part[blockIdx.x] = s;
            a.dlam_part[blockIdx.x] = 0.0;
        }
        return;
    }

    // ---- forward: Gram of [Y | r] (lower block triangle, 4 x 8 register tiles)
    const bool active = tid < NB * (NB + 1);
    const int q = tid >> 1;
    int bi = (int)((sqrtf(8.f * q + 1.f) - 1.f) * 0.5f);
    while ((bi + 1) * (bi + 2) / 2 <= q) ++bi;
    while (bi * (bi + 1) / 2 > q) --bi;
    const int bj = q - bi * (bi + 1) / 2;
    const int r0 = 8 * bi + 4 * (tid & 1), c0 = 8 * bj;
    float acc[4][8];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[p][c] = 0.f;
    for (int base = beg; base < end; base += KC) {
        const int cnt = min(KC, end - base);
        if (tid < KC) {
            scol[tid] = tid < cnt ? a.idx[base + tid] : -1;
            sval[tid] = tid < cnt ? a.val[base + tid] : 0.f;
        }
        __syncthreads();
        for (int k = warp; k < KC; k += nwarps) {
            const int c = scol[k];
            const float rv = sval[k];
            const float *y = a.Y + (int64_t)(c < 0 ? 0 : c) * f;
            for (int j = lane; j < FP; j += 32) {
                float v = 0.f;
                if (c >= 0) v = j < f ? __ldg(y + j) : (j == f ? rv : 0.f);
                Z[k * FP + j] = v;
            }
        }
        __syncthreads();
        if (active) {
            for (int k = 0; k < cnt; ++k) {
                const float4 av = *reinterpret_cast<const float4 *>(&Z[k * FP + r0]);
                const float4 cv0 = *reinterpret_cast<const float4 *>(&Z[k * FP + c0]);
                const float4 cv1 = *reinterpret_cast<const float4 *>(&Z[k * FP + c0 + 4]);
                const float ar[4] = {av.x, av.y, av.z, av.w};
                const float cr[8] = {cv0.x, cv0.y, cv0.z, cv0.w, cv1.x, cv1.y, cv1.z, cv1.w};
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[p][c] = fmaf(ar[p], cr[c], acc[p][c]);
            }
        }
        __syncthreads();
    }
    float *G = Z;
    if (active) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int c = 0; c < 8; ++c) G[(r0 + p) * GS + c0 + c] = acc[p][c];
    }
    __syncthreads();
    const float reg = (float)nu * a.lambda;
    for (int i = tid; i < f; i += nt) {
        G[i * GS + i] += reg;
        vb[i] = G[f * GS + i];
    }
    __syncthreads();
    bool ok = ldlt_factor<CtaSync>(G, GS, f, tid, nt);
    if (ok) ldlt_solve<CtaSync>(G, GS, f, vb, tid);  // vb <- x
    __syncthreads();
    float badf = 0.f;
    for (int i = tid; i < f; i += nt) badf += (ok && isfinite(vb[i])) ? 0.f : 1.f;
    badf = group_sum<CtaSync>(badf, red, tid, nt);
    if (badf > 0.f) {  // non-positive pivot: x = 0, flagged, no gradient through this row
        for (int i = tid; i < f; i += nt) {
            xo[i] = 0.f;
            vx[i] = 0.f;
        }
        if (tid == 0) atomicAdd(&a.flags[0], 1);
        for (int e = hbeg + tid; e < hend; e += nt) loss += (double)a.hval[e] * a.hval[e];
        const double s = block_sum_d(loss, dsh);
        if (tid == 0) {
            a.loss_part[blockIdx.x] = s;
            a.dlam_part[blockIdx.x] = 0.0;
        }
        return;
    }
    for (int i = tid; i < f; i += nt) {
        vx[i] = vb[i];
        xo[i] = vb[i];
        vh[i] = 0.f;
    }
    __syncthreads();

    // ---- held-out terms: loss, h = dL/dx, and the direct dL/dy_i = -2 res x_u.  The row's
    // held-out ratings are few; warp 0 walks them in order, so h and the loss are deterministic.
    if (warp == 0) {
        for (int e = hbeg; e < hend; ++e) {
            const int c = a.hidx[e];
            const float *y = a.Y + (int64_t)c * f;
            float d = 0.f;
            for (int j = lane; j < f; j += 32) d = fmaf(vx[j], __ldg(y + j), d);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            const float res = a.hval[e] - d;
            if (lane == 0) loss += (double)res * res;
            float *gy = a.dY + (int64_t)c * f;
            for (int j = lane; j < f; j += 32) {
                vh[j] += -2.f * res * __ldg(y + j);
                atomicAdd(&gy[j], -2.f * res * vx[j]);
            }
            __syncwarp();
        }
    }
    __syncthreads();

    // ---- g = A^-1 h with the same factor (vh <- g)
    ldlt_solve<CtaSync>(G, GS, f, vh, tid);
    {
        float gx = 0.f;
        for (int i = tid; i < f; i += nt) gx += vh[i] * vx[i];
        gx = group_sum<CtaSync>(gx, red, tid, nt);
        dlam = -(double)nu * (double)gx;
    }

    // ---- dL/dy_i += r g - (y.x) g - (g.y) x over the row's training ratings
    for (int e = beg + warp; e < end; e += nwarps) {
        const int c = a.idx[e];
        const float r = a.val[e];
        const float *y = a.Y + (int64_t)c * f;
        float yx = 0.f, gy = 0.f;
        for (int j = lane; j < f; j += 32) {
            const float yj = __ldg(y + j);
            yx = fmaf(yj, vx[j], yx);
            gy = fmaf(yj, vh[j], gy);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            yx += __shfl_xor_sync(0xffffffffu, yx, o);
            gy += __shfl_xor_sync(0xffffffffu, gy, o);
        }
        float *out = a.dY + (int64_t)c * f;
        for (int j = lane; j < f; j += 32)
            atomicAdd(&out[j], (r - yx) * vh[j] - gy * vx[j]);
    }
    const double sl = block_sum_d(loss, dsh);
    if (tid == 0) {
        a.loss_part[blockIdx.x] = sl;
        a.dlam_part[blockIdx.x] = dlam;
    }
}

__global__ void sum_doubles_kernel(const double *__restrict__ v, int64_t n, double *out) {
    __shared__ double sh[33];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += v[i];
    const double s = block_sum_d(acc, sh);
    if (threadIdx.x == 0) *out = s;
}

}  // namespace
}  // namespace als

using namespace als;

als_status run_adjoint(als_handle *h, const als_coo_view *held, double *loss, float *dLdY,
                       double *dLdlambda) {
    if (held->rows != h->m || held->cols != h->n || held->nnz < 0 || held->nnz > INT32_MAX ||
        (held->nnz > 0 && (!held->row_idxs || !held->col_idxs || !held->vals)))
        return set_global_error(ALS_ERR_INVALID_ARG, "held-out COO shape differs from the model");
    const int f = h->f;
    const int FP = fp_of(f);
    if (FP > MAX_FP) return set_global_error(ALS_ERR_UNSUPPORTED, "adjoint supports f <= 231");
    cudaSetDevice(h->cfg.device);
    // group the held-out ratings by user on the host (counting sort, stable)
    const int64_t m = h->m, n = h->n, nh = held->nnz;
    std::vector<int32_t> hptr((size_t)m + 1, 0), hidx((size_t)(nh > 0 ? nh : 1));
    std::vector<float> hval((size_t)(nh > 0 ? nh : 1));
    for (int64_t e = 0; e < nh; ++e) {
        const int32_t r = held->row_idxs[e], c = held->col_idxs[e];
        if (r < 0 || r >= m || c < 0 || c >= n || !std::isfinite(held->vals[e]))
            return set_global_error(ALS_ERR_INVALID_ARG, "held-out entry out of range at " +
                                                             std::to_string(e));
        hptr[r + 1]++;
    }
    for (int64_t r = 0; r < m; ++r) hptr[r + 1] += hptr[r];
    {
        std::vector<int32_t> cur(hptr.begin(), hptr.end() - 1);
        for (int64_t e = 0; e < nh; ++e) {
            const int32_t p = cur[held->row_idxs[e]]++;
            hidx[p] = held->col_idxs[e];
            hval[p] = held->vals[e];
        }
    }
    cudaStream_t st = h->stream;
    int32_t *d_hptr = nullptr, *d_hidx = nullptr;
    float *d_hval = nullptr, *d_dY = nullptr;
    double *d_parts = nullptr;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    step(cudaMalloc(&d_hptr, sizeof(int32_t) * (m + 1)));
    step(cudaMalloc(&d_hidx, sizeof(int32_t) * hidx.size()));
    step(cudaMalloc(&d_hval, sizeof(float) * hval.size()));
    step(cudaMalloc(&d_dY, sizeof(float) * (size_t)(n * f)));
    step(cudaMalloc(&d_parts, sizeof(double) * (size_t)(2 * m + 2)));
    if (e == cudaSuccess) {
        step(cudaMemcpyAsync(d_hptr, hptr.data(), sizeof(int32_t) * (m + 1), cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hidx, hidx.data(), sizeof(int32_t) * hidx.size(), cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hval, hval.data(), sizeof(float) * hval.size(), cudaMemcpyHostToDevice, st));
        step(cudaMemsetAsync(d_dY, 0, sizeof(float) * (size_t)(n * f), st));
        step(cudaMemsetAsync(h->d_flags, 0, sizeof(int32_t) * 4, st));
        AdjArgs a{};
        a.ptr = h->d_csr_ptr;
        a.idx = h->d_csr_idx;
        a.val = h->d_csr_val;
        a.hptr = d_hptr;
        a.hidx = d_hidx;
        a.hval = d_hval;
        a.Y = h->d_V;
        a.X = h->d_U;
        a.dY = d_dY;
        a.loss_part = d_parts;
        a.dlam_part = d_parts + m;
        a.flags = h->d_flags;
        a.f = f;
        a.lambda = h->cfg.lambda;
        const size_t smem = smem_of(FP);
        if (smem > 48 * 1024)
            step(cudaFuncSetAttribute(adjoint_user_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        if (e == cudaSuccess) adjoint_user_kernel<<<(unsigned)m, nt_of(FP), smem, st>>>(a, FP);
        step(cudaGetLastError());
        sum_doubles_kernel<<<1, 256, 0, st>>>(d_parts, m, d_parts + 2 * m);
        sum_doubles_kernel<<<1, 256, 0, st>>>(d_parts + m, m, d_parts + 2 * m + 1);
        double out[2] = {0.0, 0.0};
        step(cudaMemcpyAsync(out, d_parts + 2 * m, sizeof(out), cudaMemcpyDeviceToHost, st));
        if (dLdY) step(cudaMemcpyAsync(dLdY, d_dY, sizeof(float) * (size_t)(n * f), cudaMemcpyDeviceToHost, st));
        step(cudaStreamSynchronize(st));
        if (loss) *loss = out[0];
        if (dLdlambda) *dLdlambda = out[1];
    }
    void *all[] = {d_hptr, d_hidx, d_hval, d_dY, d_parts};
    for (void *p : all)
        if (p) cudaFree(p);
    if (e != cudaSuccess) {
        h->last_error = std::string("adjoint: ") + cudaGetErrorString(e);
        return set_global_error(e == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA,
                                h->last_error);
    }
    return ALS_OK;
}
