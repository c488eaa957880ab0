// adjoint.cu — reverse mode of the user half-sweep (no counterpart in the reference).
//
// Forward: x_u = A_u^-1 b_u with A_u = Y_u^T Y_u + lambda n_u I, b_u = Y_u^T r_u (the U block of
// als_model::train, als_model.cu:1797-2029).  Loss on held-out ratings H:
//   L = sum_{(u,i,r) in H} (r - x_u . y_i)^2,  dL/dx_u = h_u = -2 sum_{(u,i) in H} (r - x_u.y_i) y_i.
// Reverse: g_u = A_u^-1 h_u, solved with the same L D L^T factor as the forward solve; then
//   dL/dy_i = sum_{u in train(i)} [(r_ui - y_i . x_u) g_u - (g_u . y_i) x_u]
//           + sum_{u in H(i)} -2 (r_ui - x_u . y_i) x_u
//   dL/dlambda = -sum_u n_u g_u . x_u
// Two kernels, each in FP32 or FP64 (T):
//   adjoint_row_kernel: one CTA per user row — the Gram of [Y | r] in register tiles (as in
//     sweep_fp32.cu, the right-hand side summed apart with compensation), the L D L^T factor in
//     shared memory, the forward solve, the row's held-out terms (in order: h_u and the loss),
//     the second solve with the same factor; writes x_u and g_u, the loss and dL/dlambda parts.
//   adjoint_chunk_kernel + adjoint_combine_kernel: dL/dy_i from the item's training column (the
//     CSC) in chunks of 2,048 ratings (one CTA each: heavy items spread over many) and its
//     held-out ratings; every sum in a fixed order (warps, then chunks): deterministic, no
//     atomics.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
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
constexpr int MAX_FP = 232;      // FP32: the Gram of FP x (FP+1) floats in shared memory
constexpr int MAX_F_F64 = 128;   // FP64: the Gram of 136 x 137 doubles (149 KB)
constexpr int ITEM_WARPS = 8;
constexpr int ITEM_Q = (MAX_FP + 31) / 32;  // feature slots per lane in the item kernel
constexpr int32_t ITEM_CHUNK = 2048;        // training ratings per chunk of an item's column

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
template <typename T>
inline size_t smem_of(int fp) {
    return sizeof(T) * (zsize_of(fp) + 2 * KC + 5 * (size_t)fp + 64);
}

template <typename T>
struct AdjArgs {
    const int32_t *ptr, *idx;  // training CSR of the user side
    const float *val;
    const int32_t *hptr, *hidx;  // held-out ratings grouped by user (CSR)
    const float *hval;
    const T *Y;        // item factors, row-contiguous
    T *X, *G;          // per user: x_u and g_u (m x f)
    float *Xout;       // the handle's U (FP32 copy of x_u)
    double *loss_part, *dlam_part;  // one per row
    int32_t *flags;
    int f;
    T lambda;
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

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return fmaf(a, b, c); }

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 512 : 1024)
    adjoint_row_kernel(const AdjArgs<T> a, const int FP) {
    extern __shared__ __align__(16) unsigned char smem_bytes[];
    T *smem = reinterpret_cast<T *>(smem_bytes);
    __shared__ double dsh[33];
    const int f = a.f, NB = FP / 8, GS = FP + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int nt = blockDim.x;
    T *Z = smem;
    int32_t *scol = (int32_t *)(smem + zsize_of(FP));
    T *sval = reinterpret_cast<T *>(scol) + KC;
    T *vb = sval + KC, *vx = vb + FP, *vh = vx + FP, *red = vh + 2 * FP;

    const int row = blockIdx.x;
    const int beg = a.ptr[row], end = a.ptr[row + 1], nu = end - beg;
    const int hbeg = a.hptr[row], hend = a.hptr[row + 1];
    T *xr = a.X + (int64_t)row * f;
    T *gr = a.G + (int64_t)row * f;
    float *xo = a.Xout + (int64_t)row * f;
    double loss = 0.0, dlam = 0.0;

    auto no_gradient = [&]() {  // x = 0: held-out residuals are r itself, no path through x
        for (int i = tid; i < f; i += nt) {
            xo[i] = 0.f;
            xr[i] = T(0);
            gr[i] = T(0);
        }
        for (int e = hbeg + tid; e < hend; e += nt) loss += (double)a.hval[e] * a.hval[e];
        const double s = block_sum_d(loss, dsh);
        if (tid == 0) {
            a.loss_part[row] = s;
            a.dlam_part[row] = 0.0;
        }
    };
    if (nu == 0) {
        no_gradient();
        return;
    }

    // ---- forward: Gram of Y_u (lower block triangle, 4 x 8 register tiles), b apart
    const bool active = tid < NB * (NB + 1);
    const int q = tid >> 1;
    int bi = (int)((sqrtf(8.f * q + 1.f) - 1.f) * 0.5f);
    while ((bi + 1) * (bi + 2) / 2 <= q) ++bi;
    while (bi * (bi + 1) / 2 > q) --bi;
    const int bj = q - bi * (bi + 1) / 2;
    const int r0 = 8 * bi + 4 * (tid & 1), c0 = 8 * bj;
    T acc[4][8];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[p][c] = T(0);
    T bsum = T(0), bcomp = T(0);  // b_tid: compensated sum of 32-rating chunk sums
    for (int base = beg; base < end; base += KC) {
        const int cnt = min(KC, end - base);
        if (tid < KC) {
            scol[tid] = tid < cnt ? a.idx[base + tid] : -1;
            sval[tid] = tid < cnt ? (T)a.val[base + tid] : T(0);
        }
        __syncthreads();
        for (int k = warp; k < KC; k += nwarps) {
            const int c = scol[k];
            const T *y = a.Y + (int64_t)(c < 0 ? 0 : c) * f;
            for (int j = lane; j < FP; j += 32) Z[k * FP + j] = (c >= 0 && j < f) ? y[j] : T(0);
        }
        __syncthreads();
        if (active) {
            for (int k = 0; k < cnt; ++k) {
                const T *zk = Z + k * FP;
                T ar[4], cr[8];  // 16-byte loads (r0 a multiple of 4, c0 of 8)
                if constexpr (sizeof(T) == 4) {
                    const float4 a4 = *reinterpret_cast<const float4 *>(zk + r0);
                    const float4 c4 = *reinterpret_cast<const float4 *>(zk + c0);
                    const float4 d4 = *reinterpret_cast<const float4 *>(zk + c0 + 4);
                    ar[0] = a4.x; ar[1] = a4.y; ar[2] = a4.z; ar[3] = a4.w;
                    cr[0] = c4.x; cr[1] = c4.y; cr[2] = c4.z; cr[3] = c4.w;
                    cr[4] = d4.x; cr[5] = d4.y; cr[6] = d4.z; cr[7] = d4.w;
                } else {
#pragma unroll
                    for (int p = 0; p < 4; p += 2) {
                        const double2 v = *reinterpret_cast<const double2 *>(zk + r0 + p);
                        ar[p] = v.x; ar[p + 1] = v.y;
                    }
#pragma unroll
                    for (int c = 0; c < 8; c += 2) {
                        const double2 v = *reinterpret_cast<const double2 *>(zk + c0 + c);
                        cr[c] = v.x; cr[c + 1] = v.y;
                    }
                }
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[p][c] = fma_t<T>(ar[p], cr[c], acc[p][c]);
            }
        }
        if (tid < f) {
            T cs = T(0);
            for (int k = 0; k < cnt; ++k) cs = fma_t<T>(sval[k], Z[k * FP + tid], cs);
            const T yk = cs - bcomp;
            const T t = bsum + yk;
            bcomp = (t - bsum) - yk;
            bsum = t;
        }
        __syncthreads();
    }
    T *Gm = Z;
    if (active) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int c = 0; c < 8; ++c) Gm[(r0 + p) * GS + c0 + c] = acc[p][c];
    }
    __syncthreads();
    const T reg = (T)nu * a.lambda;
    if (tid < f) {  // (the launch has at least f threads)
        Gm[tid * GS + tid] += reg;
        vb[tid] = bsum;
    }
    __syncthreads();
    bool ok = ldlt_factor<CtaSync>(Gm, GS, f, tid, nt);
    if (ok) ldlt_solve<CtaSync>(Gm, GS, f, vb, tid);  // vb <- x
    __syncthreads();
    T badf = T(0);
    for (int i = tid; i < f; i += nt) badf += (ok && isfinite(vb[i])) ? T(0) : T(1);
    badf = group_sum<CtaSync, T>(badf, red, tid, nt);
    if (badf > T(0)) {  // non-positive pivot: x = 0, flagged, no gradient through this row
        if (tid == 0) atomicAdd(&a.flags[0], 1);
        no_gradient();
        return;
    }
    for (int i = tid; i < f; i += nt) {
        vx[i] = vb[i];
        xr[i] = vb[i];
        xo[i] = (float)vb[i];
        vh[i] = T(0);
    }
    __syncthreads();

    // ---- held-out terms: loss and h = dL/dx.  The row's held-out ratings are few; warp 0 walks
    // them in order, so h and the loss are deterministic.
    if (warp == 0) {
        for (int e = hbeg; e < hend; ++e) {
            const T *y = a.Y + (int64_t)a.hidx[e] * f;
            T d = T(0);
            for (int j = lane; j < f; j += 32) d = fma_t<T>(vx[j], y[j], d);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            const T res = (T)a.hval[e] - d;
            if (lane == 0) loss += (double)res * (double)res;
            for (int j = lane; j < f; j += 32) vh[j] += T(-2) * res * y[j];
            __syncwarp();
        }
    }
    __syncthreads();

    // ---- g = A^-1 h with the same factor (vh <- g)
    ldlt_solve<CtaSync>(Gm, GS, f, vh, tid);
    {
        T gx = T(0);
        for (int i = tid; i < f; i += nt) gx += vh[i] * vx[i];
        gx = group_sum<CtaSync, T>(gx, red, tid, nt);
        dlam = -(double)nu * (double)gx;
    }
    for (int i = tid; i < f; i += nt) gr[i] = vh[i];
    const double sl = block_sum_d(loss, dsh);
    if (tid == 0) {
        a.loss_part[row] = sl;
        a.dlam_part[row] = dlam;
    }
}

// dL/dy_i, in fixed chunks: chunk c covers ratings [cbeg[c], cend[c]) of item citem[c]'s
// training column (the CSC: users and ratings) and, for the item's first chunk, its held-out
// ratings.  Warp w of the chunk's CTA takes entries w, w + ITEM_WARPS, ... in order; lane l
// holds features l, l + 32, ...; the warps' partial vectors are added in warp order into
// part[c].  Heavy items (hundreds of thousands of ratings) spread over many CTAs this way.
template <typename T>
__global__ void __launch_bounds__(32 * ITEM_WARPS)
    adjoint_chunk_kernel(int64_t nchunks, int f, const int32_t *__restrict__ citem,
                         const int32_t *__restrict__ cbeg, const int32_t *__restrict__ cend,
                         const int32_t *__restrict__ cusr, const float *__restrict__ cval,
                         const int32_t *__restrict__ hptr, const int32_t *__restrict__ husr,
                         const float *__restrict__ hval, const T *__restrict__ Y,
                         const T *__restrict__ X, const T *__restrict__ G, T *__restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_bytes[];
    T *wp = reinterpret_cast<T *>(smem_bytes);  // [ITEM_WARPS][f]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nq = (f + 31) / 32;
    for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int64_t it = citem[ch];
        const bool first = ch == 0 || citem[ch - 1] != it;
        T y[ITEM_Q], acc[ITEM_Q];
#pragma unroll
        for (int q = 0; q < ITEM_Q; ++q) {
            const int j = lane + 32 * q;
            y[q] = q < nq && j < f ? Y[it * f + j] : T(0);
            acc[q] = T(0);
        }
        auto dot = [&](const T *v) -> T {
            T s = T(0);
#pragma unroll
            for (int q = 0; q < ITEM_Q; ++q) {
                const int j = lane + 32 * q;
                if (q < nq && j < f) s = fma_t<T>(y[q], v[j], s);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            return s;
        };
        for (int e = cbeg[ch] + warp; e < cend[ch]; e += ITEM_WARPS) {
            const T *xu = X + (int64_t)cusr[e] * f;
            const T *gu = G + (int64_t)cusr[e] * f;
            const T yx = dot(xu), gy = dot(gu);
            const T c = (T)cval[e] - yx;
#pragma unroll
            for (int q = 0; q < ITEM_Q; ++q) {
                const int j = lane + 32 * q;
                if (q < nq && j < f) acc[q] = fma_t<T>(c, gu[j], fma_t<T>(-gy, xu[j], acc[q]));
            }
        }
        if (first) {
            for (int e = hptr[it] + warp; e < hptr[it + 1]; e += ITEM_WARPS) {
                const T *xu = X + (int64_t)husr[e] * f;
                const T res = (T)hval[e] - dot(xu);
#pragma unroll
                for (int q = 0; q < ITEM_Q; ++q) {
                    const int j = lane + 32 * q;
                    if (q < nq && j < f) acc[q] = fma_t<T>(T(-2) * res, xu[j], acc[q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < ITEM_Q; ++q) {
            const int j = lane + 32 * q;
            if (q < nq && j < f) wp[warp * f + j] = acc[q];
        }
        __syncthreads();
        for (int j = threadIdx.x; j < f; j += blockDim.x) {
            T s = wp[j];
            for (int w = 1; w < ITEM_WARPS; ++w) s += wp[w * f + j];
            part[ch * f + j] = s;
        }
        __syncthreads();
    }
}

// dY[i] = the item's chunk partials added in chunk order (first[i] .. first[i + 1]).
template <typename T>
__global__ void adjoint_combine_kernel(int64_t n, int f, const int32_t *__restrict__ first,
                                       const T *__restrict__ part, T *__restrict__ dY) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * f;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / f;
        const int j = (int)(e - i * f);
        T s = T(0);
        for (int32_t c = first[i]; c < first[i + 1]; ++c) s += part[(int64_t)c * f + j];
        dY[e] = s;
    }
}

__global__ void sum_doubles_kernel(const double *__restrict__ v, int64_t n, double *out) {
    __shared__ double sh[33];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += v[i];
    const double s = block_sum_d(acc, sh);
    if (threadIdx.x == 0) *out = s;
}

__global__ void f64_to_f32_kernel(const double *__restrict__ a, int64_t n, float *__restrict__ b) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// Counting sort of the held-out triples by `key` (rows or columns), stable: ptr (nkeys + 1),
// the other index and the value per entry.
void group_by(int64_t nkeys, int64_t nh, const int32_t *key, const int32_t *other,
              const float *vals, std::vector<int32_t> &ptr, std::vector<int32_t> &oth,
              std::vector<float> &val) {
    ptr.assign((size_t)nkeys + 1, 0);
    oth.assign((size_t)(nh > 0 ? nh : 1), 0);
    val.assign((size_t)(nh > 0 ? nh : 1), 0.f);
    for (int64_t e = 0; e < nh; ++e) ptr[key[e] + 1]++;
    for (int64_t r = 0; r < nkeys; ++r) ptr[r + 1] += ptr[r];
    std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
    for (int64_t e = 0; e < nh; ++e) {
        const int32_t p = cur[key[e]]++;
        oth[p] = other[e];
        val[p] = vals[e];
    }
}

// The adjoint in precision T.  Y: device item factors in T (n x f); dLdY: host, n x f of
// OutT (float for the FP32 entry point, double for the FP64 one).
template <typename T, typename OutT>
als_status adjoint_impl(als_handle *h, const als_coo_view *held, const T *d_Y, T lambda,
                        double *loss, OutT *dLdY, double *dLdlambda) {
    const int f = h->f;
    const int FP = fp_of(f);
    const int64_t m = h->m, n = h->n, nh = held->nnz;
    std::vector<int32_t> hptr_u, hcol_u, hptr_i, hrow_i;
    std::vector<float> hval_u, hval_i;
    group_by(m, nh, held->row_idxs, held->col_idxs, held->vals, hptr_u, hcol_u, hval_u);
    group_by(n, nh, held->col_idxs, held->row_idxs, held->vals, hptr_i, hrow_i, hval_i);
    // chunks of at most ITEM_CHUNK training ratings per item (one for an item without any)
    const std::vector<int32_t> &cp = h->host_ptr[1];
    std::vector<int32_t> citem, cbeg, cend, cfirst((size_t)n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        cfirst[i] = (int32_t)citem.size();
        const int32_t b = cp[i], e = cp[i + 1];
        int32_t s = b;
        do {
            citem.push_back((int32_t)i);
            cbeg.push_back(s);
            cend.push_back(std::min(e, s + ITEM_CHUNK));
            s += ITEM_CHUNK;
        } while (s < e);
    }
    cfirst[n] = (int32_t)citem.size();
    const int64_t nchunks = (int64_t)citem.size();
    cudaStream_t st = h->stream;
    int32_t *d_hptr_u = nullptr, *d_hcol_u = nullptr, *d_hptr_i = nullptr, *d_hrow_i = nullptr;
    float *d_hval_u = nullptr, *d_hval_i = nullptr;
    T *d_X = nullptr, *d_G = nullptr, *d_dY = nullptr, *d_part = nullptr;
    int32_t *d_chunks = nullptr;  // citem, cbeg, cend (nchunks each), cfirst (n + 1)
    double *d_parts = nullptr;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    const size_t nhp = hcol_u.size();
    step(cudaMalloc(&d_hptr_u, sizeof(int32_t) * (m + 1)));
    step(cudaMalloc(&d_hcol_u, sizeof(int32_t) * nhp));
    step(cudaMalloc(&d_hval_u, sizeof(float) * nhp));
    step(cudaMalloc(&d_hptr_i, sizeof(int32_t) * (n + 1)));
    step(cudaMalloc(&d_hrow_i, sizeof(int32_t) * nhp));
    step(cudaMalloc(&d_hval_i, sizeof(float) * nhp));
    step(cudaMalloc(&d_X, sizeof(T) * (size_t)(m * f)));
    step(cudaMalloc(&d_G, sizeof(T) * (size_t)(m * f)));
    step(cudaMalloc(&d_dY, sizeof(T) * (size_t)(n * f)));
    step(cudaMalloc(&d_parts, sizeof(double) * (size_t)(2 * m + 2)));
    step(cudaMalloc(&d_chunks, sizeof(int32_t) * (size_t)(3 * nchunks + n + 1)));
    step(cudaMalloc(&d_part, sizeof(T) * (size_t)(nchunks * f + 1)));
    if (e == cudaSuccess) {
        step(cudaMemcpyAsync(d_hptr_u, hptr_u.data(), sizeof(int32_t) * (m + 1), cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hcol_u, hcol_u.data(), sizeof(int32_t) * nhp, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hval_u, hval_u.data(), sizeof(float) * nhp, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hptr_i, hptr_i.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hrow_i, hrow_i.data(), sizeof(int32_t) * nhp, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_hval_i, hval_i.data(), sizeof(float) * nhp, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_chunks, citem.data(), sizeof(int32_t) * nchunks, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_chunks + nchunks, cbeg.data(), sizeof(int32_t) * nchunks, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_chunks + 2 * nchunks, cend.data(), sizeof(int32_t) * nchunks, cudaMemcpyHostToDevice, st));
        step(cudaMemcpyAsync(d_chunks + 3 * nchunks, cfirst.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, st));
        step(cudaMemsetAsync(h->d_flags, 0, sizeof(int32_t) * 4, st));
        AdjArgs<T> a{};
        a.ptr = h->d_csr_ptr;
        a.idx = h->d_csr_idx;
        a.val = h->d_csr_val;
        a.hptr = d_hptr_u;
        a.hidx = d_hcol_u;
        a.hval = d_hval_u;
        a.Y = d_Y;
        a.X = d_X;
        a.G = d_G;
        a.Xout = h->d_U;
        a.loss_part = d_parts;
        a.dlam_part = d_parts + m;
        a.flags = h->d_flags;
        a.f = f;
        a.lambda = lambda;
        const size_t smem = smem_of<T>(FP);
        if (smem > 48 * 1024)
            step(cudaFuncSetAttribute(adjoint_row_kernel<T>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (e == cudaSuccess && m > 0) adjoint_row_kernel<T><<<(unsigned)m, nt_of(FP), smem, st>>>(a, FP);
        step(cudaGetLastError());
        const size_t ismem = sizeof(T) * ITEM_WARPS * (size_t)f;
        if (e == cudaSuccess && n > 0) {
            adjoint_chunk_kernel<T><<<(unsigned)std::min<int64_t>(nchunks, 152 * 8),
                                      32 * ITEM_WARPS, ismem, st>>>(
                nchunks, f, d_chunks, d_chunks + nchunks, d_chunks + 2 * nchunks, h->d_csc_idx,
                h->d_csc_val, d_hptr_i, d_hrow_i, d_hval_i, d_Y, d_X, d_G, d_part);
            adjoint_combine_kernel<T><<<(unsigned)std::min<int64_t>((n * f + 255) / 256, 152 * 16),
                                        256, 0, st>>>(n, f, d_chunks + 3 * nchunks, d_part, d_dY);
        }
        step(cudaGetLastError());
        sum_doubles_kernel<<<1, 256, 0, st>>>(d_parts, m, d_parts + 2 * m);
        sum_doubles_kernel<<<1, 256, 0, st>>>(d_parts + m, m, d_parts + 2 * m + 1);
        double out[2] = {0.0, 0.0};
        step(cudaMemcpyAsync(out, d_parts + 2 * m, sizeof(out), cudaMemcpyDeviceToHost, st));
        if (dLdY) {
            if (sizeof(OutT) == sizeof(T)) {
                step(cudaMemcpyAsync(dLdY, d_dY, sizeof(T) * (size_t)(n * f), cudaMemcpyDeviceToHost, st));
            } else {  // (T = double with float output does not occur)
                step(cudaErrorInvalidValue);
            }
        }
        step(cudaStreamSynchronize(st));
        if (loss) *loss = out[0];
        if (dLdlambda) *dLdlambda = out[1];
    }
    void *all[] = {d_hptr_u, d_hcol_u, d_hval_u, d_hptr_i, d_hrow_i, d_hval_i, d_X, d_G, d_dY,
                   d_parts, d_chunks, d_part};
    for (void *p : all)
        if (p) cudaFree(p);
    if (e != cudaSuccess) {
        h->last_error = std::string("adjoint: ") + cudaGetErrorString(e);
        return set_global_error(e == cudaErrorMemoryAllocation ? ALS_ERR_OUT_OF_MEMORY : ALS_ERR_CUDA,
                                h->last_error);
    }
    int32_t flags[4] = {0, 0, 0, 0};
    if (cudaMemcpy(flags, h->d_flags, sizeof(flags), cudaMemcpyDeviceToHost) == cudaSuccess)
        h->counters[1] = flags[0];
    return ALS_OK;
}

als_status check_heldout(const als_handle *h, const als_coo_view *held) {
    if (held->rows != h->m || held->cols != h->n || held->nnz < 0 || held->nnz > INT32_MAX ||
        (held->nnz > 0 && (!held->row_idxs || !held->col_idxs || !held->vals)))
        return set_global_error(ALS_ERR_INVALID_ARG, "held-out COO shape differs from the model");
    for (int64_t e = 0; e < held->nnz; ++e) {
        const int32_t r = held->row_idxs[e], c = held->col_idxs[e];
        if (r < 0 || r >= h->m || c < 0 || c >= h->n || !std::isfinite(held->vals[e]))
            return set_global_error(ALS_ERR_INVALID_ARG, "held-out entry out of range at " +
                                                             std::to_string(e));
    }
    return ALS_OK;
}

}  // namespace
}  // namespace als

using namespace als;

als_status run_adjoint(als_handle *h, const als_coo_view *held, double *loss, float *dLdY,
                       double *dLdlambda) {
    als_status s = check_heldout(h, held);
    if (s != ALS_OK) return s;
    if (fp_of(h->f) > MAX_FP) return set_global_error(ALS_ERR_UNSUPPORTED, "adjoint supports f <= 231");
    cudaSetDevice(h->cfg.device);
    return adjoint_impl<float, float>(h, held, h->d_V, h->cfg.lambda, loss, dLdY, dLdlambda);
}

als_status run_adjoint_f64(als_handle *h, const als_coo_view *held, const double *Y,
                           double lambda, double *loss, double *dLdY, double *dLdlambda) {
    als_status s = check_heldout(h, held);
    if (s != ALS_OK) return s;
    if (!Y) return set_global_error(ALS_ERR_INVALID_ARG, "null item factors");
    if (h->f > MAX_F_F64)
        return set_global_error(ALS_ERR_UNSUPPORTED, "the FP64 adjoint supports f <= 128");
    if (!(lambda >= 0.0) || !std::isfinite(lambda))
        return set_global_error(ALS_ERR_INVALID_ARG, "lambda must be finite and >= 0");
    cudaSetDevice(h->cfg.device);
    const size_t nf = (size_t)h->n * h->f;
    double *d_Y = nullptr;
    cudaError_t e = cudaMalloc(&d_Y, sizeof(double) * (nf ? nf : 1));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_Y, Y, sizeof(double) * nf, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && nf) {  // the handle's V follows, rounded to FP32
        f64_to_f32_kernel<<<(unsigned)std::min<size_t>((nf + 255) / 256, 152 * 16), 256, 0,
                            h->stream>>>(d_Y, (int64_t)nf, h->d_V);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        if (d_Y) cudaFree(d_Y);
        return set_global_error(ALS_ERR_CUDA, std::string("adjoint: ") + cudaGetErrorString(e));
    }
    s = adjoint_impl<double, double>(h, held, d_Y, lambda, loss, dLdY, dLdlambda);
    cudaFree(d_Y);
    return s;
}
