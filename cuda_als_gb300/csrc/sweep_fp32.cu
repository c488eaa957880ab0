// sweep_fp32.cu — fused FP32 half-sweep: per-row Gram + right-hand side + regularisation + solve
// in one CTA, nothing but the solution written to HBM.
//
// Reference path replaced, per row u of the half-sweep (als_model.cu:1797-2029 for U, :2030-2267
// for V):
//   b_u = sum_k r_k y_k             cusparseScsrmm2 + cublasSgeam (als_model.cu:1816-1852)
//   A_u = sum_k y_k y_k^T + lambda n_u I
//                                   calculate_vtvs* (als_model.cu:91-167, diag term :157-159)
//   x_u = A_u^-1 b_u                LU_solve_U/V (getrf no pivot + getrs, :1570-1720)
//                                   or updateXWithCGHost (cumf_als_cg/cg.cu:683-723)
// The reference writes every f x f Gram to HBM (d_xtxs) and reads it back in the solver; here
// the Gram lives in shared memory only.
//
// Layout.  The gathered panel Z (KC ratings x FP features, FP32) carries the rating itself as
// feature f.  Each thread owns a 4 x 8 register tile of the lower block triangle of the Gram
// (8 x 8 blocks, split in two), so the FMA work is the lower triangle only; each Gram entry is
// one sequential FMA chain over the row's ratings, in rating order (the order of the reference's
// calculate_vtvs, als_model.cu:137-155).  The right-hand side is summed apart, more accurately:
// thread j sums r_k y_kj over each KC-rating chunk and adds the chunk sums with compensated
// (Kahan) addition, so b_u carries about one rounding instead of the n_u of a sequential sum.
// (An FP32 sequential right-hand side costs ALS up to 4x in accuracy against FP64 after ten
// iterations at f = 100-128: its error meets the Gram's condition number in every solve.)  After
// the last chunk the tiles are stored to shared memory (stride FP+1, conflict-free column walks)
// and the CTA solves in place.
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "internal.h"
#include "solvers.cuh"

namespace als {

namespace {

constexpr int KC = 32;      // ratings gathered per chunk
constexpr int MAX_FP = 232; // shared-memory bound of the Gram (FP x (FP+1) floats)

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

// The CTA's Gram tile assignment: thread pair (2q, 2q+1) owns 8 x 8 block (bi, bj) of the lower
// block triangle, rows r0..r0+3 of it each.
struct Tile {
    bool active;
    int r0, c0;
};
__device__ __forceinline__ Tile tile_of(int tid, int NB) {
    Tile t;
    t.active = tid < NB * (NB + 1);
    const int q = tid >> 1;
    int bi = (int)((sqrtf(8.f * q + 1.f) - 1.f) * 0.5f);
    while ((bi + 1) * (bi + 2) / 2 <= q) ++bi;
    while (bi * (bi + 1) / 2 > q) --bi;
    const int bj = q - bi * (bi + 1) / 2;
    t.r0 = 8 * bi + 4 * (tid & 1);
    t.c0 = 8 * bj;
    return t;
}

// The Gram tiles and the right-hand side of ratings [beg, end) of a row: acc += sum y y^T (one
// sequential FMA chain per entry, rating order) and b_tid (tid < f): per 32-rating chunk a
// sequential sum, the chunk sums added with Kahan compensation (bsum - bcomp is the sum).
__device__ void accumulate(const SweepArgs &a, int FP, int beg, int end, const Tile &t,
                           float (&acc)[4][8], float &bsum, float &bcomp, float *Z,
                           int32_t *scol, float *sval) {
    const int f = a.f;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
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
        if (t.active) {
            for (int k = 0; k < cnt; ++k) {
                const float4 av = *reinterpret_cast<const float4 *>(&Z[k * FP + t.r0]);
                const float4 cv0 = *reinterpret_cast<const float4 *>(&Z[k * FP + t.c0]);
                const float4 cv1 = *reinterpret_cast<const float4 *>(&Z[k * FP + t.c0 + 4]);
                const float ar[4] = {av.x, av.y, av.z, av.w};
                const float cr[8] = {cv0.x, cv0.y, cv0.z, cv0.w, cv1.x, cv1.y, cv1.z, cv1.w};
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[p][c] = fmaf(ar[p], cr[c], acc[p][c]);
            }
        }
        if (tid < f) {
            float cs = 0.f;  // this chunk's r_k y_k,tid, sequential
            for (int k = 0; k < cnt; ++k) cs = fmaf(Z[k * FP + f], Z[k * FP + tid], cs);
            const float y = cs - bcomp;  // Kahan step (no products: nothing to contract)
            const float tt = bsum + y;
            bcomp = (tt - bsum) - y;
            bsum = tt;
        }
        __syncthreads();
    }
}

// From the finished Gram tiles and b: regularise, solve with the selected solver (CG warm-started
// from the current x), write x (or x = 0 and a flag for a non-SPD / non-finite row).
__device__ void solve_and_write(const SweepArgs &a, int FP, int row, int nu, const Tile &t,
                                const float (&acc)[4][8], float b_tid, float *smem) {
    const int f = a.f, GS = FP + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    float *G = smem;  // the Gram of [Y | r] replaces the panel
    int32_t *scol = (int32_t *)(smem + zsize_of(FP));
    float *sval = (float *)(scol + KC);
    float *vb = sval + KC, *vx = vb + FP, *vr = vx + FP, *vp = vr + FP, *vap = vp + FP;
    float *red = vap + FP;
    float *xo = a.X + (int64_t)row * f;
    if (t.active) {
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int c = 0; c < 8; ++c) G[(t.r0 + p) * GS + t.c0 + c] = acc[p][c];
    }
    __syncthreads();
    const float reg = (float)nu * a.lambda;  // items_cnt * lambda (als_model.cu:157-159)
    if (tid < f) {  // (the launch has at least f threads)
        G[tid * GS + tid] += reg;
        vb[tid] = b_tid;
        vx[tid] = xo[tid];
    }
    __syncthreads();

    bool ok = true;
    const int nt = blockDim.x;
    if (a.solve == ALS_SOLVE_CG_FP32 || a.solve == ALS_SOLVE_CG_FP16) {
        if (a.solve == ALS_SOLVE_CG_FP16) {  // the Gram rounded to binary16 (cg.cu:236-430)
            for (int i = warp; i < f; i += nwarps)
                for (int j = lane; j <= i; j += 32)
                    G[i * GS + j] = __half2float(__float2half_rn(G[i * GS + j]));
            __syncthreads();
        }
        cg_solve<CtaSync>(G, GS, f, vb, vx, vr, vp, vap, red, a.cg_iters, a.cg_tol, tid, nt);
    } else if (a.solve == ALS_SOLVE_LU) {
        ok = lu_nopivot_solve<CtaSync>(G, GS, f, vb, tid, nt);
        for (int i = tid; i < f; i += blockDim.x) vx[i] = vb[i];
    } else {
        ok = ldlt_factor<CtaSync>(G, GS, f, tid, nt);
        if (ok) ldlt_solve<CtaSync>(G, GS, f, vb, tid);
        for (int i = tid; i < f; i += blockDim.x) vx[i] = vb[i];
    }
    __syncthreads();
    float bad = 0.f;
    for (int i = tid; i < f; i += blockDim.x) bad += isfinite(vx[i]) ? 0.f : 1.f;
    bad = group_sum<CtaSync>(bad, red, tid, nt);
    if (!ok || bad > 0.f) {
        for (int i = tid; i < f; i += blockDim.x) xo[i] = 0.f;
        if (tid == 0 && a.flags) atomicAdd(&a.flags[0], 1);
        return;
    }
    for (int i = tid; i < f; i += blockDim.x) xo[i] = vx[i];
}

// Rows of the order slice [row_begin, row_end), one CTA each: Gram, right-hand side, solve.
__global__ void __launch_bounds__(1024) sweep_fp32_kernel(const SweepArgs a, const int FP) {
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x;
    const int slot = a.row_begin + blockIdx.x;
    const int row = a.order ? a.order[slot] : slot;
    const int beg = a.ptr[row], end = a.ptr[row + 1], nu = end - beg;
    float *xo = a.X + (int64_t)row * a.f;
    if (nu == 0) {  // no ratings: defined as x = 0 (the reference's LU would divide by zero)
        for (int i = tid; i < a.f; i += blockDim.x) xo[i] = 0.f;
        return;
    }
    const Tile t = tile_of(tid, FP / 8);
    float acc[4][8];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[p][c] = 0.f;
    float bsum = 0.f, bcomp = 0.f;
    int32_t *scol = (int32_t *)(smem + zsize_of(FP));
    accumulate(a, FP, beg, end, t, acc, bsum, bcomp, smem, scol, (float *)(scol + KC));
    solve_and_write(a, FP, row, nu, t, acc, bsum - bcomp, smem);
}

// Heavy rows: part p accumulates ratings [beg[p], end[p]) of its row and stores its tiles (FP x GS
// floats, the lower block triangle) and its compensated right-hand side (sum, compensation).
__global__ void __launch_bounds__(1024)
    gram_part_kernel(const SweepArgs a, const int FP, const int32_t *__restrict__ part_beg,
                     const int32_t *__restrict__ part_end, float *__restrict__ part) {
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x, GS = FP + 1;
    const int p = blockIdx.x;
    const Tile t = tile_of(tid, FP / 8);
    float acc[4][8];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[q][c] = 0.f;
    float bsum = 0.f, bcomp = 0.f;
    int32_t *scol = (int32_t *)(smem + zsize_of(FP));
    accumulate(a, FP, part_beg[p], part_end[p], t, acc, bsum, bcomp, smem, scol,
               (float *)(scol + KC));
    float *out = part + (int64_t)p * ((int64_t)FP * GS + 2 * FP);
    if (t.active) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int c = 0; c < 8; ++c) out[(t.r0 + q) * GS + t.c0 + c] = acc[q][c];
    }
    if (tid < a.f) {
        out[(int64_t)FP * GS + tid] = bsum;
        out[(int64_t)FP * GS + FP + tid] = bcomp;
    }
}

// Heavy row at order position h: its parts first[h]..first[h+1] added in order (the tiles
// plainly, the right-hand sides with compensation), then the common regularise / solve / write.
__global__ void __launch_bounds__(1024)
    combine_solve_kernel(const SweepArgs a, const int FP, const int32_t *__restrict__ first,
                         const float *__restrict__ part) {
    extern __shared__ __align__(16) float smem[];
    const int tid = threadIdx.x, GS = FP + 1;
    const int h = blockIdx.x;
    const int row = a.order ? a.order[h] : h;
    const int nu = a.ptr[row + 1] - a.ptr[row];
    const Tile t = tile_of(tid, FP / 8);
    float acc[4][8];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[q][c] = 0.f;
    float bsum = 0.f, bcomp = 0.f, blost = 0.f;
    const int64_t stride = (int64_t)FP * GS + 2 * FP;
    for (int32_t p = first[h]; p < first[h + 1]; ++p) {
        const float *in = part + (int64_t)p * stride;
        if (t.active) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[q][c] += in[(t.r0 + q) * GS + t.c0 + c];
        }
        if (tid < a.f) {
            const float y = in[(int64_t)FP * GS + tid] - bcomp;
            const float tt = bsum + y;
            bcomp = (tt - bsum) - y;
            bsum = tt;
            blost += in[(int64_t)FP * GS + FP + tid];
        }
    }
    solve_and_write(a, FP, row, nu, t, acc, (bsum - bcomp) - blost, smem);
}

}  // namespace

bool fp32_supported(int f) { return f >= 1 && fp_of(f) <= MAX_FP; }

cudaError_t launch_sweep_fp32(const SweepArgs &a, const Fp32Split *sp, cudaStream_t st,
                              int *launches) {
    const int FP = fp_of(a.f);
    if (nt_of(FP) < a.f) return cudaErrorInvalidConfiguration;  // thread j owns b_j
    const size_t smem = smem_of(FP);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(sweep_fp32_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(gram_part_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(combine_solve_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // the heavy rows are the first order positions: split when the slice starts there
    SweepArgs b = a;
    if (sp && sp->nheavy > 0 && a.row_begin == 0 && a.order) {
        const int32_t nh = sp->nheavy < a.row_end ? sp->nheavy : a.row_end;
        gram_part_kernel<<<(unsigned)sp->first_host[nh], nt_of(FP), smem, st>>>(
            a, FP, sp->part_beg, sp->part_end, sp->part);
        combine_solve_kernel<<<(unsigned)nh, nt_of(FP), smem, st>>>(a, FP, sp->first, sp->part);
        if (launches) *launches += 2;
        b.row_begin = nh;
    }
    const int n = b.row_end - b.row_begin;
    if (n > 0) {
        sweep_fp32_kernel<<<(unsigned)n, nt_of(FP), smem, st>>>(b, FP);
        if (launches) ++*launches;
    }
    return cudaGetLastError();
}

size_t fp32_part_floats(int f) {
    const int FP = fp_of(f);
    return (size_t)FP * (FP + 1) + 2 * (size_t)FP;
}

}  // namespace als
