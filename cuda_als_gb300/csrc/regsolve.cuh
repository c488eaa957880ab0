// regsolve.cuh — register-resident per-row solvers for the tensor-core epilogue.
//
// After tcgen05.ld, thread i of a 128-thread solver warpgroup holds row i of the (padded) Gram
// A in registers (a[0..FP)), and b_i.  Rows f <= i < FP are padded with the identity, so every
// solver runs at the compile-time size FP (a multiple of 16) and leaves x_i = 0 there.  Threads
// with i >= FP (FP < 128) hold zero rows: they join every barrier and shuffle but never index
// shared memory with i.
//
//   cg_reg        warm-started CG of cumf_als_cg/cg.cu:37-232 (same recurrences, same exit rule
//                 r'r < tol); the matvec reads p from shared memory as float4 broadcasts.
//   chol_reg      Cholesky A = L L^T, left-looking in blocks of 8 columns: the bulk of the work
//                 (dot products with the already published rows of L) runs on each thread's own
//                 registers; the 8 x 8 diagonal block is factored by its owner warp with shuffles;
//                 one barrier publishes it, one publishes the block column.
//   chol_solve_reg  L y = b and L^T x = y in the same 8-row blocks.
// Sums over threads are combined in a fixed order (deterministic).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace als {

struct GroupSync {
    int id;
    __device__ void sync() const { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
};

// Fixed-order sum over the 128 threads; `red` is a 4 x 4 float ring in shared memory, `slot`
// rotates so that consecutive calls never overwrite values still being read.
__device__ __forceinline__ float gsum128(float v, float *red, int &slot, const GroupSync &gs) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    float *r = red + 4 * (slot & 3);
    ++slot;
    if ((threadIdx.x & 31) == 0) r[((threadIdx.x >> 5) & 3)] = v;
    gs.sync();
    return (r[0] + r[1]) + (r[2] + r[3]);
}

__device__ __forceinline__ float gmax128(float v, float *red, int &slot, const GroupSync &gs) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    float *r = red + 4 * (slot & 3);
    ++slot;
    if ((threadIdx.x & 31) == 0) r[((threadIdx.x >> 5) & 3)] = v;
    gs.sync();
    return fmaxf(fmaxf(r[0], r[1]), fmaxf(r[2], r[3]));
}

// warp index inside the warpgroup that owns TMEM lanes [32w, 32w+32): tcgen05 lane quarters
// follow warp_id % 4, so thread i of the row space is (warp % 4) * 32 + lane.
template <int FP>
__device__ __forceinline__ float dot_row(const float (&a)[FP], const float *sv) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
    for (int j = 0; j < FP; j += 4) {
        const float4 v = *reinterpret_cast<const float4 *>(sv + j);
        s0 = fmaf(a[j], v.x, s0);
        s1 = fmaf(a[j + 1], v.y, s1);
        s2 = fmaf(a[j + 2], v.z, s2);
        s3 = fmaf(a[j + 3], v.w, s3);
    }
    return (s0 + s1) + (s2 + s3);
}

template <int FP>
__device__ float cg_reg(const float (&a)[FP], float bi, float xi, int i, float *sv, float *red,
                        int iters, float tol, const GroupSync &gs) {
    int slot = 0;
    const bool live = i < FP;  // threads past the padded size hold zero rows and write nothing
    if (live) sv[i] = xi;
    gs.sync();
    float r = bi - dot_row<FP>(a, sv);
    float p = r;
    float rsold = gsum128(r * r, red, slot, gs);
    for (int it = 0; it < iters; ++it) {
        if (live) sv[i] = p;  // every thread finished reading sv in the previous gsum's barrier
        gs.sync();
        const float ap = dot_row<FP>(a, sv);
        const float pap = gsum128(p * ap, red, slot, gs);
        if (!(pap > 0.f)) break;
        const float alpha = rsold / pap;
        xi = fmaf(alpha, p, xi);
        r = fmaf(-alpha, ap, r);
        const float rsnew = gsum128(r * r, red, slot, gs);
        if (rsnew < tol) break;
        const float beta = rsnew / rsold;
        rsold = rsnew;
        p = fmaf(beta, p, r);
    }
    return xi;
}

// Cholesky of the padded FP x FP matrix; thread i holds row i in a[] and leaves L[i][0..i] there.
// Ls (FP x LS floats, LS = FP + 4) receives every row of L as it is finished; Dv (FP/8 blocks of
// 8 x 8 floats) receives the inverse of each 8 x 8 diagonal block of L, which turns the triangular
// solves of the rows below a block, and later the block steps of the forward / backward solves,
// into small matrix-vector products instead of 8-step dependency chains.  Returns false on this
// thread if its pivot was not positive and finite (the caller reduces the flag).
template <int FP>
__device__ bool chol_reg(float (&a)[FP], int i, float *Ls, float *Dv, const GroupSync &gs) {
    constexpr int LS = FP + 4;
    constexpr int B = 8;
    const int lane = threadIdx.x & 31;
    const int wrow0 = i - lane;  // first row of this warp
    bool ok = true;
#pragma unroll
    for (int K = 0; K < FP / B; ++K) {
        const int k0 = K * B;
        const bool active = wrow0 + 31 >= k0;  // some row of this warp is at or below the block
        if (active && k0 > 0) {
            // a[k] -= sum_{p<k0} L[i][p] L[k][p] for the 8 columns k of the block
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                const float *lk = Ls + (k0 + kk) * LS;
                float s0 = 0.f, s1 = 0.f;
#pragma unroll
                for (int q = 0; q < k0; q += 4) {
                    const float4 l = *reinterpret_cast<const float4 *>(lk + q);
                    s0 = fmaf(a[q], l.x, s0);
                    s1 = fmaf(a[q + 1], l.y, s1);
                    s0 = fmaf(a[q + 2], l.z, s0);
                    s1 = fmaf(a[q + 3], l.w, s1);
                }
                a[k0 + kk] -= s0 + s1;
            }
        }
        float *dv = Dv + K * B * B;  // dv[r * 8 + c] = (L_block^-1)[r][c]
        if (wrow0 <= k0 && k0 < wrow0 + 32) {
            // the owner warp factors the diagonal block with shuffles (rsqrt, no divisions)
            const int src0 = k0 - wrow0;  // lane of row k0
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                float d2 = a[k0 + kk];
#pragma unroll
                for (int q = 0; q < kk; ++q) d2 -= a[k0 + q] * a[k0 + q];
                const float dk2 = __shfl_sync(0xffffffffu, d2, src0 + kk);
                const bool good = dk2 > 0.f && isfinite(dk2);
                const float inv = good ? rsqrtf(dk2) : 1.f;
                const float dk = good ? dk2 * inv : 1.f;
                if (i == k0 + kk) {
                    a[k0 + kk] = dk;
                    ok = ok && good;
                }
                float lkq[B];
#pragma unroll
                for (int q = 0; q < kk; ++q) lkq[q] = __shfl_sync(0xffffffffu, a[k0 + q], src0 + kk);
                if (i > k0 + kk && i < k0 + B) {
                    float s = a[k0 + kk];
#pragma unroll
                    for (int q = 0; q < kk; ++q) s -= a[k0 + q] * lkq[q];
                    a[k0 + kk] = s * inv;
                }
            }
            if (i >= k0 && i < k0 + B) {  // publish the block's rows (columns 0..k0+7)
                float *li = Ls + i * LS;
#pragma unroll
                for (int q = 0; q < k0 + B; q += 4)
                    *reinterpret_cast<float4 *>(li + q) =
                        make_float4(a[q], a[q + 1], a[q + 2], a[q + 3]);
            }
            __syncwarp();
            if (i >= k0 && i < k0 + B) {
                // column c = i - k0 of the block inverse: d_c = 1 / L_cc,
                // d_r = -(sum_{c <= t < r} L_rt d_t) / L_rr for r > c
                const int c = i - k0;
                const float *lb = Ls + k0 * LS + k0;  // lb[r * LS + t] = L[k0+r][k0+t]
                float d[B];
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    float acc = r == c ? 1.f : 0.f;
#pragma unroll
                    for (int t = 0; t < r; ++t)
                        if (t >= c) acc -= lb[r * LS + t] * d[t];
                    d[r] = r >= c ? acc / lb[r * LS + r] : 0.f;
                    dv[r * B + c] = d[r];
                }
            }
        }
        gs.sync();
        // rows below the block: L[i][block] = s L_block^-T, s = the block columns after (a)
        if (active && i >= k0 + B && i < FP) {
            float sblk[B];
#pragma unroll
            for (int q = 0; q < B; ++q) sblk[q] = a[k0 + q];
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                float acc = 0.f;
#pragma unroll
                for (int q = 0; q <= kk; ++q) acc = fmaf(sblk[q], dv[kk * B + q], acc);
                a[k0 + kk] = acc;
            }
            float *li = Ls + i * LS + k0;
            *reinterpret_cast<float4 *>(li) = make_float4(a[k0], a[k0 + 1], a[k0 + 2], a[k0 + 3]);
            *reinterpret_cast<float4 *>(li + 4) =
                make_float4(a[k0 + 4], a[k0 + 5], a[k0 + 6], a[k0 + 7]);
        }
        gs.sync();
    }
    return ok;
}

// x = (L L^T)^-1 b with L in Ls (rows), in each thread's registers, and the diagonal-block
// inverses in Dv; thread i returns x_i.  yv (FP floats) is shared scratch.
template <int FP>
__device__ float chol_solve_reg(const float (&a)[FP], float bi, int i, const float *Ls,
                                const float *Dv, float *yv, const GroupSync &gs) {
    constexpr int LS = FP + 4;
    constexpr int B = 8;
    const int lane = threadIdx.x & 31;
    const int wrow0 = i - lane;
    // forward: y_block = L_block^-1 (b_block - sum over earlier blocks), one block at a time
    float acc = bi;
#pragma unroll
    for (int K = 0; K < FP / B; ++K) {
        const int k0 = K * B;
        const float *dv = Dv + K * B * B;
        if (wrow0 <= k0 && k0 < wrow0 + 32) {
            const int src0 = k0 - wrow0;
            float r[B];
#pragma unroll
            for (int q = 0; q < B; ++q) r[q] = __shfl_sync(0xffffffffu, acc, src0 + q);
            if (i >= k0 && i < k0 + B) {
                const int c = i - k0;
                float y = 0.f;
#pragma unroll
                for (int q = 0; q < B; ++q)
                    if (q <= c) y = fmaf(dv[c * B + q], r[q], y);
                acc = y;
                yv[i] = y;
            }
        }
        gs.sync();
        if (i >= k0 + B) {
#pragma unroll
            for (int kk = 0; kk < B; ++kk) acc -= a[k0 + kk] * yv[k0 + kk];
        }
    }
    gs.sync();
    // backward: x_block = L_block^-T (y_block - sum over later blocks), blocks from the bottom
    float x = i < FP ? yv[i] : 0.f;
#pragma unroll
    for (int K = FP / B - 1; K >= 0; --K) {
        const int k0 = K * B;
        const float *dv = Dv + K * B * B;
        if (wrow0 <= k0 && k0 < wrow0 + 32) {
            const int src0 = k0 - wrow0;
            float r[B];
#pragma unroll
            for (int q = 0; q < B; ++q) r[q] = __shfl_sync(0xffffffffu, x, src0 + q);
            if (i >= k0 && i < k0 + B) {
                const int c = i - k0;
                float xs = 0.f;
#pragma unroll
                for (int q = 0; q < B; ++q)
                    if (q >= c) xs = fmaf(dv[q * B + c], r[q], xs);
                x = xs;
                yv[i] = xs;
            }
        }
        gs.sync();
        if (i < k0) {
#pragma unroll
            for (int kk = 0; kk < B; ++kk) x -= Ls[(k0 + kk) * LS + i] * yv[k0 + kk];
        }
    }
    gs.sync();
    return x;
}

}  // namespace als
