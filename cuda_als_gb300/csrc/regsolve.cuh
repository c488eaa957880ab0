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
//   chol_fac      Cholesky A = L L^T of the Gram copied to shared memory, left-looking in blocks
//                 of 8 columns (a compact runtime loop, so the code stays in the instruction
//                 cache); the 8 x 8 diagonal block is factored and inverted by its owner warp;
//                 one barrier publishes it, one publishes the block column.
//   chol_solve_warp  L y = b and L^T x = y by one warp with shuffles and no barrier.
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

// Cholesky of the padded FP x FP matrix held in shared memory.  On entry row i of A sits in
// Ls[i * LS .. i * LS + FP) (LS = FP + 4; every row written and published by a barrier); on exit
// Ls[i * LS + j] = L[i][j] for j <= i (the entries right of the diagonal are left as they were),
// Dv holds the inverse of each 8 x 8 diagonal block of L (Dv[K * 64 + r * 8 + c] =
// (L_KK^-1)[r][c]) and invd[j] = 1 / L[j][j].
//
// Left-looking in blocks of 8 columns.  Step (a) subtracts the products with the finished rows of
// L: a runtime loop over 8-column chunks, the thread's own row read as two float4 (rows are LS
// floats apart, so a quarter warp's float4 loads hit distinct banks) and the 8 block rows as
// float4 broadcasts.  The owner warp factors the diagonal block with shuffles (rsqrt pivots) and
// inverts it; the rows below then take their block columns as s L_KK^-T.  Two barriers per block.
// Returns false on a thread whose pivot was not positive and finite.
template <int FP>
__device__ bool chol_fac(int i, float *Ls, float *Dv, float *invd, const GroupSync &gs) {
    constexpr int LS = FP + 4;
    constexpr int B = 8;
    const int lane = threadIdx.x & 31;
    const int wrow0 = i - lane;  // first row of this warp
    const bool live = i < FP;
    float *li = Ls + (live ? i : 0) * LS;
    bool ok = true;
#pragma unroll 1
    for (int K = 0; K < FP / B; ++K) {
        const int k0 = K * B;
        float blk[B];
#pragma unroll
        for (int q = 0; q < B; ++q) blk[q] = 0.f;
        if (live && i >= k0) {
            const float4 t0 = *reinterpret_cast<const float4 *>(li + k0);
            const float4 t1 = *reinterpret_cast<const float4 *>(li + k0 + 4);
            float s[B];
#pragma unroll
            for (int q = 0; q < B; ++q) s[q] = 0.f;
#pragma unroll 2
            for (int q = 0; q < k0; q += 8) {
                const float4 o0 = *reinterpret_cast<const float4 *>(li + q);
                const float4 o1 = *reinterpret_cast<const float4 *>(li + q + 4);
#pragma unroll
                for (int kk = 0; kk < B; ++kk) {
                    const float *lk = Ls + (k0 + kk) * LS + q;
                    const float4 l0 = *reinterpret_cast<const float4 *>(lk);
                    const float4 l1 = *reinterpret_cast<const float4 *>(lk + 4);
                    float t = s[kk];
                    t = fmaf(o0.x, l0.x, t);
                    t = fmaf(o0.y, l0.y, t);
                    t = fmaf(o0.z, l0.z, t);
                    t = fmaf(o0.w, l0.w, t);
                    t = fmaf(o1.x, l1.x, t);
                    t = fmaf(o1.y, l1.y, t);
                    t = fmaf(o1.z, l1.z, t);
                    t = fmaf(o1.w, l1.w, t);
                    s[kk] = t;
                }
            }
            blk[0] = t0.x - s[0];
            blk[1] = t0.y - s[1];
            blk[2] = t0.z - s[2];
            blk[3] = t0.w - s[3];
            blk[4] = t1.x - s[4];
            blk[5] = t1.y - s[5];
            blk[6] = t1.z - s[6];
            blk[7] = t1.w - s[7];
        }
        float *dv = Dv + K * B * B;
        if (wrow0 <= k0 && k0 < wrow0 + 32) {
            // the owner warp factors the diagonal block with shuffles (rsqrt, no divisions)
            const int src0 = k0 - wrow0;  // lane of row k0
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                float d2 = blk[kk];
#pragma unroll
                for (int q = 0; q < kk; ++q) d2 -= blk[q] * blk[q];
                const float dk2 = __shfl_sync(0xffffffffu, d2, src0 + kk);
                const bool good = dk2 > 0.f && isfinite(dk2);
                const float inv = good ? rsqrtf(dk2) : 1.f;
                const float dk = good ? dk2 * inv : 1.f;
                if (i == k0 + kk) {
                    blk[kk] = dk;
                    invd[i] = inv;
                    ok = ok && good;
                }
                float lkq[B];
#pragma unroll
                for (int q = 0; q < kk; ++q) lkq[q] = __shfl_sync(0xffffffffu, blk[q], src0 + kk);
                if (i > k0 + kk && i < k0 + B) {
                    float s = blk[kk];
#pragma unroll
                    for (int q = 0; q < kk; ++q) s -= blk[q] * lkq[q];
                    blk[kk] = s * inv;
                }
            }
            if (i >= k0 && i < k0 + B) {  // publish the block's part of the row
                *reinterpret_cast<float4 *>(li + k0) = make_float4(blk[0], blk[1], blk[2], blk[3]);
                *reinterpret_cast<float4 *>(li + k0 + 4) =
                    make_float4(blk[4], blk[5], blk[6], blk[7]);
            }
            __syncwarp();
            if (i >= k0 && i < k0 + B) {
                // column c = i - k0 of the block inverse: d_c = 1 / L_cc,
                // d_r = -(sum_{c <= t < r} L_rt d_t) / L_rr for r > c
                const int c = i - k0;
                const float *lb = Ls + k0 * LS + k0;  // lb[r * LS + t] = L[k0+r][k0+t]
                const float *ib = invd + k0;
                float d[B];
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    float acc = r == c ? 1.f : 0.f;
#pragma unroll
                    for (int t = 0; t < r; ++t)
                        if (t >= c) acc -= lb[r * LS + t] * d[t];
                    d[r] = r >= c ? acc * ib[r] : 0.f;
                    dv[r * B + c] = d[r];
                }
            }
        }
        gs.sync();
        // rows below the block: L[i][block] = s L_block^-T, s = the block columns after (a)
        if (live && i >= k0 + B) {
            float o[B];
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                float acc = 0.f;
#pragma unroll
                for (int q = 0; q <= kk; ++q) acc = fmaf(blk[q], dv[kk * B + q], acc);
                o[kk] = acc;
            }
            *reinterpret_cast<float4 *>(li + k0) = make_float4(o[0], o[1], o[2], o[3]);
            *reinterpret_cast<float4 *>(li + k0 + 4) = make_float4(o[4], o[5], o[6], o[7]);
        }
        gs.sync();
    }
    return ok;
}

// x = (L L^T)^-1 v for the factor left by chol_fac, run by ONE warp (lane = its lane) with no
// barrier: lane l keeps the running values of rows l, l + 32, l + 64, l + 96 in registers.  Each
// 8-row block is a shuffle of its rows' values, a product with the block inverse (every lane
// computes all 8 results, so nothing is broadcast), and an update of the rows after it (forward)
// or before it (backward).  v (FP floats of shared memory) holds b on entry and x on exit.
template <int FP>
__device__ __forceinline__ float pick(const float (&v)[(FP + 31) / 32], int j) {
    float r = v[0];
#pragma unroll
    for (int q = 1; q < (FP + 31) / 32; ++q)
        if (j == q) r = v[q];
    return r;
}

template <int FP>
__device__ void chol_solve_warp(int lane, const float *Ls, const float *Dv, float *v) {
    constexpr int LS = FP + 4;
    constexpr int B = 8;
    constexpr int NJ = (FP + 31) / 32;
    float acc[NJ];
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
        const int r = lane + 32 * j;
        acc[j] = r < FP ? v[r] : 0.f;
    }
    // forward: L y = b.  The block loops stay rolled (compact code, no hoisted loads); the
    // running value of the block's rows is picked from acc[] by selects, not by indexing.
#pragma unroll 1
    for (int K = 0; K < FP / B; ++K) {
        const int k0 = K * B, jb = k0 >> 5, l0 = k0 & 31;
        const float *dv = Dv + K * B * B;
        const float cur = pick<FP>(acc, jb);
        float r[B], y[B];
#pragma unroll
        for (int q = 0; q < B; ++q) r[q] = __shfl_sync(0xffffffffu, cur, l0 + q);
        float mine = cur;
#pragma unroll
        for (int c = 0; c < B; ++c) {
            float t = 0.f;
#pragma unroll
            for (int q = 0; q <= c; ++q) t = fmaf(dv[c * B + q], r[q], t);
            y[c] = t;
            if (lane == l0 + c) mine = t;
        }
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int row = lane + 32 * j;
            if (j == jb) {
                if (row >= k0 && row < k0 + B) acc[j] = mine;
            }
            if (row >= k0 + B && row < FP) {
                const float4 a0 = *reinterpret_cast<const float4 *>(Ls + row * LS + k0);
                const float4 a1 = *reinterpret_cast<const float4 *>(Ls + row * LS + k0 + 4);
                float t = acc[j];
                t = fmaf(-a0.x, y[0], t);
                t = fmaf(-a0.y, y[1], t);
                t = fmaf(-a0.z, y[2], t);
                t = fmaf(-a0.w, y[3], t);
                t = fmaf(-a1.x, y[4], t);
                t = fmaf(-a1.y, y[5], t);
                t = fmaf(-a1.z, y[6], t);
                t = fmaf(-a1.w, y[7], t);
                acc[j] = t;
            }
        }
    }
    // backward: L^T x = y, blocks from the bottom
#pragma unroll 1
    for (int K = FP / B - 1; K >= 0; --K) {
        const int k0 = K * B, jb = k0 >> 5, l0 = k0 & 31;
        const float *dv = Dv + K * B * B;
        const float cur = pick<FP>(acc, jb);
        float r[B], x[B];
#pragma unroll
        for (int q = 0; q < B; ++q) r[q] = __shfl_sync(0xffffffffu, cur, l0 + q);
        float mine = cur;
#pragma unroll
        for (int c = 0; c < B; ++c) {
            float t = 0.f;
#pragma unroll
            for (int q = c; q < B; ++q) t = fmaf(dv[q * B + c], r[q], t);
            x[c] = t;
            if (lane == l0 + c) mine = t;
        }
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int row = lane + 32 * j;
            if (j == jb) {
                if (row >= k0 && row < k0 + B) acc[j] = mine;
            }
            if (row < k0) {
                float t = acc[j];
#pragma unroll
                for (int kk = 0; kk < B; ++kk) t = fmaf(-Ls[(k0 + kk) * LS + row], x[kk], t);
                acc[j] = t;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
        const int r = lane + 32 * j;
        if (r < FP) v[r] = acc[j];
    }
}

}  // namespace als
