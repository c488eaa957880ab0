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
//   cg_quad       the same CG with four rows shared by a lane quad (half of them in shared
//                 memory): a quarter of the p reads, for rows too long to keep in registers.
//   chol_fac      Cholesky A = L L^T of the Gram copied to a packed lower triangle in shared
//                 memory, left-looking in blocks of 8 columns: the dot products are spread over
//                 all 128 threads as (row, column-half) items, one thread factors and inverts
//                 each 8 x 8 diagonal block in registers, three barriers per block.
//   chol_solve_group  L y = b and L^T x = y by the group, one barrier per 8-row block.
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

// Two fixed-order sums over the 128 threads in one pass (one barrier); `red` as for gsum128 (the
// two values of a warp share a float2 of the same ring slot: 4 x 8 floats).
__device__ __forceinline__ float2 gsum128x2(float u, float v, float *red, int &slot,
                                            const GroupSync &gs) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        u += __shfl_xor_sync(0xffffffffu, u, o);
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    float2 *r = reinterpret_cast<float2 *>(red) + 4 * (slot & 3);
    ++slot;
    if ((threadIdx.x & 31) == 0) r[((threadIdx.x >> 5) & 3)] = make_float2(u, v);
    gs.sync();
    const float2 a = r[0], b = r[1], c = r[2], d = r[3];
    return make_float2((a.x + b.x) + (c.x + d.x), (a.y + b.y) + (c.y + d.y));
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

// CG with one reduction per iteration (Chronopoulos and Gear, 1989): with w = A r, the two dot
// products gamma = r'r and delta = r'w are summed together, and p'Ap = delta - beta gamma / alpha
// follows from the recurrences.  In exact arithmetic the iterates are those of the reference's
// CG (cumf_als_cg/cg.cu:37-232, warm start, at most `iters` updates, exit when r'r < tol after an
// update, stop before an update whose p'Ap is not positive); a product of A follows every update
// but the last, so without an early exit it performs the same iters + 1 products, with one
// barrier and one two-value reduction per iteration instead of three barriers and two
// reductions.  `mul(v)` returns (A v)_i after publishing v_i to the group (it synchronises).
template <class Mul>
__device__ __forceinline__ float cg_single_reduction(Mul mul, float bi, float xi, float *red,
                                                     int iters, float tol, const GroupSync &gs) {
    int slot = 0;
    float r = bi - mul(xi);
    gs.sync();  // every thread has read x out of the shared vector before r overwrites it
    float w = mul(r);
    float2 gd = gsum128x2(r * r, r * w, red, slot, gs);
    float gamma = gd.x, pap = gd.y;
    float p = r, s = w, alpha = 0.f;
    for (int it = 0; it < iters; ++it) {
        if (!(pap > 0.f)) break;
        alpha = gamma / pap;
        xi = fmaf(alpha, p, xi);
        r = fmaf(-alpha, s, r);
        if (it + 1 == iters) break;  // no further update: the product would be unused
        w = mul(r);
        gd = gsum128x2(r * r, r * w, red, slot, gs);
        if (gd.x < tol) break;
        const float beta = gd.x / gamma;
        pap = gd.y - beta * gd.x / alpha;  // p_new' A p_new
        gamma = gd.x;
        p = fmaf(beta, p, r);
        s = fmaf(beta, s, w);
    }
    return xi;
}

template <int FP>
__device__ float cg_reg(const float (&a)[FP], float bi, float xi, int i, float *sv, float *red,
                        int iters, float tol, const GroupSync &gs) {
    const bool live = i < FP;  // threads past the padded size hold zero rows and write nothing
    auto mul = [&](float v) -> float {
        if (live) sv[i] = v;  // every thread finished reading sv at the previous reduction
        gs.sync();
        return dot_row<FP>(a, sv);
    };
    return cg_single_reduction(mul, bi, xi, red, iters, tol, gs);
}

// CG as cg_reg with the rows quad-blocked (FP = 112).  The four lanes 4a..4a+3 of a warp share
// rows 4a..4a+3: lane 4a+c holds columns 16k+4c..16k+4c+3 (k < NK = FP/16) of all four, rows 4a
// and 4a+1 in registers (ar[0], ar[1]), rows 4a+2 and 4a+3 in shared memory (slots 2k and 2k+1
// of `sa`, the thread's own float4 in each).  A product reads FP/4 floats of p a thread, one
// float4 per chunk shared by the four rows, where a whole row a thread needs all FP of them; the
// quad's partial sums are then reduced and scattered so that lane 4a+c ends with row 4a+c.
constexpr int CGQ_SLOT = 130;  // float4 a slot: 128 threads + 2 (staggers the slots' banks)

__device__ __forceinline__ float4 shfl_xor4(float4 v, int m) {
    return make_float4(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m),
                       __shfl_xor_sync(0xffffffffu, v.z, m), __shfl_xor_sync(0xffffffffu, v.w, m));
}

template <int NK>
__device__ __forceinline__ float dot_quad(const float4 (&ar)[2][NK], const float4 *sa,
                                          const float *sv, int t) {
    const int c = t & 3;
    const float4 *pv = reinterpret_cast<const float4 *>(sv) + c;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int k = 0; k < NK; ++k) {
        const float4 v = pv[4 * k];
        const float4 s2 = sa[(2 * k) * CGQ_SLOT + t];
        const float4 s3 = sa[(2 * k + 1) * CGQ_SLOT + t];
        a0 = fmaf(ar[0][k].x, v.x, fmaf(ar[0][k].y, v.y, fmaf(ar[0][k].z, v.z, fmaf(ar[0][k].w, v.w, a0))));
        a1 = fmaf(ar[1][k].x, v.x, fmaf(ar[1][k].y, v.y, fmaf(ar[1][k].z, v.z, fmaf(ar[1][k].w, v.w, a1))));
        a2 = fmaf(s2.x, v.x, fmaf(s2.y, v.y, fmaf(s2.z, v.z, fmaf(s2.w, v.w, a2))));
        a3 = fmaf(s3.x, v.x, fmaf(s3.y, v.y, fmaf(s3.z, v.z, fmaf(s3.w, v.w, a3))));
    }
    // reduce-scatter over the quad: lanes c, c^2 combine rows {0,1} (c < 2) or {2,3}, then
    // lanes c, c^1 combine row c
    const bool hi = (c & 2) != 0;
    float k0 = hi ? a2 : a0, k1 = hi ? a3 : a1;
    const float s0 = hi ? a0 : a2, s1 = hi ? a1 : a3;
    k0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    k1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    const bool odd = (c & 1) != 0;
    return (odd ? k1 : k0) + __shfl_xor_sync(0xffffffffu, odd ? k0 : k1, 1);
}

// The quad-blocked rows hold the Gram without its diagonal term: thread i adds dreg * v_i (lambda
// n_u, or 1 on a padded row, whose Gram row is zero) to each product.
template <int NK>
__device__ float cg_quad(const float4 (&ar)[2][NK], const float4 *sa, float bi, float xi, int i,
                         float *sv, float *red, int iters, float tol, const GroupSync &gs,
                         float dreg) {
    constexpr int FP = 16 * NK;
    const bool live = i < FP;
    auto mul = [&](float v) -> float {
        if (live) sv[i] = v;
        gs.sync();
        return fmaf(dreg, v, dot_quad<NK>(ar, sa, sv, i));
    };
    return cg_single_reduction(mul, bi, xi, red, iters, tol, gs);
}

// Packed lower triangle of an FP x FP factor in shared memory.  Row i (block K = i / 8) keeps
// columns 0 .. 8(K+1)-1, so every 8 x 8 block a row touches is whole; rows are laid out one
// after the other with 4 floats of skew each, which keeps the float4 loads of 8 consecutive
// rows on distinct banks.  Offsets are multiples of 4 floats (16-byte aligned float4 access).
__device__ __forceinline__ int tri_off(int i) {
    const int K = i >> 3;
    return 8 * (K + 1) * (4 * K + (i & 7)) + 4 * i;
}
template <int FP>
struct TriLayout {
    static constexpr int floats = 32 * (FP / 8) * (FP / 8 + 1) + 4 * FP;
};

// Cholesky A = L L^T of the padded FP x FP matrix held in Ls (packed, tri_off rows; entry (i, j)
// for j <= i must be set, the rest of each row's blocks is scratch).  On exit entry (i, j <= i)
// holds L[i][j], Dv[K * 64 + r * 8 + c] = (L_KK^-1)[r][c] for r >= c (the inverse of each 8 x 8
// diagonal block) and invd[j] = 1 / L[j][j].  Called by the 128 threads of a group (et = 0..127);
// thread `lead` factors the diagonal blocks.
//
// Left-looking in blocks of 8 columns, three barriers per block:
//  (a) every (row r >= k0, half h) pair subtracts L[r][0:k0] . L[k0+4h+kk][0:k0], kk < 4, from
//      its 4 entries: work spread evenly over the 128 threads whatever the row count left;
//  (b) one thread (lead) factors the 8 x 8 diagonal block in registers (rsqrt pivots) and
//      inverts it;
//  (c) every row below takes its block columns as s L_KK^-T.
// Returns false (on thread lead) if a pivot was not positive and finite.
template <int FP>
__device__ bool chol_fac(int et, int lead, float *Ls, float *Dv, float *invd, const GroupSync &gs) {
    constexpr int B = 8;
    bool ok = true;
#pragma unroll 1
    for (int K = 0; K < FP / B; ++K) {
        const int k0 = K * B;
        if (k0 > 0) {
            const int nitems = 2 * (FP - k0);
            for (int t = et; t < nitems; t += 128) {
                const int r = k0 + (t >> 1), c0 = k0 + 4 * (t & 1);
                float *lr = Ls + tri_off(r);
                const float *l0 = Ls + tri_off(c0), *l1 = Ls + tri_off(c0 + 1);
                const float *l2 = Ls + tri_off(c0 + 2), *l3 = Ls + tri_off(c0 + 3);
                float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll 2
                for (int q = 0; q < k0; q += 4) {
                    const float4 o = *reinterpret_cast<const float4 *>(lr + q);
                    const float4 a0 = *reinterpret_cast<const float4 *>(l0 + q);
                    const float4 a1 = *reinterpret_cast<const float4 *>(l1 + q);
                    const float4 a2 = *reinterpret_cast<const float4 *>(l2 + q);
                    const float4 a3 = *reinterpret_cast<const float4 *>(l3 + q);
                    s0 = fmaf(o.x, a0.x, s0); s1 = fmaf(o.x, a1.x, s1);
                    s2 = fmaf(o.x, a2.x, s2); s3 = fmaf(o.x, a3.x, s3);
                    s0 = fmaf(o.y, a0.y, s0); s1 = fmaf(o.y, a1.y, s1);
                    s2 = fmaf(o.y, a2.y, s2); s3 = fmaf(o.y, a3.y, s3);
                    s0 = fmaf(o.z, a0.z, s0); s1 = fmaf(o.z, a1.z, s1);
                    s2 = fmaf(o.z, a2.z, s2); s3 = fmaf(o.z, a3.z, s3);
                    s0 = fmaf(o.w, a0.w, s0); s1 = fmaf(o.w, a1.w, s1);
                    s2 = fmaf(o.w, a2.w, s2); s3 = fmaf(o.w, a3.w, s3);
                }
                float4 *d = reinterpret_cast<float4 *>(lr + c0);
                float4 v = *d;
                v.x -= s0; v.y -= s1; v.z -= s2; v.w -= s3;
                *d = v;
            }
            gs.sync();
        }
        if (et == lead) {
            // (b) factor: right-looking inside the block, everything in registers
            float m[B][B];
#pragma unroll
            for (int r = 0; r < B; ++r) {
                const float *lr = Ls + tri_off(k0 + r) + k0;
                const float4 x = *reinterpret_cast<const float4 *>(lr);
                const float4 y = *reinterpret_cast<const float4 *>(lr + 4);
                m[r][0] = x.x; m[r][1] = x.y; m[r][2] = x.z; m[r][3] = x.w;
                m[r][4] = y.x; m[r][5] = y.y; m[r][6] = y.z; m[r][7] = y.w;
            }
            float iv[B];
#pragma unroll
            for (int k = 0; k < B; ++k) {
                const float dk2 = m[k][k];
                const bool good = dk2 > 0.f && isfinite(dk2);
                ok = ok && good;
                const float inv = good ? rsqrtf(dk2) : 1.f;
                m[k][k] = good ? dk2 * inv : 1.f;
                iv[k] = inv;
#pragma unroll
                for (int r = k + 1; r < B; ++r) m[r][k] *= inv;
#pragma unroll
                for (int r = k + 1; r < B; ++r)
#pragma unroll
                    for (int j = k + 1; j <= r; ++j) m[r][j] = fmaf(-m[r][k], m[j][k], m[r][j]);
            }
#pragma unroll
            for (int r = 0; r < B; ++r) {  // L rows (entries right of the diagonal: zero)
                float *lr = Ls + tri_off(k0 + r) + k0;
                *reinterpret_cast<float4 *>(lr) = make_float4(
                    m[r][0], r >= 1 ? m[r][1] : 0.f, r >= 2 ? m[r][2] : 0.f, r >= 3 ? m[r][3] : 0.f);
                *reinterpret_cast<float4 *>(lr + 4) =
                    make_float4(r >= 4 ? m[r][4] : 0.f, r >= 5 ? m[r][5] : 0.f,
                                r >= 6 ? m[r][6] : 0.f, r >= 7 ? m[r][7] : 0.f);
            }
            *reinterpret_cast<float4 *>(invd + k0) = make_float4(iv[0], iv[1], iv[2], iv[3]);
            *reinterpret_cast<float4 *>(invd + k0 + 4) = make_float4(iv[4], iv[5], iv[6], iv[7]);
            // inverse, one column at a time: D[c][c] = 1 / L_cc,
            // D[r][c] = -(sum_{c <= t < r} L[r][t] D[t][c]) / L[r][r]
            float *dv = Dv + K * B * B;
#pragma unroll
            for (int c = 0; c < B; ++c) {
                float d[B];
#pragma unroll
                for (int r = c; r < B; ++r) {
                    if (r == c) {
                        d[r] = iv[c];
                    } else {
                        float acc = 0.f;
#pragma unroll
                        for (int t = c; t < r; ++t) acc = fmaf(m[r][t], d[t], acc);
                        d[r] = -acc * iv[r];
                    }
                    dv[r * B + c] = d[r];
                }
            }
        }
        gs.sync();
        // (c) rows below the block
        const float *dv = Dv + K * B * B;
        for (int t = et; t < FP - k0 - B; t += 128) {
            float *lr = Ls + tri_off(k0 + B + t) + k0;
            const float4 x = *reinterpret_cast<const float4 *>(lr);
            const float4 y = *reinterpret_cast<const float4 *>(lr + 4);
            const float sb[B] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
            float o[B];
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                float acc = 0.f;
#pragma unroll
                for (int q = 0; q <= kk; ++q) acc = fmaf(sb[q], dv[kk * B + q], acc);
                o[kk] = acc;
            }
            *reinterpret_cast<float4 *>(lr) = make_float4(o[0], o[1], o[2], o[3]);
            *reinterpret_cast<float4 *>(lr + 4) = make_float4(o[4], o[5], o[6], o[7]);
        }
        gs.sync();
    }
    return ok;
}

// x = (L L^T)^-1 v for the factor left by chol_fac, by the whole group: thread t keeps the
// running value of row t.  Per 8-row block (forward, then backward from the bottom) the warp that
// owns the block's rows forms its 8 results with the block's inverse (lane l0 + c computes result
// c from shuffles of the block rows' running values) and publishes them in `xb`; after one barrier
// every thread folds them into its own row: forward L[t][k0..k0+7] . y, backward
// L[k0..k0+7][t] . x.  Each row sees the same FMA sequence as in a one-warp solve.  Blocks use the
// two 8-float halves of `xb` in turn (the backward sweep starting on the half the forward sweep did
// not end on), so a block's writer never overwrites values a thread has yet to read.  v (FP floats
// of shared memory) holds b on entry and x on exit, each thread reading and writing its own row.
template <int FP>
__device__ void chol_solve_group(int et, const float *Ls, const float *Dv, float *v, float *xb,
                                 const GroupSync &gs) {
    constexpr int B = 8;
    constexpr int NB = FP / B;
    const int lane = et & 31, w = et >> 5;
    const bool live = et < FP;
    float acc = live ? v[et] : 0.f;
    // forward: L y = b
#pragma unroll 1
    for (int K = 0; K < NB; ++K) {
        const int k0 = K * B;
        float *yb = xb + (K & 1) * B;
        if (w == (k0 >> 5)) {  // warp-uniform: the warp holding rows k0..k0+7
            const int l0 = k0 & 31, c = lane - l0;
            float r[B];
#pragma unroll
            for (int q = 0; q < B; ++q) r[q] = __shfl_sync(0xffffffffu, acc, l0 + q);
            if (c >= 0 && c < B) {
                const float *dr = Dv + K * B * B + c * B;  // row c of the block's inverse, q <= c
                float y = 0.f;
#pragma unroll
                for (int q = 0; q < B; ++q)
                    if (q <= c) y = fmaf(dr[q], r[q], y);
                acc = y;
                yb[c] = y;
            }
        }
        gs.sync();
        if (live && et >= k0 + B) {
            const float4 a0 = *reinterpret_cast<const float4 *>(Ls + tri_off(et) + k0);
            const float4 a1 = *reinterpret_cast<const float4 *>(Ls + tri_off(et) + k0 + 4);
            const float4 y0 = *reinterpret_cast<const float4 *>(yb);
            const float4 y1 = *reinterpret_cast<const float4 *>(yb + 4);
            float t = acc;
            t = fmaf(-a0.x, y0.x, t);
            t = fmaf(-a0.y, y0.y, t);
            t = fmaf(-a0.z, y0.z, t);
            t = fmaf(-a0.w, y0.w, t);
            t = fmaf(-a1.x, y1.x, t);
            t = fmaf(-a1.y, y1.y, t);
            t = fmaf(-a1.z, y1.z, t);
            t = fmaf(-a1.w, y1.w, t);
            acc = t;
        }
    }
    // backward: L^T x = y, blocks from the bottom
#pragma unroll 1
    for (int K = NB - 1; K >= 0; --K) {
        const int k0 = K * B;
        float *xk = xb + ((K + 1) & 1) * B;
        if (w == (k0 >> 5)) {
            const int l0 = k0 & 31, c = lane - l0;
            float r[B];
#pragma unroll
            for (int q = 0; q < B; ++q) r[q] = __shfl_sync(0xffffffffu, acc, l0 + q);
            if (c >= 0 && c < B) {
                const float *dc = Dv + K * B * B + c;  // column c of the block's inverse, q >= c
                float x = 0.f;
#pragma unroll
                for (int q = 0; q < B; ++q)
                    if (q >= c) x = fmaf(dc[q * B], r[q], x);
                acc = x;
                xk[c] = x;
            }
        }
        gs.sync();
        if (live && et < k0) {
            const float4 x0 = *reinterpret_cast<const float4 *>(xk);
            const float4 x1 = *reinterpret_cast<const float4 *>(xk + 4);
            const float xs[B] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
            float t = acc;
#pragma unroll
            for (int kk = 0; kk < B; ++kk) t = fmaf(-Ls[tri_off(k0 + kk) + et], xs[kk], t);
            acc = t;
        }
    }
    if (live) v[et] = acc;
}

}  // namespace als
