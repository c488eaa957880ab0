// solvers.cuh — per-row solvers of the normal equations A x = b in shared memory, used by the
// FP32 and the tensor-core half-sweeps.  A is symmetric and held as its lower triangle with row
// stride gs; every routine is run by a group of `nt` threads (whole warps) that synchronise
// through Sync::sync() — the whole CTA in the FP32 kernel, one named barrier of the solver
// warpgroup in the warp-specialised tensor-core kernel.
//
// Reference solvers restated: LU without pivoting + the two triangular solves
// (cublasSgetrfBatched/getrsBatched with PivotArray = NULL, als_model.cu:1594, :1615-1627) and
// the warm-started CG of cumf_als_cg/cg.cu:37-232.  LDL^T is this build's Cholesky.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace als {

struct CtaSync {
    __device__ static void sync() { __syncthreads(); }
};

template <int ID, int NT>
struct NamedSync {
    __device__ static void sync() { asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(NT) : "memory"); }
};

// Deterministic group sum (fixed combination order); red holds >= 33 values.
template <class Sync, typename T = float>
__device__ T group_sum(T v, T *red, int tid, int nt) {
    const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    Sync::sync();
    if (tid == 0) {
        T s = T(0);
        for (int w = 0; w < nwarps; ++w) s += red[w];
        red[32] = s;
    }
    Sync::sync();
    const T s = red[32];
    Sync::sync();
    return s;
}

__device__ __forceinline__ float sym_at(const float *G, int gs, int i, int j) {
    return i >= j ? G[i * gs + j] : G[j * gs + i];
}

// ap = A p, one warp per row.
template <class Sync>
__device__ void sym_matvec(const float *G, int gs, int f, const float *p, float *ap, int tid,
                           int nt) {
    const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    for (int i = warp; i < f; i += nwarps) {
        float s = 0.f;
        for (int j = lane; j < f; j += 32) s = fmaf(sym_at(G, gs, i, j), p[j], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) ap[i] = s;
    }
    Sync::sync();
}

// Square-root-free Cholesky A = L D L^T in place on the lower triangle (right-looking; the
// multipliers l_ik = a_ik / d_k are applied on the fly, one barrier per column).  Returns false,
// uniformly over the group, on a pivot that is not positive and finite.
template <class Sync, typename T>
__device__ bool ldlt_factor(T *G, int gs, int f, int tid, int nt) {
    const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    for (int k = 0; k < f; ++k) {
        const T piv = G[k * gs + k];
        if (!(piv > T(0)) || !isfinite(piv)) return false;
        const T inv = T(1) / piv;
        for (int i = k + 1 + warp; i < f; i += nwarps) {
            const T lik = G[i * gs + k] * inv;
            for (int j = k + 1 + lane; j <= i; j += 32) G[i * gs + j] -= lik * G[j * gs + k];
        }
        Sync::sync();
    }
    return true;
}

// b <- (L D L^T)^-1 b, by the group's first warp.
template <class Sync, typename T>
__device__ void ldlt_solve(const T *G, int gs, int f, T *b, int tid) {
    if ((tid >> 5) == 0) {
        const int lane = tid & 31;
        for (int k = 0; k < f; ++k) {  // L z = b
            const T zk = b[k];
            const T inv = T(1) / G[k * gs + k];
            for (int i = k + 1 + lane; i < f; i += 32) b[i] -= G[i * gs + k] * inv * zk;
            __syncwarp();
        }
        for (int k = lane; k < f; k += 32) b[k] = b[k] / G[k * gs + k];  // D w = z
        __syncwarp();
        for (int k = f - 1; k >= 0; --k) {  // L^T x = w
            const T xk = b[k];
            for (int i = lane; i < k; i += 32) b[i] -= G[k * gs + i] / G[i * gs + i] * xk;
            __syncwarp();
        }
    }
    Sync::sync();
}

// LU without pivoting of the full matrix (the lower triangle is mirrored first), then getrs.
template <class Sync>
__device__ bool lu_nopivot_solve(float *G, int gs, int f, float *b, int tid, int nt) {
    const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    for (int i = warp; i < f; i += nwarps)
        for (int j = i + 1 + lane; j < f; j += 32) G[i * gs + j] = G[j * gs + i];
    Sync::sync();
    for (int k = 0; k < f; ++k) {
        const float piv = G[k * gs + k];
        if (piv == 0.f || !isfinite(piv)) return false;
        const float inv = 1.0f / piv;
        for (int i = k + 1 + warp; i < f; i += nwarps) {
            const float l = G[i * gs + k] * inv;
            for (int j = k + 1 + lane; j < f; j += 32) G[i * gs + j] -= l * G[k * gs + j];
        }
        Sync::sync();
    }
    if (warp == 0) {
        for (int k = 0; k < f; ++k) {  // unit-lower L, l_ik = a_ik / u_kk
            const float zk = b[k];
            const float inv = 1.0f / G[k * gs + k];
            for (int i = k + 1 + lane; i < f; i += 32) b[i] -= G[i * gs + k] * inv * zk;
            __syncwarp();
        }
        for (int k = f - 1; k >= 0; --k) {  // upper U
            __syncwarp();
            const float xk = b[k] / G[k * gs + k];
            __syncwarp();
            if (lane == 0) b[k] = xk;
            for (int i = lane; i < k; i += 32) b[i] -= G[i * gs + k] * xk;
            __syncwarp();
        }
    }
    Sync::sync();
    return true;
}

// Warm-started CG (cumf_als_cg/cg.cu:37-232): x from the previous factors, r = b - A x, p = r;
// per step alpha = r'r / p'Ap, x += alpha p, r -= alpha Ap, exit once r'r < tol,
// beta = r'r_new / r'r_old, p = r + beta p.  Sums run in a fixed order (the reference uses
// float atomics).  A zero p'Ap (r already 0) ends the iteration instead of dividing 0/0.
template <class Sync>
__device__ void cg_solve(const float *G, int gs, int f, const float *b, float *x, float *r,
                         float *p, float *ap, float *red, int iters, float tol, int tid, int nt) {
    sym_matvec<Sync>(G, gs, f, x, ap, tid, nt);
    float part = 0.f;
    for (int i = tid; i < f; i += nt) {
        const float ri = b[i] - ap[i];
        r[i] = ri;
        p[i] = ri;
        part += ri * ri;
    }
    float rsold = group_sum<Sync>(part, red, tid, nt);
    for (int it = 0; it < iters; ++it) {
        sym_matvec<Sync>(G, gs, f, p, ap, tid, nt);
        part = 0.f;
        for (int i = tid; i < f; i += nt) part += p[i] * ap[i];
        const float pap = group_sum<Sync>(part, red, tid, nt);
        if (!(pap > 0.f)) break;
        const float alpha = rsold / pap;
        part = 0.f;
        for (int i = tid; i < f; i += nt) {
            x[i] += alpha * p[i];
            const float ri = r[i] - alpha * ap[i];
            r[i] = ri;
            part += ri * ri;
        }
        const float rsnew = group_sum<Sync>(part, red, tid, nt);
        if (rsnew < tol) break;
        const float beta = rsnew / rsold;
        rsold = rsnew;
        for (int i = tid; i < f; i += nt) p[i] = r[i] + beta * p[i];
        Sync::sync();
    }
}

}  // namespace als
