// init.cu — the reference's factor initialisation on the GPU, bit for bit.
//
// als_model::train starts from srand(0); VT[k] = 0.2 * ((float)rand() / (float)RAND_MAX) for
// k < n f, UT = 0 (als_model.cu:1772-1784).  glibc's rand() (the additive feedback generator of
// random_r, TYPE_3: degree 31, separation 3) is the linear recurrence
//   r_0 = seed (0 taken as 1), r_i = 16807 r_{i-1} mod (2^31 - 1) for 0 < i < 31,
//   r_i = r_{i-31} for 31 <= i < 34,  r_i = r_{i-31} + r_{i-3} (mod 2^32) for i >= 34,
// and the k-th call returns r_{344+k} >> 1.  Linear over Z/2^32, so the 31-value window
// w_i = (r_{i-30} .. r_i) jumps ahead by S steps as w_{i+S} = M^S w_i (M the recurrence's 31 x 31
// companion matrix).  The host computes T = M^S and its powers T^(2^k) by squaring (a few
// million operations); GPU thread b builds the window at the start of its block of S calls as
// T^b w_0 (one matrix-vector product per set bit of b) and runs the recurrence from it, 31 calls
// per round with the window in registers.  Every output goes through the reference's own
// arithmetic: (float)(r >> 1) / (float)RAND_MAX in FP32 (RAND_MAX rounds to 2^31), times 0.2 in
// FP64, rounded to FP32.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"

namespace als {

namespace {

constexpr int DEG = 31;                  // the generator's degree
constexpr int64_t BLOCK_CALLS = DEG * 64;  // rand() calls per GPU thread
constexpr int MAX_POW = 40;                 // T^(2^k), k < MAX_POW: up to 2^40 blocks

using Mat = std::vector<uint32_t>;  // DEG x DEG, row-major, arithmetic mod 2^32

Mat mat_mul(const Mat &A, const Mat &B) {
    Mat C((size_t)DEG * DEG, 0u);
    for (int i = 0; i < DEG; ++i)
        for (int k = 0; k < DEG; ++k) {
            const uint32_t a = A[i * DEG + k];
            if (!a) continue;
            for (int j = 0; j < DEG; ++j) C[i * DEG + j] += a * B[k * DEG + j];
        }
    return C;
}

// w_0 = (r_313 .. r_343), the window before the first call, and T^(2^k) for k < npow.
void jump_tables(int npow, std::vector<uint32_t> &w0, std::vector<uint32_t> &pows) {
    std::vector<uint32_t> r(344);
    r[0] = 1u;  // srand(0): glibc takes seed 0 as 1
    for (int i = 1; i < DEG; ++i) {
        // 16807 r mod (2^31 - 1) by Schrage's split, as glibc computes it (no 64-bit products)
        const int32_t word = (int32_t)r[i - 1];
        const int32_t hi = word / 127773, lo = word % 127773;
        int32_t w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        r[i] = (uint32_t)w;
    }
    for (int i = DEG; i < 34; ++i) r[i] = r[i - DEG];
    for (int i = 34; i < 344; ++i) r[i] = r[i - 31] + r[i - 3];
    w0.assign(r.begin() + 343 - 30, r.begin() + 344);
    Mat M((size_t)DEG * DEG, 0u);  // w_{i+1} = M w_i
    for (int k = 0; k + 1 < DEG; ++k) M[k * DEG + k + 1] = 1u;
    M[(DEG - 1) * DEG + 0] = 1u;
    M[(DEG - 1) * DEG + 28] = 1u;
    Mat T((size_t)DEG * DEG, 0u), P = M;  // T = M^S
    for (int k = 0; k < DEG; ++k) T[k * DEG + k] = 1u;
    for (int64_t e = BLOCK_CALLS; e; e >>= 1) {
        if (e & 1) T = mat_mul(T, P);
        if (e > 1) P = mat_mul(P, P);
    }
    pows.resize((size_t)npow * DEG * DEG);
    for (int k = 0; k < npow; ++k) {
        std::copy(T.begin(), T.end(), pows.begin() + (size_t)k * DEG * DEG);
        if (k + 1 < npow) T = mat_mul(T, T);
    }
}

__global__ void rand_init_kernel(const uint32_t *__restrict__ tables, int npow, int64_t blocks,
                                 int64_t total, float *__restrict__ V) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= blocks) return;
    uint32_t x[DEG];
#pragma unroll
    for (int k = 0; k < DEG; ++k) x[k] = tables[k];  // w_0
    const uint32_t *pows = tables + DEG;
    for (int k = 0; k < npow; ++k) {  // x <- T^b w_0, one product per set bit of b
        if (!((b >> k) & 1)) continue;
        const uint32_t *P = pows + (size_t)k * DEG * DEG;
        uint32_t y[DEG];
#pragma unroll
        for (int i = 0; i < DEG; ++i) {
            uint32_t s = 0u;
#pragma unroll
            for (int j = 0; j < DEG; ++j) s += __ldg(P + i * DEG + j) * x[j];
            y[i] = s;
        }
#pragma unroll
        for (int i = 0; i < DEG; ++i) x[i] = y[i];
    }
    const int64_t beg = b * BLOCK_CALLS;
    const int64_t end = beg + BLOCK_CALLS < total ? beg + BLOCK_CALLS : total;
    for (int64_t base = beg; base < end; base += DEG) {
        // step j: r_new = r_{i-30} + r_{i-2}, written over r_{i-30} (slot j)
#pragma unroll
        for (int j = 0; j < DEG; ++j) {
            x[j] += x[(j + 28) % DEG];
            if (base + j < end) {
                const float q = (float)(int32_t)(x[j] >> 1) / 2147483648.0f;  // (float)RAND_MAX
                V[base + j] = (float)(0.2 * (double)q);
            }
        }
    }
}

}  // namespace

cudaError_t init_factors_device(int64_t m, int64_t n, int f, float *U, float *V,
                                cudaStream_t st) {
    const int64_t total = n * (int64_t)f;
    cudaError_t e = cudaMemsetAsync(U, 0, sizeof(float) * (size_t)(m * f), st);
    if (e != cudaSuccess || total <= 0) return e;
    const int64_t blocks = (total + BLOCK_CALLS - 1) / BLOCK_CALLS;
    int npow = 1;
    while (npow < MAX_POW && (int64_t(1) << npow) < blocks) ++npow;
    std::vector<uint32_t> w0, pows;
    jump_tables(npow, w0, pows);
    std::vector<uint32_t> tables(w0);
    tables.insert(tables.end(), pows.begin(), pows.end());
    uint32_t *d_t = nullptr;
    e = cudaMallocAsync(&d_t, sizeof(uint32_t) * tables.size(), st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(d_t, tables.data(), sizeof(uint32_t) * tables.size(),
                        cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        rand_init_kernel<<<(unsigned)((blocks + 127) / 128), 128, 0, st>>>(d_t, npow, blocks,
                                                                           total, V);
        e = cudaGetLastError();
    }
    // the table upload reads pageable host memory: wait for it before `tables` goes away
    const cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFreeAsync(d_t, st);
    return e != cudaSuccess ? e : e2;
}

}  // namespace als
