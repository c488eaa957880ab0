// index_kernels.cu — integer work of the sweep, bit-exact: exclusive scan, stable LSD radix sort,
// stable CSR->CSC transpose and the degree order of rows.
//
// The reference transposes offline with scipy (data/netflix/prepare_netflix_data.py:102-109,
// data/toy_data_2/prepare_toy_data_2.py:195-200: R.tocsr(), R.tocsc()) and loads both layouts
// from disk (main.cpp:68-71).  Here the CSC is built on the GPU from the CSR: a stable sort of
// the entries by column index keeps them in row order inside each column, which is exactly the
// order scipy's csr_tocsc produces.  All of it is HBM-bound integer traffic: coalesced tiles of
// 4096 keys per CTA, one 256-bin histogram per tile, a device-wide scan of the digit-major
// histogram matrix, then a stable scatter ranked with warp match-any.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <utility>
#include <string>

#include "internal.h"

namespace als {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 2048

constexpr int RADIX_BITS = 8;
constexpr int RADIX_BINS = 1 << RADIX_BITS;  // 256 == threads per CTA
constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ROUNDS = 16;                                 // keys per lane (histogram)
constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;          // 4096
// The scatter is latency-bound (each CTA loads its whole tile, ranks it, then writes it): it
// runs the same 4,096-key tile with twice the threads and half the keys a lane, so that two
// CTAs of 16 warps fit an SM within its registers (at 16 keys a lane, 99 registers held it to
// two CTAs of 8 warps).
constexpr int SCAT_THREADS = 512;
constexpr int SCAT_WARPS = SCAT_THREADS / 32;                     // 16
constexpr int SCAT_ROUNDS = RADIX_TILE / SCAT_THREADS;            // 8 keys per lane
constexpr int SCAT_WARP_SPAN = 32 * SCAT_ROUNDS;                  // 256 contiguous keys / warp
static_assert(SCAT_THREADS >= RADIX_BINS && RADIX_BINS % 32 == 0, "one thread per digit");

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Block-wide exclusive scan of per-thread sums (fixed order); returns this thread's prefix and
// the block total in *total.
__device__ int block_exclusive_scan(int v, int *total) {
    __shared__ int warp_sums[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    int warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0;
    *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();  // warp_sums is reused by the next call
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_reduce_kernel(const int32_t *__restrict__ in, int64_t n, int32_t *__restrict__ bsums) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i)
        if (base + i < n) s += in[base + i];
    int total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0) bsums[blockIdx.x] = total;
}

// One CTA scans the block sums in place (exclusive), looping over tiles with a carry.
__global__ void __launch_bounds__(SCAN_THREADS)
scan_bsums_kernel(int32_t *__restrict__ bsums, int64_t nb) {
    int carry = 0;
    for (int64_t t0 = 0; t0 < nb; t0 += SCAN_TILE) {
        int64_t base = t0 + (int64_t)threadIdx.x * SCAN_ITEMS;
        int v[SCAN_ITEMS];
        int s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            v[i] = base + i < nb ? bsums[base + i] : 0;
            s += v[i];
        }
        int total;
        int pre = block_exclusive_scan(s, &total) + carry;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            if (base + i < nb) bsums[base + i] = pre;
            pre += v[i];
        }
        carry += total;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS)
scan_apply_kernel(const int32_t *__restrict__ in, int32_t *__restrict__ out, int64_t n,
                  const int32_t *__restrict__ bsums, int with_total) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int total;
    int pre = block_exclusive_scan(s, &total) + bsums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < n) out[base + i] = pre;
        pre += v[i];
    }
    if (with_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_THREADS - 1)
        out[n] = pre;  // last thread's running sum == grand total
}

// ---- radix sort -----------------------------------------------------------------------------

__global__ void __launch_bounds__(RADIX_THREADS)
radix_hist_kernel(const int32_t *__restrict__ keys, int64_t n, int shift, int64_t ntiles,
                  int32_t *__restrict__ hist) {
    __shared__ int h[RADIX_BINS];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * RADIX_TILE;
#pragma unroll 4
    for (int i = 0; i < RADIX_ROUNDS; ++i) {
        int64_t pos = base + (int64_t)i * RADIX_THREADS + threadIdx.x;
        if (pos < n) atomicAdd(&h[(keys[pos] >> shift) & (RADIX_BINS - 1)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Payload words moved with the keys: pass 0 reads in[w] at the key's position (or, for word
// `pos_word`, takes the position itself), later passes read the previous pass's outputs.
struct Payload {
    const int32_t *in[3];
    int32_t *out[3];
    int pos_word;  // -1: none
};

// Stable scatter.  Warp w of tile t owns the contiguous key range [t*4096 + w*256, +256) and
// walks it in 8 rounds of 32; a key's rank inside its warp is (keys of the same digit in earlier
// rounds) + (lanes below it with the same digit in this round), found with match.any.  The warp
// offsets per digit are an exclusive prefix over warps, the tile's digit starts an exclusive
// scan over digits.  The keys and their W payload words are first placed in shared memory in
// digit order (the tile sorted by digit), then streamed out: consecutive threads write
// consecutive addresses of a digit's run, so the global stores coalesce instead of scattering 32
// ways per instruction.  A key's destination, goff[d] + (warp offset within d) + rank, is the
// same either way (stable).  Dynamic shared memory: (1 + W) x RADIX_TILE words.
template <int W>
__global__ void __launch_bounds__(SCAT_THREADS, 2)
radix_scatter_kernel(const int32_t *__restrict__ keys_in, int32_t *__restrict__ keys_out,
                     Payload pl, int64_t n, int shift, int64_t ntiles,
                     const int32_t *__restrict__ hist_scan) {
    extern __shared__ int32_t tile_words[];  // skey[RADIX_TILE], then W payload tiles
    __shared__ int wcnt[SCAT_WARPS][RADIX_BINS];
    __shared__ int goff[RADIX_BINS];
    __shared__ int tstart[RADIX_BINS];
    __shared__ int wsum[RADIX_BINS / 32];
    int32_t *skey = tile_words;
    int32_t *spay = tile_words + RADIX_TILE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool digit_thread = threadIdx.x < RADIX_BINS;  // whole warps: RADIX_BINS % 32 == 0
    for (int i = threadIdx.x; i < SCAT_WARPS * RADIX_BINS; i += SCAT_THREADS) (&wcnt[0][0])[i] = 0;
    if (digit_thread) goff[threadIdx.x] = hist_scan[(int64_t)threadIdx.x * ntiles + blockIdx.x];
    __syncthreads();

    // tile-local 32-bit offsets (n <= INT32_MAX): one 64-bit base per array
    const int64_t tile0 = (int64_t)blockIdx.x * RADIX_TILE;
    const int nvalid = (int)(n - tile0 < RADIX_TILE ? n - tile0 : RADIX_TILE);
    const int32_t *kin = keys_in + tile0;
    const int wbase = warp * SCAT_WARP_SPAN;
    const unsigned lt_mask = (1u << lane) - 1u;
    int32_t key[SCAT_ROUNDS], pay[W][SCAT_ROUNDS];
    int rank[SCAT_ROUNDS];
#pragma unroll
    for (int q = 0; q < SCAT_ROUNDS; ++q) {
        const int o = wbase + q * 32 + lane;
        const bool valid = o < nvalid;
        key[q] = valid ? kin[o] : 0;
#pragma unroll
        for (int w = 0; w < W; ++w)
            pay[w][q] = !valid ? 0 : w == pl.pos_word ? (int32_t)(tile0 + o) : pl.in[w][tile0 + o];
    }
#pragma unroll
    for (int q = 0; q < SCAT_ROUNDS; ++q) {
        const bool valid = wbase + q * 32 + lane < nvalid;
        // invalid lanes get a private digit so they never match a real one
        const int d = valid ? ((key[q] >> shift) & (RADIX_BINS - 1)) : (RADIX_BINS + lane);
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int before = valid ? wcnt[warp][d] : 0;
        rank[q] = valid ? before + __popc(peers & lt_mask) : -1;
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == lane) wcnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    int cnt = 0, incl = 0;  // keys of digit threadIdx.x in this tile; inclusive scan over digits
    if (digit_thread) {
        for (int w = 0; w < SCAT_WARPS; ++w) {  // exclusive prefix over warps for this digit
            const int t = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = cnt;
            cnt += t;
        }
        incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[warp] = incl;
    }
    __syncthreads();
    if (digit_thread) {  // tstart = exclusive scan of cnt over the 256 digits
        int add = 0;
        for (int w = 0; w < warp; ++w) add += wsum[w];
        const int ts = add + incl - cnt;
        tstart[threadIdx.x] = ts;
        goff[threadIdx.x] -= ts;  // a sorted slot j of digit d goes to goff[d] + j
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < SCAT_ROUNDS; ++q) {
        if (rank[q] < 0) continue;
        const int d = (key[q] >> shift) & (RADIX_BINS - 1);
        const int lp = tstart[d] + wcnt[warp][d] + rank[q];
        skey[lp] = key[q];
#pragma unroll
        for (int w = 0; w < W; ++w) spay[w * RADIX_TILE + lp] = pay[w][q];
    }
    __syncthreads();
#pragma unroll 2
    for (int j = threadIdx.x; j < nvalid; j += SCAT_THREADS) {
        const int32_t k = skey[j];
        const int d = (k >> shift) & (RADIX_BINS - 1);
        const int dst = goff[d] + j;
        keys_out[dst] = k;
#pragma unroll
        for (int w = 0; w < W; ++w) pl.out[w][dst] = spay[w * RADIX_TILE + j];
    }
}

// One scatter pass: the launch with its dynamic shared memory ((1 + W) 16 KB tiles; the limit
// is raised first, as the static counters and the dynamic tiles together pass 48 KB).
template <int W>
cudaError_t launch_scatter(const int32_t *keys_in, int32_t *keys_out, const Payload &pl, int64_t n,
                           int shift, int64_t ntiles, const int32_t *hist, cudaStream_t st) {
    const size_t dyn = sizeof(int32_t) * (size_t)(1 + W) * RADIX_TILE;
    cudaError_t e = cudaFuncSetAttribute(radix_scatter_kernel<W>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    radix_scatter_kernel<W><<<(unsigned)ntiles, SCAT_THREADS, dyn, st>>>(keys_in, keys_out, pl, n,
                                                                       shift, ntiles, hist);
    return cudaGetLastError();
}

// Row pointers are clamped to [0, nnz]: a malformed pointer array can never write outside.
__global__ void expand_rows_kernel(int64_t rows, int64_t nnz, const int32_t *__restrict__ ptr,
                                   int32_t *__restrict__ coo_rows) {
    const int lane = threadIdx.x & 31;
    int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < rows; r += nwarps) {
        int32_t b = max(0, min((int32_t)nnz, ptr[r])), e = max(b, min((int32_t)nnz, ptr[r + 1]));
        for (int32_t k = b + lane; k < e; k += 32) coo_rows[k] = (int32_t)r;
    }
}

// (row, value) of each CSR position side by side, so the permutation gather below reads one
// 8-byte pair (one sector) per rating instead of two 4-byte values from two arrays.
__global__ void pack_rows_vals_kernel(int64_t nnz, const int32_t *__restrict__ coo_rows,
                                      const float *__restrict__ val, int2 *__restrict__ pk) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x)
        pk[p] = make_int2(coo_rows[p], __float_as_int(val[p]));
}

__global__ void gather_csc_kernel(int64_t nnz, const int32_t *__restrict__ perm,
                                  const int2 *__restrict__ pk, int32_t *__restrict__ ridx,
                                  float *__restrict__ cval) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int2 v = pk[perm[p]];
        ridx[p] = v.x;
        cval[p] = __int_as_float(v.y);
    }
}

// col_ptrs[c] = first position whose sorted key >= c (lower bound), written without atomics.
__global__ void col_ptrs_from_sorted_kernel(int64_t nnz, int64_t cols,
                                            const int32_t *__restrict__ skeys,
                                            int32_t *__restrict__ cptr) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p <= nnz;
         p += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = p == 0 ? 0 : (int64_t)skeys[p - 1] + 1;
        int64_t hi = p == nnz ? cols : (int64_t)skeys[p];
        lo = lo < 0 ? 0 : lo;  // keys outside [0, cols) cannot write outside cptr[0..cols]
        hi = hi > cols ? cols : hi;
        for (int64_t c = lo; c <= hi; ++c) cptr[c] = (int32_t)p;
    }
}

__global__ void degree_keys_kernel(int64_t rows, const int32_t *__restrict__ ptr, int32_t maxd,
                                   int32_t *__restrict__ keys) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += (int64_t)gridDim.x * blockDim.x)
        keys[r] = maxd - (ptr[r + 1] - ptr[r]);
}

__global__ void count_bad_kernel(int64_t nnz, const int32_t *__restrict__ idx, int32_t limit,
                                 const float *__restrict__ val, int32_t *bad) {
    int local = 0;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x) {
        int32_t c = idx[p];
        float v = val ? val[p] : 0.0f;
        if (c < 0 || c >= limit || !isfinite(v)) ++local;
    }
    local = __reduce_add_sync(0xffffffffu, local);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(bad, local);
}

int grid_for(int64_t work, int threads, int cap = 152 * 16) {
    int64_t g = ceil_div(work > 0 ? work : 1, threads);
    return (int)(g < cap ? g : cap);
}

}  // namespace

// ---------------------------------------------------------------------------------------------

size_t scan_scratch_bytes(int64_t n) {
    return align256(sizeof(int32_t) * (size_t)(ceil_div(n > 0 ? n : 1, SCAN_TILE) + 1));
}

cudaError_t exclusive_scan_i32(const int32_t *in, int32_t *out, int64_t n, bool with_total,
                               void *scratch, cudaStream_t st) {
    if (n <= 0) {
        if (with_total) return cudaMemsetAsync(out, 0, sizeof(int32_t), st);
        return cudaSuccess;
    }
    int64_t nb = ceil_div(n, SCAN_TILE);
    int32_t *bsums = (int32_t *)scratch;
    scan_reduce_kernel<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, bsums);
    scan_bsums_kernel<<<1, SCAN_THREADS, 0, st>>>(bsums, nb);
    scan_apply_kernel<<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, out, n, bsums,
                                                              with_total ? 1 : 0);
    return cudaGetLastError();
}

static int radix_passes(int32_t max_key) {
    int bits = 0;
    while (bits < 31 && (int64_t(1) << bits) <= (int64_t)max_key) ++bits;
    int p = (bits + RADIX_BITS - 1) / RADIX_BITS;
    return p < 1 ? 1 : p;
}

size_t radix_sort_scratch_bytes(int64_t n) {
    int64_t ntiles = ceil_div(n > 0 ? n : 1, RADIX_TILE);
    size_t hist = (size_t)RADIX_BINS * (size_t)ntiles;
    return 4 * align256(sizeof(int32_t) * (size_t)(n > 0 ? n : 1)) +
           align256(sizeof(int32_t) * hist) + scan_scratch_bytes((int64_t)hist);
}

cudaError_t radix_sort_pairs(const int32_t *keys_in, const int32_t *vals_in, int32_t *keys_out,
                             int32_t *vals_out, int64_t n, int32_t max_key, void *scratch,
                             cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int64_t ntiles = ceil_div(n, RADIX_TILE);
    const size_t arr = align256(sizeof(int32_t) * (size_t)n);
    char *s = (char *)scratch;
    int32_t *bk[2] = {(int32_t *)s, (int32_t *)(s + 2 * arr)};
    int32_t *bv[2] = {(int32_t *)(s + arr), (int32_t *)(s + 3 * arr)};
    s += 4 * arr;
    int32_t *hist = (int32_t *)s;
    s += align256(sizeof(int32_t) * (size_t)RADIX_BINS * (size_t)ntiles);
    void *scan_scratch = s;

    const int passes = radix_passes(max_key);
    const int32_t *src_k = keys_in, *src_v = vals_in;
    for (int p = 0; p < passes; ++p) {
        int32_t *dst_k = p == passes - 1 ? keys_out : bk[p & 1];
        int32_t *dst_v = p == passes - 1 ? vals_out : bv[p & 1];
        const int shift = p * RADIX_BITS;
        radix_hist_kernel<<<(unsigned)ntiles, RADIX_THREADS, 0, st>>>(src_k, n, shift, ntiles,
                                                                       hist);
        cudaError_t e = exclusive_scan_i32(hist, hist, (int64_t)RADIX_BINS * ntiles, false,
                                           scan_scratch, st);
        if (e != cudaSuccess) return e;
        Payload pl{};
        pl.in[0] = src_v;
        pl.out[0] = dst_v;
        pl.pos_word = src_v ? -1 : 0;  // no values given: the positions themselves
        e = launch_scatter<1>(src_k, dst_k, pl, n, shift, ntiles, hist, st);
        if (e != cudaSuccess) return e;
        src_k = dst_k;
        src_v = dst_v;
    }
    return cudaGetLastError();
}

// Key + payload sets a payload-carrying sort of `cols` column ids passes through: the first pass
// reads the inputs and the last writes the outputs, so one pass needs none, two passes one (the
// 17,770 columns of the Netflix shape), more passes two in turn.
static int transpose_sets(int64_t cols) {
    const int passes = radix_passes((int32_t)(cols > 0 ? cols - 1 : 0));
    return passes >= 3 ? 2 : passes - 1;
}

size_t transpose_scratch_bytes(int64_t rows, int64_t cols, int64_t nnz, bool compact) {
    (void)rows;
    const size_t arr = align256(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    if (compact) return 3 * arr + radix_sort_scratch_bytes(nnz);
    // rows of the CSR, the sorted keys, the ping-pong sets of key + three payload words, the
    // per-tile digit histogram and its scan
    const int64_t ntiles = ceil_div(nnz > 0 ? nnz : 1, RADIX_TILE);
    const size_t hist = (size_t)RADIX_BINS * (size_t)ntiles;
    return (2 + 4 * (size_t)transpose_sets(cols)) * arr + align256(sizeof(int32_t) * hist) +
           scan_scratch_bytes((int64_t)hist);
}

cudaError_t expand_rows(int64_t rows, int64_t nnz, const int32_t *ptr, int32_t *coo_rows,
                        cudaStream_t st) {
    if (rows <= 0) return cudaSuccess;
    expand_rows_kernel<<<grid_for(rows * 32, 256), 256, 0, st>>>(rows, nnz, ptr, coo_rows);
    return cudaGetLastError();
}

cudaError_t csr_to_csc_device(int64_t rows, int64_t cols, int64_t nnz, const int32_t *ptr,
                              const int32_t *idx, const float *val, int32_t *cptr,
                              int32_t *ridx, float *cval, void *scratch, cudaStream_t st,
                              int32_t *coo_rows_out, int32_t *perm_out, bool compact) {
    if (nnz <= 0) return cudaMemsetAsync(cptr, 0, sizeof(int32_t) * (size_t)(cols + 1), st);
    const size_t arr = align256(sizeof(int32_t) * (size_t)nnz);
    char *s = (char *)scratch;
    int32_t *coo_rows = coo_rows_out ? coo_rows_out : (int32_t *)s;
    int32_t *skeys = (int32_t *)(s + arr);
    cudaError_t e = expand_rows(rows, nnz, ptr, coo_rows, st);
    if (e != cudaSuccess) return e;
    if (compact) {
        // sort (column, CSR position), then gather the (row, value) pairs by that permutation
        int32_t *perm = perm_out ? perm_out : (int32_t *)(s + 2 * arr);
        void *sort_scratch = s + 3 * arr;
        e = radix_sort_pairs(idx, nullptr, skeys, perm, nnz, (int32_t)(cols > 0 ? cols - 1 : 0),
                             sort_scratch, st);
        if (e != cudaSuccess) return e;
        // the sort's four n-int buffers are free again: the packed pairs take two of them
        int2 *pk = reinterpret_cast<int2 *>(sort_scratch);
        pack_rows_vals_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, coo_rows, val, pk);
        gather_csc_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, perm, pk, ridx, cval);
    } else {
        // sort the columns with the rating's row and value (and its CSR position when the caller
        // keeps the permutation) as payload: the last pass writes the CSC arrays themselves
        const int nsets = transpose_sets(cols);
        int32_t *set[2][4] = {};
        for (int k = 0; k < nsets; ++k)
            for (int w = 0; w < 4; ++w) set[k][w] = (int32_t *)(s + (2 + 4 * k + w) * arr);
        const int64_t ntiles = ceil_div(nnz, RADIX_TILE);
        char *hs = s + (2 + 4 * (size_t)nsets) * arr;
        int32_t *hist = (int32_t *)hs;
        void *scan_scratch = hs + align256(sizeof(int32_t) * (size_t)RADIX_BINS * ntiles);
        const int passes = radix_passes((int32_t)(cols > 0 ? cols - 1 : 0));
        for (int pass = 0; pass < passes; ++pass) {
            const bool last = pass == passes - 1;
            const int32_t *src_k = pass == 0 ? idx : set[(pass - 1) & 1][0];
            int32_t *dst_k = last ? skeys : set[pass & 1][0];
            Payload pl{};
            pl.pos_word = pass == 0 && perm_out ? 2 : -1;
            for (int w = 0; w < 3; ++w) {
                pl.in[w] = pass == 0 ? (w == 0 ? coo_rows : w == 1 ? (const int32_t *)val : nullptr)
                                     : set[(pass - 1) & 1][1 + w];
                pl.out[w] = last ? (w == 0 ? ridx : w == 1 ? (int32_t *)cval : perm_out)
                                 : set[pass & 1][1 + w];
            }
            radix_hist_kernel<<<(unsigned)ntiles, RADIX_THREADS, 0, st>>>(src_k, nnz, pass * RADIX_BITS,
                                                                         ntiles, hist);
            e = exclusive_scan_i32(hist, hist, (int64_t)RADIX_BINS * ntiles, false, scan_scratch, st);
            if (e != cudaSuccess) return e;
            e = perm_out ? launch_scatter<3>(src_k, dst_k, pl, nnz, pass * RADIX_BITS, ntiles, hist, st)
                         : launch_scatter<2>(src_k, dst_k, pl, nnz, pass * RADIX_BITS, ntiles, hist, st);
            if (e != cudaSuccess) return e;
        }
    }
    col_ptrs_from_sorted_kernel<<<grid_for(nnz + 1, 256), 256, 0, st>>>(nnz, cols, skeys, cptr);
    return cudaGetLastError();
}

size_t degree_order_scratch_bytes(int64_t rows) {
    return 2 * align256(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1)) +
           radix_sort_scratch_bytes(rows);
}

cudaError_t degree_order_device(int64_t rows, const int32_t *ptr, int32_t max_degree,
                                int32_t *perm, void *scratch, cudaStream_t st) {
    if (rows <= 0) return cudaSuccess;
    const size_t arr = align256(sizeof(int32_t) * (size_t)rows);
    char *s = (char *)scratch;
    int32_t *keys = (int32_t *)s;
    int32_t *skeys = (int32_t *)(s + arr);
    degree_keys_kernel<<<grid_for(rows, 256), 256, 0, st>>>(rows, ptr, max_degree, keys);
    return radix_sort_pairs(keys, nullptr, skeys, perm, rows, max_degree, s + 2 * arr, st);
}

__global__ void gather_f32_kernel(int64_t n, const int32_t *__restrict__ perm,
                                  const float *__restrict__ src, float *__restrict__ dst) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x)
        dst[p] = src[perm[p]];
}

cudaError_t ptrs_from_sorted(int64_t n, int64_t nkeys, const int32_t *skeys, int32_t *ptr,
                             cudaStream_t st) {
    if (n <= 0) return cudaMemsetAsync(ptr, 0, sizeof(int32_t) * (size_t)(nkeys + 1), st);
    col_ptrs_from_sorted_kernel<<<grid_for(n + 1, 256), 256, 0, st>>>(n, nkeys, skeys, ptr);
    return cudaGetLastError();
}

cudaError_t gather_f32(int64_t n, const int32_t *perm, const float *src, float *dst,
                       cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    gather_f32_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, perm, src, dst);
    return cudaGetLastError();
}

cudaError_t count_bad_entries(int64_t nnz, const int32_t *idx, int32_t limit, const float *val,
                              int32_t *bad, cudaStream_t st) {
    if (nnz <= 0) return cudaSuccess;
    count_bad_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, idx, limit, val, bad);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// CSR -> CSC without any allocation, for callers that may not allocate device memory.
//
// Some callers cannot call cudaMalloc (or have torch or any other allocator do it for them):
// plug-ins hosted by an engine that owns all device memory and forbids allocations inside its
// callbacks, and latency-critical loops that must not synchronise on the allocator.  For them the
// transpose's scratch lives in one file-scope device array of NOALLOC_SCRATCH_BYTES (16 MiB),
// which every GPU that loads this library holds until the process exits.  The compact transpose
// needs 28 bytes per rating plus 1 KiB per 4,096 ratings (its radix histograms), each array
// rounded up to 256 bytes, which admits at most 593,856 ratings; larger inputs are rejected with
// ALS_ERR_INVALID_ARG before anything runs.
//
// In host code the array's name is only a host-side stand-in, so the device address is looked up
// with cudaGetSymbolAddress (with the device current) on the first call made in each CUDA
// context, and looked up again when the device's context changes (after cudaDeviceReset the
// module reloads at another address).  Every call shares the one array: calls whose work
// overlaps on the GPU (different streams, or several threads) race on it and must be serialised
// by the caller.  The transpose writes every scratch word before it reads it, so no clearing is
// needed between calls.
// ---------------------------------------------------------------------------------------------

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 16u << 20;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};
unsigned long long g_noalloc_ctx[NOALLOC_MAX_DEVICES] = {};  // cuCtxGetId of the lookup's context

// The unique id of the calling thread's current CUDA context (cuCtxGetCurrent + cuCtxGetId
// through the runtime's driver entry points; no link against libcuda); 0 if unavailable.
unsigned long long current_context_id() {
    typedef int (*GetCurrentFn)(void **);
    typedef int (*GetIdFn)(void *, unsigned long long *);
    static const std::pair<GetCurrentFn, GetIdFn> fns = []() {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) !=
                cudaSuccess || qa != cudaDriverEntryPointSuccess)
            a = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) !=
                cudaSuccess || qb != cudaDriverEntryPointSuccess)
            b = nullptr;
        return std::make_pair(reinterpret_cast<GetCurrentFn>(a), reinterpret_cast<GetIdFn>(b));
    }();
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (!fns.first || !fns.second || fns.first(&ctx) != 0 || !ctx || fns.second(ctx, &id) != 0)
        return 0;
    return id;
}

}  // namespace

}  // namespace als

extern "C" als_status als_csr_to_csc_device_noalloc(const als_csr_view *csr, int32_t *col_ptrs,
                                                    int32_t *row_idxs, float *vals,
                                                    void *stream) {
    using namespace als;
    if (!csr || !col_ptrs || !csr->row_ptrs ||
        (csr->nnz > 0 && (!row_idxs || !vals || !csr->col_idxs || !csr->vals)))
        return set_global_error(ALS_ERR_INVALID_ARG, "null argument");
    if (csr->rows < 0 || csr->cols < 0 || csr->nnz < 0 || csr->nnz > INT32_MAX ||
        csr->rows >= INT32_MAX || csr->cols >= INT32_MAX)
        return set_global_error(ALS_ERR_INVALID_ARG, "shape out of range");
    const size_t need = transpose_scratch_bytes(csr->rows, csr->cols, csr->nnz, true);
    if (need > NOALLOC_SCRATCH_BYTES)
        return set_global_error(
            ALS_ERR_INVALID_ARG,
            "als_csr_to_csc_device_noalloc: " + std::to_string(csr->nnz) +
                " ratings need " + std::to_string(need) + " bytes of scratch, more than its fixed " +
                std::to_string(NOALLOC_SCRATCH_BYTES) + "-byte array; use als_csr_to_csc_device");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return set_global_error(ALS_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return set_global_error(ALS_ERR_UNSUPPORTED, "device ordinal beyond 63");
    void *scratch = nullptr;
    {
        // cudaGetDevice made the device's primary context current if it was not yet
        const unsigned long long ctx = current_context_id();
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
            // set-up, once per device and context, with that device current
            void *addr = nullptr;
            e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
            if (e != cudaSuccess || !addr)
                return set_global_error(ALS_ERR_CUDA,
                                        std::string("cudaGetSymbolAddress: ") +
                                            cudaGetErrorString(e));
            g_noalloc_addr[dev] = addr;
            g_noalloc_ctx[dev] = ctx;
        }
        scratch = g_noalloc_addr[dev];
    }
    e = csr_to_csc_device(csr->rows, csr->cols, csr->nnz, csr->row_ptrs, csr->col_idxs,
                          csr->vals, col_ptrs, row_idxs, vals, scratch, (cudaStream_t)stream,
                          nullptr, nullptr, /*compact=*/true);
    if (e != cudaSuccess)
        return set_global_error(ALS_ERR_CUDA, std::string("csr_to_csc: ") + cudaGetErrorString(e));
    return ALS_OK;
}

