// sweep_tc.cu — tensor-core half-sweep: per-row Gram + right-hand side on tcgen05 (BF16 in, FP32
// accumulate in TMEM), regularisation and solve fused behind it, nothing but x_u written to HBM.
//
// Reference path replaced (per half-sweep, als_model.cu:1797-2029 / :2030-2267):
//   float2half_array (als_model.cu:54-60)            -> quantise_bf16 below (padded BF16 table)
//   csrmm2 + geam RHS (als_model.cu:1816-1852)      -> second MMA against the rating tile
//   calculate_vtvs_smem_row_major_tensor* (:428-1490, wmma 16x16x16, f <= 112 only)
//                                                    -> tcgen05.mma M=128, N=roundup(f,16)
//   LU_solve / updateXWithCGHost (:1570-1720, cg.cu) -> register solvers (regsolve.cuh) or the
//                                                       shared-memory LU (solvers.cuh)
//
// One persistent CTA per SM; rows are taken from an atomic counter in descending-degree order, so
// a 400k-rating row occupies one SM while the others drain the rest.  Warp roles:
//   solver warpgroups (first, group g = warps 4g..4g+3): group g takes every NEPI-th row.  Thread
//            i reads row i of the Gram from TMEM, adds lambda n_u to its diagonal and runs the
//            selected solver (registers / shared memory, or the tensor core for the FP16-Gram CG);
//            Cholesky refinement re-reads A from TMEM for the residual b - A x (in FP64 for rows
//            whose Cholesky diagonal ratio exceeds cond_threshold).
//   producer: walks the rows' stages (KC = 64 ratings each) and copies each stage's column ids
//            and ratings into a metadata ring MD stages ahead with cp.async, then publishes it.
//   MMA issuer: per 16 ratings one M=128 x N=Ng x K=16 MMA (Gram: A = B = the gathered panel,
//            both MN-major) and one M=128 x N=16 MMA (RHS: B = the rating tile), into one of
//            NBUF TMEM accumulators; tcgen05.commit frees the stage / publishes the row.  (The
//            tensor-core CG at f <= 112 fuses the two: one N=Ng+16 MMA, the ratings written into
//            feature column Ng of the panel by the gather warp once its rows have landed.)
//   NGATHER gather warps: take the published stages round-robin, write the rating tile (row 0 of
//            a K-major tile), arm the stage's barrier and issue one tile::gather4 per lane.
// Operand layout (one stage): 2 atoms of 64 features x KC ratings; atom a, rating k, feature chunk
// c (8 features, 16 B) sits at a*8192 + (k/8)*1024 + (k%8)*128 + ((c%8) ^ (k%8))*16, i.e. the
// canonical SWIZZLE_128B MN-major layout with LBO = 8192 (between 64-feature atoms) and
// SBO = 1024 (between 8-rating groups).  Features f..127 are zero (written once).
//
// Every wait is bounded by %globaltimer: a wait that runs out sets the status word, the kernel
// drains its own MMAs and copies, frees TMEM and returns; the host reports ALS_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "handle.h"
#include "internal.h"
#include "sweep_tc_kernel.cuh"
#include "tc.h"

namespace als {
namespace tcg {

__global__ void quantise_bf16_kernel(const float *__restrict__ Y, int64_t rows, int f, int fst,
                                     __nv_bfloat16 *__restrict__ out) {
    const int64_t total = rows * (int64_t)fst;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / fst;
        const int j = (int)(e - r * fst);
        out[e] = __float2bfloat16_rn(j < f ? Y[r * f + j] : 0.f);
    }
}

// FP8 (e4m3) copy of a factor table with one power-of-two scale per feature: d_j = 2^e_j with
// the smallest e_j that puts the column's largest magnitude at or below 448 (e4m3's largest
// finite value), so max |Y_.j| / d_j lies in (224, 448] and no value saturates; then
// q_rj = e4m3(Y_rj / d_j) (round to nearest even), rows of 128 bytes (features f..127 zero).
// Because d is a power of two, Y_u^T Y_u = D (Q_u^T Q_u) D and Y_u^T r = D Q_u^T r exactly: one
// scale per row and column of every Gram, applied when the solver reads the accumulator.
__global__ void colmax_kernel(const float *__restrict__ Y, int64_t rows, int f,
                              unsigned int *__restrict__ cmax) {
    // thread j of a block keeps column j's running maximum over the block's rows (a row's f
    // values are consecutive: coalesced), then one atomic per block and column; non-negative
    // floats order as their bit patterns, and a NaN (above +inf) surfaces as a NaN scale, whose
    // rows the solver flags as non-finite
    const int j = threadIdx.x;
    if (j >= f) return;
    unsigned int mx = 0u;
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x)
        mx = max(mx, __float_as_uint(fabsf(Y[r * f + j])));
    if (mx) atomicMax(&cmax[j], mx);
}

// The scale exponent of a column from the bit pattern of its largest magnitude.
__device__ __forceinline__ int e4m3_scale_exp(unsigned int bits) {
    if (bits == 0u) return 0;
    const int E = (int)((bits >> 23) & 0xffu) - 127;  // (subnormal maxima: E = -127)
    const unsigned int mant = bits & 0x7fffffu;
    // max = m 2^E, m in [1, 2): max / 2^(E-8) = 256 m <= 448 iff m <= 1.75
    const int e = mant <= 0x600000u ? E - 8 : E - 7;
    return e < -126 ? -126 : (e > 127 ? 127 : e);
}

__global__ void quantise_e4m3_kernel(const float *__restrict__ Y, int64_t rows, int f,
                                     const unsigned int *__restrict__ cmax,
                                     float *__restrict__ dscale, uint8_t *__restrict__ out) {
    __shared__ float inv[MAXF];
    for (int j = threadIdx.x; j < MAXF; j += blockDim.x) {
        const int e = j < f ? e4m3_scale_exp(cmax[j]) : 0;
        inv[j] = __uint_as_float((uint32_t)(127 - e) << 23);  // 2^-e (|e| <= 126: normal)
        if (blockIdx.x == 0) dscale[j] = __uint_as_float((uint32_t)(127 + e) << 23);
    }
    __syncthreads();
    const int64_t total = rows * (int64_t)(F8_ROW_BYTES / 4);  // four bytes per thread step
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total;
         w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = w / (F8_ROW_BYTES / 4);
        const int j0 = (int)(w - r * (F8_ROW_BYTES / 4)) * 4;
        uint32_t word = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int j = j0 + k;
            const float v = j < f ? Y[r * f + j] * inv[j] : 0.f;
            word |= (uint32_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3) << (8 * k);
        }
        reinterpret_cast<uint32_t *>(out)[w] = word;
    }
}

}  // namespace tcg
}  // namespace als

// ------------------------------------------------------------------------------------- host side

using namespace als;

static int tcg_solver(int solve_type) {
    switch (solve_type) {
    case ALS_SOLVE_CG_FP32: return tcg::SOLVER_CG;
    case ALS_SOLVE_CG_FP16: return tcg::SOLVER_CGTC;
    case ALS_SOLVE_LU: return tcg::SOLVER_LU;
    default: return tcg::SOLVER_CHOL;
    }
}
struct TcState {
    CUtensorMap tmap[2];   // [side]: TMA map of the side's 16- or 8-bit table (64-byte aligned)
    tcg::Geometry geo[tcg::NSOLVER];  // per solver (CG, Cholesky, LU, tensor-core CG)
    bool f8 = false;                   // FP8 (e4m3) operands instead of BF16
    __nv_bfloat16 *d_bf[2] = {nullptr, nullptr};  // [side]: table gathered by that side
    uint8_t *d_f8[2] = {nullptr, nullptr};        // [side]: FP8 table (rows of 128 bytes)
    float *d_scale[2] = {nullptr, nullptr};       // [side]: its per-feature scales [MAXF]
    unsigned int *d_cmax = nullptr;               // column maxima (bit patterns) [MAXF]
    int32_t *d_work = nullptr;                     // one row counter per bucket
    int num_sms = 0;
    cudaEvent_t ev_q[2] = {nullptr, nullptr};
};

bool tc_path_supported(int f) { return f >= 1 && f <= tcg::MAXF; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// The gather map of a BF16 table of `rows` x fst: box = 64 features (128 bytes, the swizzle
// span) x 1 row, as tile::gather4 requires; features past fst read as zero.
static bool encode_table_map(CUtensorMap *map, void *table, int64_t rows, int fst) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)fst, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)fst * sizeof(__nv_bfloat16)};
    const cuuint32_t box[2] = {64, 1};
    const cuuint32_t estride[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, table, dims, strides, box, estride,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The gather map of an FP8 table of `rows` x 128 bytes: box = 128 features (one 128-byte line,
// the swizzle span) x 1 row.
static bool encode_table_map_f8(CUtensorMap *map, void *table, int64_t rows) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)tcg::F8_ROW_BYTES, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)tcg::F8_ROW_BYTES};
    const cuuint32_t box[2] = {(cuuint32_t)tcg::F8_ROW_BYTES, 1};
    const cuuint32_t estride[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, table, dims, strides, box, estride,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

als_status tc_prepare(als_handle *h, std::string *why) {
    if (!tc_path_supported(h->f)) {
        *why = "tensor-core path supports f in 1..128";
        return ALS_ERR_UNSUPPORTED;
    }
    int dev = 0, major = 0, minor = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (major != 10) {
        *why = "tensor-core path needs a Blackwell (sm_10x) GPU, found sm_" +
               std::to_string(major) + std::to_string(minor);
        return ALS_ERR_UNSUPPORTED;
    }
    TcState *t = new TcState();
    h->tc = t;
    t->f8 = h->precision == ALS_PREC_FP8;
    size_t smem_max = 0;
    for (int sv = 0; sv < tcg::NSOLVER; ++sv) {
        t->geo[sv] = tcg::geometry(h->f, sv, t->f8);
        smem_max = std::max(smem_max, t->geo[sv].smem);
    }
    t->num_sms = sms;
    const int64_t opp[2] = {h->n, h->m};  // side 0 gathers V rows, side 1 gathers U rows
    for (int s = 0; s < 2 && t->f8; ++s) {
        const size_t bytes = (size_t)tcg::F8_ROW_BYTES * (size_t)(opp[s] + 1);
        if (cudaMalloc(&t->d_f8[s], bytes) != cudaSuccess ||
            cudaMemset(t->d_f8[s], 0, bytes) != cudaSuccess ||
            cudaMalloc(&t->d_scale[s], sizeof(float) * tcg::MAXF) != cudaSuccess) {
            *why = "out of memory for the FP8 factor tables";
            return ALS_ERR_OUT_OF_MEMORY;
        }
        if (!encode_table_map_f8(&t->tmap[s], t->d_f8[s], opp[s] + 1)) {
            *why = "cuTensorMapEncodeTiled failed for the FP8 table";
            return ALS_ERR_CUDA;
        }
    }
    if (t->f8 && cudaMalloc(&t->d_cmax, sizeof(unsigned int) * tcg::MAXF) != cudaSuccess) {
        *why = "out of memory";
        return ALS_ERR_OUT_OF_MEMORY;
    }
    for (int s = 0; s < 2 && !t->f8; ++s) {
        const size_t bytes = sizeof(__nv_bfloat16) * (size_t)(opp[s] + 1) * t->geo[0].fst;
        if (cudaMalloc(&t->d_bf[s], bytes) != cudaSuccess ||
            cudaMemset(t->d_bf[s], 0, bytes) != cudaSuccess) {
            *why = "out of memory for the BF16 factor tables";
            return ALS_ERR_OUT_OF_MEMORY;
        }
        if (!encode_table_map(&t->tmap[s], t->d_bf[s], opp[s] + 1, t->geo[0].fst)) {
            *why = "cuTensorMapEncodeTiled failed for the BF16 table";
            return ALS_ERR_CUDA;
        }
    }
    if (cudaMalloc(&t->d_work, sizeof(int32_t) * 8) != cudaSuccess) {
        *why = "out of memory";
        return ALS_ERR_OUT_OF_MEMORY;
    }
    for (auto &e : t->ev_q) cudaEventCreate(&e);
    // sets every solver variant's shared-memory limit, which also loads them now, so no launch
    // inside a timed region (the autotuner's) loads a module
    cudaError_t e;
    switch (t->geo[0].fp) {
    case 32: e = t->f8 ? tcg::configure_32_e4m3(smem_max) : tcg::configure_32(smem_max); break;
    case 64: e = t->f8 ? tcg::configure_64_e4m3(smem_max) : tcg::configure_64(smem_max); break;
    case 112: e = t->f8 ? tcg::configure_112_e4m3(smem_max) : tcg::configure_112(smem_max); break;
    default: e = t->f8 ? tcg::configure_128_e4m3(smem_max) : tcg::configure_128(smem_max); break;
    }
    if (e != cudaSuccess) {
        *why = std::string("configuring the tcgen05 sweep kernels (shared-memory limit, register "
                           "split): ") + cudaGetErrorString(e);
        return ALS_ERR_CUDA;
    }
    return ALS_OK;
}

void tc_release(als_handle *h) {
    TcState *t = h->tc;
    if (!t) return;
    for (auto p : t->d_bf)
        if (p) cudaFree(p);
    for (auto p : t->d_f8)
        if (p) cudaFree(p);
    for (auto p : t->d_scale)
        if (p) cudaFree(p);
    if (t->d_cmax) cudaFree(t->d_cmax);
    if (t->d_work) cudaFree(t->d_work);
    for (auto e : t->ev_q)
        if (e) cudaEventDestroy(e);
    delete t;
    h->tc = nullptr;
}

void tc_invalidate_graphs(als_handle *) {}

als_status tc_values_changed(als_handle *) { return ALS_OK; }

// The BF16 copy of the table a side gathers (features f..fst-1 zero, plus an all-zero last row
// that pads ragged stages).
als_status tc_quantise(als_handle *h, int side, int *launches, std::string *why) {
    TcState *t = h->tc;
    const int64_t opp = side == 0 ? h->n : h->m;
    const float *Y = side == 0 ? h->d_V : h->d_U;
    record_event(t->ev_q[0], h->stream);
    if (t->f8) {
        const int grid = (int)std::max<int64_t>(
            1, std::min<int64_t>((opp * h->f + 255) / 256, (int64_t)t->num_sms * 8));
        cudaError_t e = cudaMemsetAsync(t->d_cmax, 0, sizeof(unsigned int) * tcg::MAXF, h->stream);
        if (e == cudaSuccess) {
            const int cgrid =
                (int)std::max<int64_t>(1, std::min<int64_t>(opp, (int64_t)t->num_sms * 16));
            tcg::colmax_kernel<<<cgrid, tcg::MAXF, 0, h->stream>>>(Y, opp, h->f, t->d_cmax);
            tcg::quantise_e4m3_kernel<<<grid, 256, 0, h->stream>>>(Y, opp, h->f, t->d_cmax,
                                                                   t->d_scale[side], t->d_f8[side]);
            *launches += 2;
            e = cudaGetLastError();
        }
        record_event(t->ev_q[1], h->stream);
        if (e != cudaSuccess) {
            *why = std::string("FP8 quantise: ") + cudaGetErrorString(e);
            return ALS_ERR_CUDA;
        }
        return ALS_OK;
    }
    const int64_t total = opp * t->geo[0].fst;
    const int grid = (int)std::max<int64_t>(
        1, std::min<int64_t>((total + 255) / 256, (int64_t)t->num_sms * 8));
    tcg::quantise_bf16_kernel<<<grid, 256, 0, h->stream>>>(Y, opp, h->f, t->geo[0].fst,
                                                           t->d_bf[side]);
    ++*launches;
    record_event(t->ev_q[1], h->stream);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        *why = std::string("quantise_bf16_kernel: ") + cudaGetErrorString(e);
        return ALS_ERR_CUDA;
    }
    return ALS_OK;
}

// One persistent launch over the rows order[lo..hi) of the side with the given ALS_SOLVE_*
// solver; `slot` picks the bucket's row counter.
cudaError_t tc_launch_bucket(const als_handle *h, int side, int32_t lo, int32_t hi, int solve,
                             int slot, int *launches) {
    const TcState *t = h->tc;
    cudaStream_t st = h->stream;
    const int solver = tcg_solver(solve);
    const tcg::Geometry &g = t->geo[solver];
    const int64_t opp = side == 0 ? h->n : h->m;
    cudaError_t e = cudaMemsetAsync(t->d_work + slot, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    tcg::Params p{};
    p.tmap = t->tmap[side];
    p.ptr = side == 0 ? h->d_csr_ptr : h->d_csc_ptr;
    p.idx = side == 0 ? h->d_csr_idx : h->d_csc_idx;
    p.val = side == 0 ? h->d_csr_val : h->d_csc_val;
    p.order = h->d_order[side] + lo;
    p.Ybf = t->d_bf[side];
    p.dscale = t->d_scale[side];
    p.X = side == 0 ? h->d_U : h->d_V;
    p.work = t->d_work + slot;
    p.flags = h->d_flags;
    p.nrows = hi - lo;
    p.zero_row = (int32_t)opp;
    p.f = h->f;
    p.fst = g.fst;
    p.ng = g.ng;
    p.acc_stride = g.acc_stride;
    p.tmem_cols = g.tmem_cols;
    p.nbuf = g.nbuf;
    p.nepi = g.nepi;
    p.solve = solver;
    p.cg_iters = h->cfg.cg_steps;
    p.refine_steps = h->cfg.refine_steps;
    p.lambda = h->cfg.lambda;
    p.cg_tol = h->cfg.cg_tol;
    p.cond_threshold = h->cfg.cond_threshold;
    p.wait_ns = h->wait_ns ? (unsigned long long)h->wait_ns : tcg::WAIT_NS;
    const int grid = (int)std::min<int64_t>(p.nrows, t->num_sms);
    if (grid <= 0) return cudaSuccess;
    switch (g.fp) {
    case 32: t->f8 ? tcg::launch_32_e4m3(p, g, grid, st) : tcg::launch_32(p, g, grid, st); break;
    case 64: t->f8 ? tcg::launch_64_e4m3(p, g, grid, st) : tcg::launch_64(p, g, grid, st); break;
    case 112:
        t->f8 ? tcg::launch_112_e4m3(p, g, grid, st) : tcg::launch_112(p, g, grid, st);
        break;
    default:
        t->f8 ? tcg::launch_128_e4m3(p, g, grid, st) : tcg::launch_128(p, g, grid, st);
        break;
    }
    ++*launches;
    return cudaGetLastError();
}
