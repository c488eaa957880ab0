// sweep_tc_kernel.cuh — the tcgen05 half-sweep kernel template (see sweep_tc.cu for the
// design); instantiated per padded size by sweep_tc_fp*.cu.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "regsolve.cuh"
#include "solvers.cuh"

namespace als {
namespace tcg {

constexpr int KC = 64;                       // ratings per stage
constexpr int MAX_NSTAGE = 16;
// CG at FP = 64, 112 and 128 quad-blocks its rows (cg_quad): half of a row's values in
// registers, half in shared memory (2 FP/16 slots of CGQ_SLOT float4 a group), so four groups
// (FP = 64, 112) or three (FP = 128, as many as its accumulators) fit an SM.
__host__ __device__ constexpr bool cg_quad_rows(int solver, int fp) {
    return solver == 0 && fp >= 64;
}
__host__ __device__ constexpr int cgq_floats(int fp) { return 2 * (fp / 16) * 130 * 4; }
constexpr int ATOM_BYTES = 1024;             // 8 ratings x 128 B
constexpr int ATOM_STRIDE = (KC / 8) * ATOM_BYTES;  // 8192: LBO between 64-feature atoms
constexpr int TILE_BYTES = 2 * ATOM_STRIDE;  // 128 features
constexpr int R_BYTES = 2 * ATOM_BYTES;      // K-major rating tile, N = 16 rows x 64 ratings
constexpr int STAGE_BYTES = TILE_BYTES + R_BYTES;
// FP8 stages: one 128-feature atom of KC ratings (8 KB) and the rating tile
constexpr int TILE_BYTES_F8 = ATOM_STRIDE;
constexpr int STAGE_BYTES_F8 = TILE_BYTES_F8 + R_BYTES;
__host__ __device__ constexpr int stage_bytes(bool f8) { return f8 ? STAGE_BYTES_F8 : STAGE_BYTES; }
__host__ __device__ constexpr int tile_bytes(bool f8) { return f8 ? TILE_BYTES_F8 : TILE_BYTES; }
constexpr int MAXF = 128;
constexpr int MAX_NBUF = 4;
// Producer metadata ring: each stage's column ids and ratings are copied into shared memory MD
// stages ahead of its gathers (MR slots, MR > MD), so their HBM latency never stalls the gathers.
constexpr int MD = 12;
constexpr int MR = 16;
// Warp roles: the solver warpgroups come first (group g = warps 4g..4g+3, so warp w reads TMEM
// lanes 32 (w % 4) ..), then the producer (metadata look-ahead), the MMA issuer and the gather
// warps.  One warp issues a tile::gather4 only every ~90 cycles, so the stages go round-robin to
// several gather warps, which also write each stage's rating tile and arm its barrier.
constexpr int MAX_NGATHER = 6;
constexpr int MRING_BYTES = MR * KC * 8 + MR * 16;   // column ids, ratings, Meta per slot
// SOLVER_CGTC: CG on the Gram rounded to binary16's significand (the reference's FP16-Gram CG),
// its products A p run on the tensor core from the accumulator left in TMEM.
enum { SOLVER_CG = 0, SOLVER_CHOL = 1, SOLVER_LU = 2, SOLVER_CGTC = 3 };
constexpr int NSOLVER = 4;
// The tensor-core CG's operand tile for p: K = FP rows (the Gram's columns) x N = 16 columns of
// f16, no swizzle, core matrices of 8 columns x 8 rows (16 bytes) at (k/8) * 256 + (n/8) * 128;
// columns 0 and 1 hold p's high and low f16 parts, the others stay zero.
__host__ __device__ constexpr int cgtc_tile_floats(int fp) { return (fp / 8) * 64 + 64; }

// TMEM accumulators (ng + 16 columns: four fit in 512 columns unless FP = 128, whose rows have
// ng = 128: two at a 256-column stride, or three at 160 for the quad-blocked CG, whose stride
// need not be a power of two) and solver groups: CG and LU read their row out of TMEM into
// registers at once and release the buffer, so the MMA fills the next row while they solve;
// their register-resident rows allow two groups per SM.  A Cholesky group keeps its buffer until
// refinement has re-read A, and its factor lives in shared memory: one group per buffer; so does
// the quad-blocked CG (half of each row in shared memory), and the tensor-core CG, whose products
// read A from the buffer until the solve ends.
__host__ __device__ constexpr int nbuf_of(int solver, int fp) {
    return fp != 128 ? 4 : cg_quad_rows(solver, fp) ? 3 : 2;
}
__host__ __device__ constexpr int acc_stride_of(int solver, int fp, int ng) {
    return ng + 16 <= 128 ? 128 : nbuf_of(solver, fp) == 3 ? 160 : 256;
}
__host__ __device__ constexpr int nepi_of(int solver, int fp) {
    return solver == 1 || solver == 3 || cg_quad_rows(solver, fp) ? nbuf_of(solver, fp)
                                                                   : nbuf_of(solver, fp) / 2;
}
// Gather warps: one warp issues a tile::gather4 only every ~90 cycles, so the gathers want several
// warps, up to about six (ten made the tensor-core CG slower: the SM's gathers are then saturated
// and the extra warps only add hand-offs).  A launch's registers are shared out per four warps, so
// above 640 threads a thread keeps 80 and at 640 it keeps 96.  The tensor-core CG (about 60 a
// thread) takes six gather warps; the Cholesky factor, LU and the four-group quad-blocked CG (84
// to 96 a thread) two.  The three-group quad-blocked CG at FP = 128 splits the registers
// (setmaxnreg): launched with six gather warps at 96 a thread, its solver warpgroups take 128 and
// the two service warpgroups (producer, MMA issuer, gather warps) give theirs back down to
// SERVICE_REGS, the sum being exactly what the launch holds (launch_regs_of x threads).  (The same
// split for the four groups at FP = 64 and 112, 80 a thread at launch, made their light rows,
// bound by the solves, 1-8% slower.)
__host__ __device__ constexpr bool regsplit_of(int solver, int fp) {
    return cg_quad_rows(solver, fp) && fp == 128;
}
__host__ __device__ constexpr int ngather_of(int solver, int fp) {
    return solver == 3 || regsplit_of(solver, fp) ? 6 : 2;
}
__host__ __device__ constexpr int nthreads_of(int solver, int fp) {
    return 128 * nepi_of(solver, fp) + 32 * (2 + ngather_of(solver, fp));
}
constexpr int SERVICE_REGS = 48;
__host__ __device__ constexpr int solver_regs_of(int solver, int fp) { return fp == 128 ? 128 : 96; }
__host__ __device__ constexpr int launch_regs_of(int solver, int fp) {
    return (solver_regs_of(solver, fp) * 128 * nepi_of(solver, fp) +
            SERVICE_REGS * 32 * (2 + ngather_of(solver, fp))) /
           nthreads_of(solver, fp);
}

// Bound of every spin-wait: the role waits use Params::wait_ns (the handle's limit, by default
// WAIT_NS); the drains at the end of a CTA (in-flight MMAs, gathers, product chains) always get
// WAIT_NS, so that a CTA that gave up still lets every copy it issued land before it exits.
constexpr unsigned long long WAIT_NS = 10ull * 1000 * 1000 * 1000;  // 10 s

struct Meta {  // per stage / per accumulator
    int32_t row;    // -1 = end of work
    int32_t cnt;    // ratings in this stage
    int32_t flags;  // 1 = first stage of the row, 2 = last stage of the row
    int32_t nu;     // ratings of the row
};

struct Params {
    // 2-D map of the BF16 table (fst features x n_opp + 1 rows), box 64 features x 1 row,
    // 128-byte swizzle: the producer's tile::gather4 loads read 4 rows of it per instruction
    CUtensorMap tmap;
    const int32_t *ptr, *idx, *order;
    const float *val;
    const __nv_bfloat16 *Ybf;  // (n_opp + 1) x fst, row n_opp all zero
    const float *dscale;       // FP8 operands: the table's per-feature scales (powers of two)
    float *X;                  // this side's FP32 factors (in: CG warm start, out: solution)
    int32_t *work;             // atomic row counter (zeroed before the launch)
    int32_t *flags;            // [0] flagged rows, [1] FP64-refined rows, [2] timeouts
    int32_t nrows, zero_row, f, fst, ng, acc_stride, tmem_cols, nbuf, nepi, solve, cg_iters;
    int32_t refine_steps;
    float lambda, cg_tol, cond_threshold;
    unsigned long long wait_ns;  // bound of the role waits (the drains keep WAIT_NS)
};

// Per-warpgroup shared scratch: L rows (or the FP32 Gram for the shared-memory LU) unless the
// solver is CG, then two vectors, the reduction ring and the shared-memory solvers' vectors.
template <int FP>
struct GroupSmem {
    static constexpr int LS = FP + 4;
    static constexpr size_t ls_floats = (size_t)FP * LS;
    static constexpr size_t floats = ls_floats + 2 * FP + 16 + 5 * 128 + 64;
};
template <int FP, int SOLVER>
struct GroupLayout {
    // Cholesky: packed L then the 8 x 8 diagonal-block inverses; LU: the square Gram (+ unused)
    static constexpr size_t ls_floats = SOLVER == 0   ? (cg_quad_rows(SOLVER, FP) ? cgq_floats(FP) : 0)
                                        : SOLVER == 1 ? TriLayout<FP>::floats + 8 * FP
                                        : SOLVER == 3 ? cgtc_tile_floats(FP)
                                                      : GroupSmem<FP>::ls_floats + 8 * FP;
    // (the tensor-core CG's groups start on 128-byte boundaries: its tile is an MMA operand;
    // the quad-blocked CG needs no vectors past the reduction ring)
    static constexpr size_t floats =
        SOLVER == 3 ? (ls_floats + 2 * FP + 16 + 5 * 128 + 64 + 31) / 32 * 32
        : cg_quad_rows(SOLVER, FP) ? ls_floats + 2 * FP + 32
                                   : ls_floats + 2 * FP + 16 + 5 * 128 + 64;
};

struct Geometry {
    int fp, fst, ng, acc_stride, tmem_cols, nbuf, nepi, nthreads;
    size_t smem;
};
// FP8 (e4m3) operands: each gathered factor row is one 128-byte line (features 0..127, one byte
// each: the table's row pitch), so a stage's panel is one 128-feature swizzle atom of KC
// ratings, and one MMA covers K = 32 ratings.  The per-feature scales of the table sit in shared
// memory behind the solver groups' scratch.
constexpr int F8_ROW_BYTES = 128;
constexpr int F8_K = 32;

__host__ __device__ inline int gs_of(int f) { return (f + 1) % 2 ? f + 1 : f + 2; }

inline int fp_of(int f) {
    const int r = (f + 15) / 16 * 16;
    return r <= 32 ? 32 : r <= 64 ? 64 : r <= 112 ? 112 : 128;
}

__host__ __device__ constexpr size_t group_floats(int fp, int solver) {
    return solver == 0   ? (cg_quad_rows(solver, fp)
                                ? (size_t)cgq_floats(fp) + 2 * (size_t)fp + 32
                                : 2 * (size_t)fp + 16 + 5 * 128 + 64)
           : solver == 1 ? 32 * (size_t)(fp / 8) * (fp / 8 + 1) + 4 * (size_t)fp + 8 * (size_t)fp +
                               2 * (size_t)fp + 16 + 5 * 128 + 64
           : solver == 3 ? ((size_t)cgtc_tile_floats(fp) + 2 * (size_t)fp + 16 + 5 * 128 + 64 + 31) /
                               32 * 32
                         : (size_t)fp * (fp + 4) + 8 * (size_t)fp + 2 * (size_t)fp + 16 + 5 * 128 + 64;
}
// Stage-ring depth: as many stages as the shared memory left beside the solver groups' scratch,
// the metadata ring and the barriers holds (at most MAX_NSTAGE).  On Gram-bound rows a stage's
// life (gather issue, the rows' L2 round trip, the MMAs, the commit that frees the slot) is
// long against its MMA time, so the stages in flight set the rate; on solve-bound rows more
// stages cost nothing (one CTA per SM).  FP8 stages are 10 KB instead of 18 KB.
constexpr size_t SMEM_BUDGET = 232448 - 2048;  // the opt-in limit per CTA, less alignment slack
__host__ __device__ constexpr int nstage_fit(int solver, int fp, bool f8) {
    return (int)((SMEM_BUDGET - sizeof(float) * group_floats(fp, solver) * nepi_of(solver, fp) -
                  (size_t)MRING_BYTES - 1024 - (f8 ? sizeof(float) * MAXF : 0)) /
                 (size_t)stage_bytes(f8));
}
__host__ __device__ constexpr int nstage_of(int solver, int fp, bool f8) {
    return nstage_fit(solver, fp, f8) > MAX_NSTAGE ? MAX_NSTAGE : nstage_fit(solver, fp, f8);
}

inline Geometry geometry(int f, int solver, bool f8 = false) {
    Geometry g;
    g.fp = fp_of(f);
    g.fst = (f + 7) / 8 * 8;
    g.ng = (f + 15) / 16 * 16;
    g.acc_stride = acc_stride_of(solver, g.fp, g.ng);
    // Accumulators rotate over the groups (group g takes rows g, g + nepi, ...; row k lands in
    // buffer k % nbuf); nbuf_of agrees with ng + 16 for every f of that padded size.
    g.nbuf = nbuf_of(solver, g.fp);
    g.nepi = nepi_of(solver, g.fp);
    // the allocation is a power of two of at least 32 columns (three 160-column buffers: 512)
    int cols = 32;
    while (cols < g.nbuf * g.acc_stride) cols *= 2;
    g.tmem_cols = cols;
    g.nthreads = nthreads_of(solver, g.fp);
    const int ns = nstage_of(solver, g.fp, f8);
    size_t bytes = (size_t)ns * stage_bytes(f8);                     // operand ring
    bytes += sizeof(float) * group_floats(g.fp, solver) * g.nepi;    // per-group scratch
    if (f8) bytes += sizeof(float) * MAXF;                            // per-feature scales
    bytes += MRING_BYTES;                                            // metadata ring
    bytes += 1024;                                                   // metas, barriers, scalars
    g.smem = bytes + 1024;                                           // 1024-B alignment slack
    return g;
}

// ---------------------------------------------------------------------------------- PTX helpers

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar)
                 : "memory");
}
// A try suspends the thread until the phase completes (the hardware wakes it then) or
// MBAR_SUSPEND_NS pass, so a waiting warp takes no issue slots from the warps that work.
constexpr uint32_t MBAR_SUSPEND_NS = 20000;
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(MBAR_SUSPEND_NS)
        : "memory");
    return ok != 0;
}
// Bounded wait (`limit` ns, checked every 16 failed tries, i.e. within ~0.3 ms); false on
// timeout or (when abort != nullptr) once another role aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort,
                                          unsigned long long limit) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    for (uint32_t i = 0;; ++i) {
        if (mbar_try(bar, parity)) return true;
        if ((i & 15) == 15) {
            if (abort && *abort) return false;
            if (now_ns() - t0 > limit) return false;
        }
    }
}
// Warp-uniform wait: lane 0 waits, the outcome is broadcast (no lane can diverge on a timeout),
// and __syncwarp orders every lane's later memory accesses after lane 0's acquire.
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity, volatile int *abort,
                                               unsigned long long limit) {
    int ok = 0;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, abort, limit) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    return ok != 0;
}
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// 4-byte asynchronous global -> shared copy (the ratings of a stage have no alignment), with an
// L2 cache policy: the column ids and ratings stream through once per half-sweep (evict first),
// so they do not push the gathered factor table (evict last) out of L2.
__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src, uint64_t policy) {
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;" ::"r"(dst),
                 "l"(src), "l"(policy)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Arrive on `bar` and add `bytes` to the transaction count its current phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
// TMA gather: rows r0..r3 of the 2-D tensor map, features x .. x+63 (x * 2 bytes a multiple of
// 16), land as four consecutive 128-byte rows at dst (128-byte swizzle by address); the bytes
// count against `bar`'s transaction count.  `policy` is an L2 cache policy: the gathered table is
// re-read by every SM for the whole half-sweep.
__device__ __forceinline__ void tma_gather4(uint32_t dst, const CUtensorMap *tmap, int x, int r0,
                                            int r1, int r2, int r3, uint32_t bar,
                                            uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
        ".L2::cache_hint [%0], [%1, {%2, %3, %4, %5, %6}], [%7], %8;" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(bar),
        "l"(policy)
        : "memory");
}
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor, SWIZZLE_128B, sm_100 layout (version 1 at bits 46-47).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D F32, A/B BF16, majors, N, M.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
           ((b_mn ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Instruction descriptor of tcgen05.mma kind::f8f6f4: D F32, A/B E4M3 (format 0), majors, N, M.
__host__ __device__ constexpr uint32_t idesc_e4m3(int M, int N, bool a_mn, bool b_mn) {
    return (1u << 4) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_e4m3(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}
// Shared-memory descriptor without swizzle (canonical layout of 8-row x 16-byte core matrices):
// lbo = bytes between core matrices adjacent along K, sbo = along M/N.
__device__ __forceinline__ uint64_t sdesc_plain(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// Instruction descriptor of tcgen05.mma kind::f16 with F16 A (from TMEM) and B (K-major), F32 D.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D (TMEM) (+)= A (TMEM, M lanes x K f16 packed two to a column) x B (shared memory).
__device__ __forceinline__ void mma_f16_tmem_a(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc,
                                               uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
        "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// registers -> TMEM (8 columns of this warp's 32 lanes); the caller waits with tmem_wait_st.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t *v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]),
                 "r"(v[7])
                 : "memory");
}
// 2^e as a float for |e| <= 126 (exact).
__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((uint32_t)(127 + e) << 23); }
// floor(log2(x)) of a positive normal float; 0 for zero.
__device__ __forceinline__ int exp2_of(float x) {
    return x > 0.f ? (int)((__float_as_uint(x) >> 23) & 0xffu) - 127 : 0;
}

__device__ __forceinline__ void tmem_wait_st() {
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float &a, float &b) {
    asm volatile(
        "{\n\ttcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a), "=f"(b)
        : "r"(taddr)
        : "memory");
}

// TMEM -> registers.  The load and its wait::ld sit in one asm block, so the outputs are only
// defined once the data has arrived.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "{\n\ttcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// TMEM -> registers: the Gram row's FP columns and b (column bcol, one more 1-column load) with
// one wait::ld per block of at most 64 columns (larger blocks put the row in local memory);
// loads and their wait share one asm block, so no output is read before it arrived.
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, uint32_t bcol, float (&a)[32], float &b) {
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%32}, [%34];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a[0]), "=f"(a[1]), "=f"(a[2]), "=f"(a[3]), "=f"(a[4]), "=f"(a[5]), "=f"(a[6]), "=f"(a[7]), "=f"(a[8]), "=f"(a[9]), "=f"(a[10]), "=f"(a[11]), "=f"(a[12]), "=f"(a[13]), "=f"(a[14]), "=f"(a[15]), "=f"(a[16]), "=f"(a[17]), "=f"(a[18]), "=f"(a[19]), "=f"(a[20]), "=f"(a[21]), "=f"(a[22]), "=f"(a[23]), "=f"(a[24]), "=f"(a[25]), "=f"(a[26]), "=f"(a[27]), "=f"(a[28]), "=f"(a[29]), "=f"(a[30]), "=f"(a[31]), "=f"(b)
        : "r"(taddr + 0u), "r"(taddr + bcol)
        : "memory");
}
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, uint32_t bcol, float (&a)[64], float &b) {
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%65];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%66];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%64}, [%67];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a[0]), "=f"(a[1]), "=f"(a[2]), "=f"(a[3]), "=f"(a[4]), "=f"(a[5]), "=f"(a[6]), "=f"(a[7]), "=f"(a[8]), "=f"(a[9]), "=f"(a[10]), "=f"(a[11]), "=f"(a[12]), "=f"(a[13]), "=f"(a[14]), "=f"(a[15]), "=f"(a[16]), "=f"(a[17]), "=f"(a[18]), "=f"(a[19]), "=f"(a[20]), "=f"(a[21]), "=f"(a[22]), "=f"(a[23]), "=f"(a[24]), "=f"(a[25]), "=f"(a[26]), "=f"(a[27]), "=f"(a[28]), "=f"(a[29]), "=f"(a[30]), "=f"(a[31]), "=f"(a[32]), "=f"(a[33]), "=f"(a[34]), "=f"(a[35]), "=f"(a[36]), "=f"(a[37]), "=f"(a[38]), "=f"(a[39]), "=f"(a[40]), "=f"(a[41]), "=f"(a[42]), "=f"(a[43]), "=f"(a[44]), "=f"(a[45]), "=f"(a[46]), "=f"(a[47]), "=f"(a[48]), "=f"(a[49]), "=f"(a[50]), "=f"(a[51]), "=f"(a[52]), "=f"(a[53]), "=f"(a[54]), "=f"(a[55]), "=f"(a[56]), "=f"(a[57]), "=f"(a[58]), "=f"(a[59]), "=f"(a[60]), "=f"(a[61]), "=f"(a[62]), "=f"(a[63]), "=f"(b)
        : "r"(taddr + 0u), "r"(taddr + 32u), "r"(taddr + bcol)
        : "memory");
}
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, uint32_t bcol, float (&a)[112], float &b) {
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a[0]), "=f"(a[1]), "=f"(a[2]), "=f"(a[3]), "=f"(a[4]), "=f"(a[5]), "=f"(a[6]), "=f"(a[7]), "=f"(a[8]), "=f"(a[9]), "=f"(a[10]), "=f"(a[11]), "=f"(a[12]), "=f"(a[13]), "=f"(a[14]), "=f"(a[15]), "=f"(a[16]), "=f"(a[17]), "=f"(a[18]), "=f"(a[19]), "=f"(a[20]), "=f"(a[21]), "=f"(a[22]), "=f"(a[23]), "=f"(a[24]), "=f"(a[25]), "=f"(a[26]), "=f"(a[27]), "=f"(a[28]), "=f"(a[29]), "=f"(a[30]), "=f"(a[31]), "=f"(a[32]), "=f"(a[33]), "=f"(a[34]), "=f"(a[35]), "=f"(a[36]), "=f"(a[37]), "=f"(a[38]), "=f"(a[39]), "=f"(a[40]), "=f"(a[41]), "=f"(a[42]), "=f"(a[43]), "=f"(a[44]), "=f"(a[45]), "=f"(a[46]), "=f"(a[47]), "=f"(a[48]), "=f"(a[49]), "=f"(a[50]), "=f"(a[51]), "=f"(a[52]), "=f"(a[53]), "=f"(a[54]), "=f"(a[55]), "=f"(a[56]), "=f"(a[57]), "=f"(a[58]), "=f"(a[59]), "=f"(a[60]), "=f"(a[61]), "=f"(a[62]), "=f"(a[63])
        : "r"(taddr + 0u), "r"(taddr + 32u)
        : "memory");
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%49];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47}, [%50];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%48}, [%51];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a[64]), "=f"(a[65]), "=f"(a[66]), "=f"(a[67]), "=f"(a[68]), "=f"(a[69]), "=f"(a[70]), "=f"(a[71]), "=f"(a[72]), "=f"(a[73]), "=f"(a[74]), "=f"(a[75]), "=f"(a[76]), "=f"(a[77]), "=f"(a[78]), "=f"(a[79]), "=f"(a[80]), "=f"(a[81]), "=f"(a[82]), "=f"(a[83]), "=f"(a[84]), "=f"(a[85]), "=f"(a[86]), "=f"(a[87]), "=f"(a[88]), "=f"(a[89]), "=f"(a[90]), "=f"(a[91]), "=f"(a[92]), "=f"(a[93]), "=f"(a[94]), "=f"(a[95]), "=f"(a[96]), "=f"(a[97]), "=f"(a[98]), "=f"(a[99]), "=f"(a[100]), "=f"(a[101]), "=f"(a[102]), "=f"(a[103]), "=f"(a[104]), "=f"(a[105]), "=f"(a[106]), "=f"(a[107]), "=f"(a[108]), "=f"(a[109]), "=f"(a[110]), "=f"(a[111]), "=f"(b)
        : "r"(taddr + 64u), "r"(taddr + 96u), "r"(taddr + bcol)
        : "memory");
}
__device__ __forceinline__ void tmem_ld_row(uint32_t taddr, uint32_t bcol, float (&a)[128], float &b) {
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%64];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%65];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a[0]), "=f"(a[1]), "=f"(a[2]), "=f"(a[3]), "=f"(a[4]), "=f"(a[5]), "=f"(a[6]), "=f"(a[7]), "=f"(a[8]), "=f"(a[9]), "=f"(a[10]), "=f"(a[11]), "=f"(a[12]), "=f"(a[13]), "=f"(a[14]), "=f"(a[15]), "=f"(a[16]), "=f"(a[17]), "=f"(a[18]), "=f"(a[19]), "=f"(a[20]), "=f"(a[21]), "=f"(a[22]), "=f"(a[23]), "=f"(a[24]), "=f"(a[25]), "=f"(a[26]), "=f"(a[27]), "=f"(a[28]), "=f"(a[29]), "=f"(a[30]), "=f"(a[31]), "=f"(a[32]), "=f"(a[33]), "=f"(a[34]), "=f"(a[35]), "=f"(a[36]), "=f"(a[37]), "=f"(a[38]), "=f"(a[39]), "=f"(a[40]), "=f"(a[41]), "=f"(a[42]), "=f"(a[43]), "=f"(a[44]), "=f"(a[45]), "=f"(a[46]), "=f"(a[47]), "=f"(a[48]), "=f"(a[49]), "=f"(a[50]), "=f"(a[51]), "=f"(a[52]), "=f"(a[53]), "=f"(a[54]), "=f"(a[55]), "=f"(a[56]), "=f"(a[57]), "=f"(a[58]), "=f"(a[59]), "=f"(a[60]), "=f"(a[61]), "=f"(a[62]), "=f"(a[63])
        : "r"(taddr + 0u), "r"(taddr + 32u)
        : "memory");
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%65];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%66];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%64}, [%67];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=f"(a[64]), "=f"(a[65]), "=f"(a[66]), "=f"(a[67]), "=f"(a[68]), "=f"(a[69]), "=f"(a[70]), "=f"(a[71]), "=f"(a[72]), "=f"(a[73]), "=f"(a[74]), "=f"(a[75]), "=f"(a[76]), "=f"(a[77]), "=f"(a[78]), "=f"(a[79]), "=f"(a[80]), "=f"(a[81]), "=f"(a[82]), "=f"(a[83]), "=f"(a[84]), "=f"(a[85]), "=f"(a[86]), "=f"(a[87]), "=f"(a[88]), "=f"(a[89]), "=f"(a[90]), "=f"(a[91]), "=f"(a[92]), "=f"(a[93]), "=f"(a[94]), "=f"(a[95]), "=f"(a[96]), "=f"(a[97]), "=f"(a[98]), "=f"(a[99]), "=f"(a[100]), "=f"(a[101]), "=f"(a[102]), "=f"(a[103]), "=f"(a[104]), "=f"(a[105]), "=f"(a[106]), "=f"(a[107]), "=f"(a[108]), "=f"(a[109]), "=f"(a[110]), "=f"(a[111]), "=f"(a[112]), "=f"(a[113]), "=f"(a[114]), "=f"(a[115]), "=f"(a[116]), "=f"(a[117]), "=f"(a[118]), "=f"(a[119]), "=f"(a[120]), "=f"(a[121]), "=f"(a[122]), "=f"(a[123]), "=f"(a[124]), "=f"(a[125]), "=f"(a[126]), "=f"(a[127]), "=f"(b)
        : "r"(taddr + 64u), "r"(taddr + 96u), "r"(taddr + bcol)
        : "memory");
}

// ------------------------------------------------------------------------------------- kernels

// sum_j D[i][j] x_j re-read from TMEM in 16-column chunks (FP64 products and sums when WIDE)
template <int FP, bool WIDE>
__device__ __forceinline__ double tmem_rowdot(uint32_t tb, int ng, const float *xs) {
    double acc = 0.0;
    float accf = 0.f;
#pragma unroll
    for (int c = 0; c < FP; c += 16) {
        if (c < ng) {
            float v[16];
            tmem_ld16(tb + c, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                if (WIDE)
                    acc = fma((double)v[j], (double)xs[c + j], acc);
                else
                    accf = fmaf(v[j], xs[c + j], accf);
            }
        }
    }
    return WIDE ? acc : (double)accf;
}

// A group's serial work (the waits on its barriers, the tensor-core CG's MMA chains, the
// Cholesky factor's diagonal blocks and triangular solves) runs on warp g % 4 of group g: warps
// are spread over the SM's four sub-partitions by warp index % 4, so the groups' leaders sit on
// four different schedulers instead of all on the first.
__device__ __forceinline__ int lead_of(int g) { return 32 * (g & 3); }
__device__ __forceinline__ int lane_of(int i) { return i & 31; }

// The tensor-core CG's per-group state that outlives a row: the phase of its product barrier, and
// whether the leader's last commit has not been seen to complete (drained before the CTA ends).
struct CgTcState {
    uint32_t phase = 0;       // product calls so far (the barrier phase each one waits for)
    uint32_t committed = 0;   // the phase of the leader's last commit
    bool unconfirmed = false;
};

// CG of cumf_als_cg/cg.cu:236-300 (the FP16-Gram variant: the regularised Gram held to binary16's
// 11-bit significand, vectors and sums in FP32; same recurrences, warm start, step cap and
// r'r < tol exit as the FP32 CG, cg.cu:37-232) with every product A p on the tensor core.  The
// regularised Gram, scaled by 2^-ka so its largest entry (on the diagonal) stays below 2^15, is
// rounded to binary16 and written back into its accumulator packed two to a column (columns
// [0, ng/2) of the buffer, read as the f16 A operand, M = 128 lanes x K = ng); p, scaled by a power
// of two from the residual norm, goes to the group's operand tile as two f16 columns, p = hi + lo
// (22 significant bits); one M = 128 x N = 16 x K = ng chain (ng / 16 MMAs) per product writes
// A [hi lo] to columns [ng, ng + 16) (b was read from there before), and thread i sums its two
// values and undoes both scales (powers of two: exact).  The scaling keeps binary16's 11-bit
// rounding but not its exponent range: no entry overflows or loses bits to subnormals.  The
// group's leader (et == lead) issues the chain and commits it to `bar`; every warp waits on the
// barrier itself.  Thread i holds x_i, r_i, p_i; padded rows (i >= f) keep zeros.
template <int FP>
__device__ float cg_tc(const Params &p, uint32_t tcol, uint32_t trow, float bi, float xi, int i,
                       int et, int lead, __half *Bh, int ka, uint32_t bar, CgTcState &st,
                       float *red, volatile int *abort, const GroupSync &gs, bool &ok) {
    int slot = 0;
    const int ng = p.ng;
    const uint32_t idesc = idesc_f16(128, 16);
    const uint32_t bt = smem_u32(Bh);
    const int bo = (i >> 3) * 128 + (i & 7);  // (k = i, n = 0) in the tile; n = 1 is 8 halves on
    auto product = [&](float v, int kp) -> float {  // v scaled by 2^kp before the split
        if (i < ng) {
            const float ps = v * pow2f(kp);
            const __half hi = __float2half_rn(ps);
            Bh[bo] = hi;
            Bh[bo + 8] = __float2half_rn(ps - __half2float(hi));
        }
        fence_async_smem();  // the tile is read by the tensor core (async proxy)
        tc_fence_before();   // the previous product's tcgen05.ld precede the next MMA
        gs.sync();
        if (et == lead && !*abort) {
            tc_fence_after();
            for (int kk = 0; kk < ng / 16; ++kk)
                mma_f16_tmem_a(tcol + (uint32_t)ng, tcol + 8u * kk,
                               sdesc_plain(bt + 512u * kk, 256, 128), idesc, kk > 0 ? 1u : 0u);
            mma_commit(bar);
            st.unconfirmed = true;
            st.committed = st.phase;
        }
        const bool done = mbar_wait_warp(bar, st.phase & 1, abort, p.wait_ns);
        if (done) {
            if (et == lead) st.unconfirmed = false;
        } else {
            ok = false;
            if ((threadIdx.x & 31) == 0) *abort = 1;
        }
        ++st.phase;
        tc_fence_after();
        float d0, d1;
        tmem_ld2(trow + (uint32_t)ng, d0, d1);
        return (d0 + d1) * pow2f(ka - kp);
    };
    // the warm start is O(1) (factor values); later products scale p by its residual's RMS
    auto scale_of = [&](float rs) -> int {
        const int e = exp2_of(sqrtf(rs / (float)ng));
        return e > 60 ? -60 : e < -60 ? 60 : -e;
    };
    float r = bi - product(xi, 0);
    float pv = r;
    float rsold = gsum128(r * r, red, slot, gs);
    for (int it = 0; it < p.cg_iters; ++it) {
        const float ap = product(pv, scale_of(rsold));
        const float pap = gsum128(pv * ap, red, slot, gs);
        if (!(pap > 0.f)) break;
        const float alpha = rsold / pap;
        xi = fmaf(alpha, pv, xi);
        r = fmaf(-alpha, ap, r);
        const float rsnew = gsum128(r * r, red, slot, gs);
        if (rsnew < p.cg_tol) break;
        const float beta = rsnew / rsold;
        rsold = rsnew;
        pv = fmaf(beta, pv, r);
    }
    return i < p.f ? xi : 0.f;
}

// The solver warpgroup's work on one row whose Gram row i sits in TMEM at tb.
// Returns true when it released the accumulator itself (arrived on `release` once every thread
// of the group had read its row out of TMEM); otherwise the caller releases it afterwards.
// With FP8 operands (F8) the accumulator holds Q^T Q and Q^T r of the scaled table Q = Y D^-1
// (D = diag(dsc), powers of two): every value read from TMEM is multiplied back, A_ij by
// d_i d_j and b_i by d_i, which is exact.
template <int FP, int SOLVER, bool F8>
__device__ bool solve_row(const Params &p, const Meta &m, uint32_t tb, int i, int et, int g,
                          float *gsm, const GroupSync &gs, uint32_t release, float xw,
                          uint32_t mvbar, CgTcState &cst, volatile int *abort, bool &ok,
                          const float *dsc) {
    float *Ls = gsm;
    float *sv = gsm + GroupLayout<FP, SOLVER>::ls_floats;
    float *yv = sv + FP;
    float *red = yv + FP;   // reduction ring: 16 floats, 32 for the CGs' two-value sums
    float *vec = red + 16;  // 5 x 128 floats for the shared-memory solvers (not the CGs)
    const int f = p.f;
    float *xo = p.X + (int64_t)m.row * f;
    const float reg = (float)m.nu * p.lambda;  // items_cnt * lambda (als_model.cu:157-159)
    const float di = F8 && i < FP ? dsc[i] : 1.f;  // this thread's row scale (1 unless FP8)

    float bi = 0.f;
    if constexpr (SOLVER == SOLVER_CHOL) {
        float v[16];
        tmem_ld16(tb + p.ng, v);
        bi = i < f ? v[0] * di : 0.f;
    }
    int slot = 0;
    float xi = 0.f;
    bool good = true;
    bool released = false;
    if constexpr (SOLVER == SOLVER_CHOL) {
        // Cholesky (+ refinement against the TMEM copy of A).  The regularised Gram's lower
        // triangle moves to the packed shared-memory layout in 32-column chunks (a warp reads
        // only the chunks its rows reach), the group factors it and runs each pair of
        // triangular solves.
        float *Dv = Ls + TriLayout<FP>::floats;
        float *invd = vec;                                                   // 1 / L_jj
        volatile int *cflag = reinterpret_cast<volatile int *>(vec + 128);  // [0] bad, [1] wide
        const int wg = i >> 5;                                               // warp in the group
        const int len = 8 * ((i >> 3) + 1);                                  // stored columns
        float *li = Ls + tri_off(i < FP ? i : 0);
#pragma unroll
        for (int c = 0; c < FP; c += 32) {
            if (c < 32 * (wg + 1)) {  // warp-uniform: rows 32wg.. reach column 32wg + 31
                float v[32];
#pragma unroll
                for (int h = 0; h < 32; h += 16) {
                    if (c + h < FP && c + h < p.ng) {
                        tmem_ld16(tb + c + h, v + h);
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; ++j) v[h + j] = 0.f;
                    }
                }
                if constexpr (F8) {
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (c + j < FP) v[j] *= di * dsc[c + j];
                }
#pragma unroll
                for (int j = 0; j < 32; ++j)  // padded rows (i >= f): the identity
                    v[j] = c + j == i ? (i < f ? v[j] + reg : 1.f) : (i < f ? v[j] : 0.f);
                if (i < FP) {
#pragma unroll
                    for (int j = 0; j < 32 && c + j < FP; j += 4)
                        if (c + j < len)
                            *reinterpret_cast<float4 *>(li + c + j) =
                                make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                }
            }
        }
        if (i < FP) yv[i] = bi;
        if (et == 0) cflag[0] = 0;
        gs.sync();
        if (!chol_fac<FP>(et, lead_of(g), Ls, Dv, invd, gs)) cflag[0] = 1;
        gs.sync();
        good = cflag[0] == 0;
        if (good) {
            float *xb = vec + 256;  // the triangular solves' per-block results (16 floats)
            chol_solve_group<FP>(i, Ls, Dv, yv, xb, gs);
            if (wg == (g & 3)) {
                // condition estimate from the Cholesky diagonal: (max L_jj / min L_jj)^2
                float dmax = 0.f, dmin = 3.0e38f;
                for (int j = lane_of(i); j < f; j += 32) {
                    const float l = 1.f / invd[j];
                    dmax = fmaxf(dmax, l);
                    dmin = fminf(dmin, l);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
                    dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
                }
                if (i == lead_of(g))
                    cflag[1] = (dmax / dmin) * (dmax / dmin) > p.cond_threshold ? 1 : 0;
            }
            gs.sync();
            xi = i < f ? yv[i] : 0.f;
            const bool wide = cflag[1] != 0;
            for (int s = 0; s < p.refine_steps; ++s) {
                if (i < FP) sv[i] = xi * di;  // (FP8: sum_j A'_ij d_j x_j, then times d_i)
                gs.sync();
                const double ax = (wide ? tmem_rowdot<FP, true>(tb, p.ng, sv)
                                        : tmem_rowdot<FP, false>(tb, p.ng, sv)) * (double)di;
                float ri;
                if (wide)
                    ri = (float)((double)bi - ax - (double)reg * (double)xi);
                else
                    ri = bi - (float)ax - reg * xi;
                if (i < FP) yv[i] = i < f ? ri : 0.f;  // (the solve reads and writes each
                chol_solve_group<FP>(i, Ls, Dv, yv, xb, gs);  //  thread's own row)
                if (i < f) xi += yv[i];
            }
            if (wide && et == 0 && p.refine_steps > 0) atomicAdd(&p.flags[1], 1);
        }
    } else if constexpr (SOLVER == SOLVER_CGTC) {
        // the largest entry of the regularised Gram (on its diagonal: PSD) sets the scale 2^-ka;
        // a warp reads the two 16-column chunks holding its 32 lanes' diagonal entries
        const int lg = i & ~31;
        float dii = 0.f;
#pragma unroll
        for (int h = 0; h < 32; h += 16) {
            if (lg + h < p.ng) {  // warp-uniform
                float v[16];
                tmem_ld16(tb + lg + h, v);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (lg + h + j == i) dii = v[j];
            }
        }
        dii = i < f ? dii * di * di + reg : 0.f;
        const float dmax = gmax128(dii, red, slot, gs);
        const int ka = exp2_of(dmax) > 14 ? exp2_of(dmax) - 14 : 0;
        const float sa = pow2f(-ka);
        // b_i, then row i (+ lambda n_u on the diagonal) scaled, rounded to binary16 and packed
        // into columns [0, ng/2) (each 16-column chunk is read before its 8 packed columns land)
        {
            float b0, b1;
            tmem_ld2(tb + p.ng, b0, b1);
            bi = i < f ? b0 * di : 0.f;
        }
#pragma unroll
        for (int c = 0; c < FP; c += 16) {
            if (c < p.ng) {  // warp-uniform
                float v[16];
                tmem_ld16(tb + c, v);
                if constexpr (F8) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] *= di * dsc[c + j];
                }
                uint32_t w[8];
#pragma unroll
                for (int j = 0; j < 16; j += 2) {
                    float a0 = i < f ? v[j] : 0.f, a1 = i < f ? v[j + 1] : 0.f;  // padded: zero
                    if (c + j == i && i < f) a0 += reg;
                    if (c + j + 1 == i && i < f) a1 += reg;
                    const __half2 h2 = __floats2half2_rn(a0 * sa, a1 * sa);  // .x = column c + j
                    w[j >> 1] = *reinterpret_cast<const uint32_t *>(&h2);
                }
                tmem_st8(tb + c / 2, w);
            }
        }
        tmem_wait_st();
        xi = cg_tc<FP>(p, tb & 0xFFFFu, tb, bi, i < f ? xw : 0.f, i, et, lead_of(g),
                       reinterpret_cast<__half *>(Ls), ka, mvbar, cst, red, abort, gs, ok);
    } else {
        // CG / LU work on the row in registers: a[j] = A[i][j] (+ lambda n_u on the diagonal)
        // (xw, the CG warm start, was loaded by the caller as soon as the row was known)
        if constexpr (cg_quad_rows(SOLVER, FP)) {
            // quad-blocked rows (cg_quad): chunk k (columns 16k..16k+15) of row i is cut into
            // four float4, one per lane of the quad; rows 4a+2, 4a+3 go straight to their
            // owners' shared slots, rows 4a, 4a+1 move across the quad by shuffles (lane c
            // takes rows 4a and 4a+1 from lanes c^m, m = 1, 2, 3, or keeps its own)
            constexpr int NK = FP / 16;
            static_assert(CGQ_SLOT * 4 * 2 * NK == cgq_floats(FP), "quad slot layout");
            float4 *sa = reinterpret_cast<float4 *>(Ls);
            float4 ar[2][NK];
            const int c = i & 3;
            const int qa = i & ~3;
            {
                float b0, b1;
                tmem_ld2(tb + p.ng, b0, b1);
                bi = i < f ? b0 * di : 0.f;
            }
            // The accumulator's columns f..ng-1 are zero (the table's padded features are zero
            // and the gathers fill zeros past them), so only a chunk reaching column ng (b) is
            // cut there; rows i >= f are cleared; the diagonal term (lambda n_u, 1 on the padded
            // rows) is added in every product instead (cg_quad).
#pragma unroll
            for (int k = 0; k < NK; ++k) {
                float v[16];
                if (16 * k < p.ng) {  // warp-uniform
                    tmem_ld16(tb + 16 * k, v);
                    if constexpr (F8) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) v[j] *= di * dsc[16 * k + j];
                    }
                    if (16 * k + 16 > p.ng) {  // warp-uniform: the chunk holding column ng
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (16 * k + j >= p.ng) v[j] = 0.f;
                    }
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] = i < f ? v[j] : 0.f;
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j) v[j] = 0.f;
                }
                float4 V[4];
#pragma unroll
                for (int g4 = 0; g4 < 4; ++g4)
                    V[g4] = make_float4(v[4 * g4], v[4 * g4 + 1], v[4 * g4 + 2], v[4 * g4 + 3]);
                if (c >= 2) {
#pragma unroll
                    for (int g4 = 0; g4 < 4; ++g4)
                        sa[(2 * k + c - 2) * CGQ_SLOT + qa + g4] = V[g4];
                }
                const float4 s1 = c == 0 ? V[1] : V[0];
                const float4 s2 = c == 0 ? V[2] : V[3];
                const float4 s3 = c == 0 ? V[3] : V[2];
                const float4 r1 = shfl_xor4(s1, 1), r2 = shfl_xor4(s2, 2), r3 = shfl_xor4(s3, 3);
                ar[0][k] = c == 0 ? V[0] : c == 1 ? r1 : c == 2 ? r2 : r3;
                ar[1][k] = c == 0 ? r1 : c == 1 ? V[1] : c == 2 ? r3 : r2;
            }
            tc_fence_before();
            gs.sync();  // (also orders the slots' stores before the first product)
            if (et == 0) mbar_arrive(release);
            released = true;
            xi = cg_quad<NK>(ar, sa, bi, xw, i, sv, red, p.cg_iters, p.cg_tol, gs,
                             i < f ? reg : 1.f);
        } else {
        // the Gram row (columns < ng) and b (column ng) in one or two TMEM round trips
        float a[FP];
        {
            float b;
            tmem_ld_row(tb, (uint32_t)p.ng, a, b);
#pragma unroll
            for (int j = 0; j < FP; ++j) a[j] = j < p.ng && i < f ? (F8 ? a[j] * di * dsc[j] : a[j]) : 0.f;
            bi = i < f ? b * di : 0.f;
        }
#pragma unroll
        for (int j = 0; j < FP; ++j)
            if (j == i) a[j] = i < f ? a[j] + reg : 1.f;  // identity on the padded rows
        // the row is in registers: hand the accumulator back to the MMA issuer now
        tc_fence_before();
        gs.sync();
        if (et == 0) mbar_arrive(release);
        released = true;

        if constexpr (SOLVER == SOLVER_CG) {
            xi = cg_reg<FP>(a, bi, xw, i, sv, red, p.cg_iters, p.cg_tol, gs);
        } else {
            // reference semantics: LU without pivoting of the full matrix, in shared memory
            const int GS = gs_of(f);
            float *G = Ls;
            if (i < f) {
#pragma unroll
                for (int j = 0; j < FP; ++j)
                    if (j < f) G[i * GS + j] = a[j];
            }
            float *vb = vec;
            if (i < f) vb[i] = bi;
            gs.sync();
            if (g == 0)
                good = lu_nopivot_solve<NamedSync<1, 128>>(G, GS, f, vb, et, 128);
            else
                good = lu_nopivot_solve<NamedSync<2, 128>>(G, GS, f, vb, et, 128);
            xi = i < f ? vb[i] : 0.f;
            gs.sync();
        }
        }
    }
    const float nonfinite = gsum128((i < f && !isfinite(xi)) ? 1.f : 0.f, red, slot, gs);
    if (!good || nonfinite > 0.f) {
        if (i < f) xo[i] = 0.f;
        if (et == 0) atomicAdd(&p.flags[0], 1);
    } else if (i < f) {
        xo[i] = xi;
    }
    return released;
}

template <int FP, int SOLVER, bool F8>
__global__ void __launch_bounds__(nthreads_of(SOLVER, FP), 1)
    sweep_tc_kernel(const __grid_constant__ Params p) {
    constexpr int NSTAGE = nstage_of(SOLVER, FP, F8);
    constexpr int SBYTES = stage_bytes(F8), TBYTES = tile_bytes(F8);
    static_assert(NSTAGE >= 2 && NSTAGE <= MAX_NSTAGE, "stage ring");
    constexpr int NEPI = nepi_of(SOLVER, FP);
    constexpr int WP = 4 * NEPI;  // producer warp; then the MMA issuer and the gather warps
    constexpr int WM = WP + 1;
    constexpr int WG = WP + 2;
    constexpr int NGATHER = ngather_of(SOLVER, FP);
    // One MMA per 16 ratings for the Gram and the right-hand side together: the gather warp of a
    // stage waits for its bytes, writes the stage's ratings into feature column ng of the panel
    // (the gather left it zero: ng >= fst) and marks the stage ready; the MMA issuer waits for
    // ready and issues M=128 x N=ng+16 (Gram in columns [0, ng), b in column ng; row ng of the
    // accumulator then holds b^T, a padded row the solvers ignore).  Where the gather warps have
    // the time: the tensor-core CG's six; FP = 128 (ng = 128) has no free column.  FP8 stages
    // take the e4m3 rating into byte ng of each 128-byte row: one MMA per 32 ratings instead of
    // a Gram MMA and an N = 16 right-hand-side MMA (the same e4m3 products, summed in one pass).
    constexpr bool FUSED = SOLVER == SOLVER_CGTC && FP <= 112;
    static_assert(NGATHER <= MAX_NGATHER, "");
    // Register split: setmaxnreg acts per warpgroup, so the solver warps and the service warps
    // each form whole warpgroups, and the registers the solvers take are exactly those the
    // service warps give back out of the launch's own (a larger .inc would wait forever; the host
    // also checks the compiled count, configure_fp).
    constexpr bool REGSPLIT = regsplit_of(SOLVER, FP);
    static_assert(!REGSPLIT || (WP % 4 == 0 && (2 + NGATHER) % 4 == 0), "whole warpgroups");
    static_assert(!REGSPLIT || (solver_regs_of(SOLVER, FP) * 128 * NEPI +
                                    SERVICE_REGS * 32 * (2 + NGATHER) ==
                                launch_regs_of(SOLVER, FP) * nthreads_of(SOLVER, FP)),
                  "register split");
    static_assert(!REGSPLIT || (launch_regs_of(SOLVER, FP) % 8 == 0 &&
                                launch_regs_of(SOLVER, FP) * nthreads_of(SOLVER, FP) <= 65536),
                  "register split");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *ring = smem;
    float *gscratch = (float *)(ring + NSTAGE * SBYTES);
    float *dsc = gscratch + GroupLayout<FP, SOLVER>::floats * NEPI;  // [MAXF] FP8 scales
    int32_t *mcol = (int32_t *)(dsc + (F8 ? MAXF : 0));                             // [MR][KC]
    float *mval = reinterpret_cast<float *>(mcol + MR * KC);                            // [MR][KC]
    Meta *mmeta = reinterpret_cast<Meta *>(mval + MR * KC);                             // [MR]
    Meta *smeta = reinterpret_cast<Meta *>(mmeta + MR);                                 // [NSTAGE]
    Meta *ameta = smeta + NSTAGE;
    uint64_t *bars = (uint64_t *)(ameta + MAX_NBUF);  // 16-byte aligned: Meta is 16 bytes
    uint64_t *full = bars, *empty = bars + NSTAGE;
    uint64_t *acc_full = bars + 2 * NSTAGE;
    uint64_t *acc_empty = acc_full + MAX_NBUF, *acc_meta = acc_empty + MAX_NBUF;
    uint64_t *drain = acc_meta + MAX_NBUF;
    uint64_t *mvbar = drain + 1;  // [MAX_NBUF]: the tensor-core CG's product barrier per group
    uint64_t *ready = mvbar + MAX_NBUF;  // [MAX_NSTAGE]: stage's ratings in the panel (FUSED)
    uint32_t *tmem_slot = (uint32_t *)(ready + MAX_NSTAGE);
    volatile int *abort = (volatile int *)(tmem_slot + 1);
    volatile int *grp_ok = abort + 1;  // per-group broadcast of the leader's wait outcome
    volatile int *pub = grp_ok + MAX_NBUF;  // stages whose metadata has landed (producer)
    volatile int *fin = pub + 1;            // the producer has published its last stage
    volatile int *done = fin + 1;               // [NGATHER]: stages gather warp h has taken its
                                                // metadata from (slot t % MR free again)
    volatile int *armed = done + MAX_NGATHER;   // [NSTAGE]: the last stage armed in each slot

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nbuf = p.nbuf;

    // zero the operand ring once: features f..127 and rating-tile rows 1..15 are never written
    for (int i = tid; i < NSTAGE * SBYTES / 16; i += blockDim.x)
        reinterpret_cast<uint4 *>(ring)[i] = make_uint4(0, 0, 0, 0);
    if constexpr (SOLVER == SOLVER_CGTC) {  // the groups' operand tiles: columns 2..15 stay zero
        for (int i = tid; i < (int)(GroupLayout<FP, SOLVER>::floats * NEPI / 4); i += blockDim.x)
            reinterpret_cast<float4 *>(gscratch)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if constexpr (F8) {  // padded features scale by 1 (their values are zero)
        for (int j = tid; j < MAXF; j += blockDim.x) dsc[j] = j < p.f ? p.dscale[j] : 1.f;
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) {
            // the gathering warp's arrive.expect_tx; the TMA bytes complete the phase
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
            armed[s] = -1;
        }
        for (int h = 0; h < NGATHER; ++h) done[h] = 0;
        for (int b = 0; b < MAX_NBUF; ++b) {
            mbar_init(smem_u32(&acc_full[b]), 1);
            mbar_init(smem_u32(&acc_empty[b]), 1);
            mbar_init(smem_u32(&acc_meta[b]), 1);
            mbar_init(smem_u32(&mvbar[b]), 1);
        }
        mbar_init(smem_u32(drain), 1);
        for (int u = 0; u < MAX_NSTAGE; ++u) mbar_init(smem_u32(&ready[u]), 1);
        *abort = 0;
        *pub = 0;
        *fin = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    if (warp == WM) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(p.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // (the solver warpgroups first: each role's register budget covers the code it runs)
    if (warp < WP) {
        if constexpr (REGSPLIT)
            asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(solver_regs_of(SOLVER, FP)) : "memory");
        // ------------------------------------------------------------------ solver warpgroups
        const int g = warp >> 2;
        const int et = tid - 128 * g;                // 0..127 inside the group
        const int lanegrp = (warp & 3) * 32;         // TMEM lanes this warp may read
        const int i = lanegrp + lane;                // row of the Gram held by this thread
        const GroupSync gs{1 + g};
        float *gsm = gscratch + GroupLayout<FP, SOLVER>::floats * g;
        volatile int *okflag = grp_ok + g;
        bool ok = true;
        CgTcState cst;
        auto group_wait = [&](uint32_t bar, uint32_t parity) -> bool {
            if (et == lead_of(g)) *okflag = mbar_wait(bar, parity, abort, p.wait_ns) ? 1 : 0;
            gs.sync();
            const bool r = *okflag != 0;
            gs.sync();
            return r;
        };
        for (uint32_t acc_it = g;; acc_it += NEPI) {
            const uint32_t buf = acc_it % nbuf;
            const uint32_t use = acc_it / nbuf;
            if (!group_wait(smem_u32(&acc_meta[buf]), use & 1)) { ok = false; break; }
            const Meta m = ameta[buf];
            if (m.row < 0) break;
            // the CG warm start is an HBM load: issue it as soon as the row is known, before the
            // wait for its Gram
            const float xw = ((SOLVER == SOLVER_CG || SOLVER == SOLVER_CGTC) && i < p.f && m.nu > 0)
                                 ? p.X[(int64_t)m.row * p.f + i] : 0.f;
            if (!group_wait(smem_u32(&acc_full[buf]), use & 1)) { ok = false; break; }
            tc_fence_after();
            bool released = false;
            if (m.nu > 0) {
                const uint32_t tb = tmem_base + ((uint32_t)lanegrp << 16) + buf * p.acc_stride;
                released = solve_row<FP, SOLVER, F8>(p, m, tb, i, et, g, gsm, gs,
                                                     smem_u32(&acc_empty[buf]), xw,
                                                     smem_u32(&mvbar[g]), cst, abort, ok, dsc);
            } else if (i < p.f) {
                p.X[(int64_t)m.row * p.f + i] = 0.f;  // no ratings: defined as x = 0
            }
            if (!released) {
                tc_fence_before();
                gs.sync();
                if (et == 0) mbar_arrive(smem_u32(&acc_empty[buf]));
            }
        }
        // a product chain whose completion was not seen (a wait ran out) finishes before TMEM is
        // released: after a failed wait the leader issues nothing more, so it is the last one
        // (product calls after the abort commit nothing: wait for the last commit's phase)
        if (SOLVER == SOLVER_CGTC && et == lead_of(g) && cst.unconfirmed)
            mbar_wait(smem_u32(&mvbar[g]), cst.committed & 1, nullptr, WAIT_NS);
        if (!ok) {  // (the tensor-core CG's waits are per warp: each failing warp counts)
            *abort = 1;
            if (SOLVER == SOLVER_CGTC ? lane == 0 : et == 0) atomicAdd(&p.flags[2], 1);
        }
    } else {
        if constexpr (REGSPLIT)
            asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(SERVICE_REGS) : "memory");
        if (warp == WP) {
            // ------------------------------------------------------------------ producer
            // Two cursors walk the same sequence of stages (KC ratings of one row each).  The
            // look-ahead cursor issues a stage's column ids and ratings as 4-byte cp.async into the
            // metadata ring MD stages ahead, with its Meta; the publishing cursor waits for that
            // cp.async group and publishes the stage to the gather warps, which do the rest.  Rows
            // come in chunks from the atomic counter (one at a time among the first `head` slots, the
            // heaviest rows, then CH at a time), pipelined two chunks ahead so the dependent
            // order[] -> ptr[] loads have landed when a chunk starts.
            constexpr int CH = 8;
            const int head = 4 * (int)gridDim.x;
            int grab_size = 1;
            auto grab = [&](int &cb, int &cc) {
                int b = 0;
                if (lane == 0) b = atomicAdd(p.work, grab_size);
                b = __shfl_sync(0xffffffffu, b, 0);
                cb = b;
                cc = max(0, min(grab_size, p.nrows - b));
                if (b + grab_size >= head) grab_size = CH;
            };
            // chunk pipeline: current (row, beg, end in lane j), next (row, beg, end), next-next (row)
            int ccnt, crow, cbeg, cend, n1cnt, n1row, n1beg, n1end, n2cnt, n2row;
            {
                int cb;
                grab(cb, ccnt);
                crow = lane < ccnt ? p.order[cb + lane] : 0;
                grab(cb, n1cnt);
                n1row = lane < n1cnt ? p.order[cb + lane] : 0;
                grab(cb, n2cnt);
                n2row = lane < n2cnt ? p.order[cb + lane] : 0;
                cbeg = lane < ccnt ? p.ptr[crow] : 0;
                cend = lane < ccnt ? p.ptr[crow + 1] : 0;
                n1beg = lane < n1cnt ? p.ptr[n1row] : 0;
                n1end = lane < n1cnt ? p.ptr[n1row + 1] : 0;
            }
            const uint64_t stream_pol = l2_evict_first_policy();  // column ids and ratings: once
            int aj = 0;                                          // look-ahead cursor: row of chunk
            int abase = __shfl_sync(0xffffffffu, cbeg, 0);       // and first rating of its stage
            uint32_t gen = 0;                                    // stages issued by the look-ahead
            // the metadata slot of stage g is free once the gather warp of stage g - MR has taken the
            // column ids, ratings and Meta out of it (bounded wait; false on timeout or abort)
            auto slot_free = [&](uint32_t g) -> bool {
                if (g < (uint32_t)MR) return true;
                const uint32_t old = g - MR;
                int r = 1;
                if (lane == 0) {
                    const volatile int *d = done + old % NGATHER;
                    const unsigned long long t0 = now_ns();
                    for (uint32_t k = 0;; ++k) {
                        if ((uint32_t)*d > old) break;
                        if ((k & 255) == 255 && (*abort || now_ns() - t0 > p.wait_ns)) {
                            r = 0;
                            break;
                        }
                    }
                    __threadfence_block();
                }
                return __shfl_sync(0xffffffffu, r, 0) != 0;
            };
            // issue the metadata of stage `gen`: 1 issued, 0 no rows left, -1 its slot never freed
            auto generate = [&]() -> int {
                while (aj >= ccnt) {
                    if (ccnt <= 0) return 0;
                    ccnt = n1cnt; crow = n1row; cbeg = n1beg; cend = n1end;
                    n1cnt = n2cnt; n1row = n2row;
                    n1beg = lane < n1cnt ? p.ptr[n1row] : 0;     // n2's row ids landed a chunk ago
                    n1end = lane < n1cnt ? p.ptr[n1row + 1] : 0;
                    int cb;
                    grab(cb, n2cnt);
                    n2row = lane < n2cnt ? p.order[cb + lane] : 0;
                    aj = 0;
                    if (ccnt <= 0) return 0;
                    abase = __shfl_sync(0xffffffffu, cbeg, 0);
                }
                if (!slot_free(gen)) return -1;
                const int row = __shfl_sync(0xffffffffu, crow, aj);
                const int beg = __shfl_sync(0xffffffffu, cbeg, aj);
                const int end = __shfl_sync(0xffffffffu, cend, aj);
                const int cnt = min(KC, end - abase);
                const int slot = (int)(gen % MR);
                int32_t *mc = mcol + slot * KC;
                float *mv = mval + slot * KC;
    #pragma unroll
                for (int h = 0; h < KC; h += 32) {
                    if (lane + h < cnt) {
                        cp_async4(smem_u32(mc + lane + h), p.idx + abase + lane + h, stream_pol);
                        cp_async4(smem_u32(mv + lane + h), p.val + abase + lane + h, stream_pol);
                    } else {
                        mc[lane + h] = p.zero_row;   // the ragged tail gathers the all-zero row
                        mv[lane + h] = 0.f;
                    }
                }
                cp_commit();
                if (lane == 0) {
                    Meta m;
                    m.row = row;
                    m.cnt = cnt;
                    m.flags = (abase == beg ? 1 : 0) | (abase + KC >= end ? 2 : 0);
                    m.nu = end - beg;
                    mmeta[slot] = m;
                }
                abase += KC;
                if (abase >= end) {
                    ++aj;
                    abase = aj < ccnt ? __shfl_sync(0xffffffffu, cbeg, aj < ccnt ? aj : 0) : 0;
                }
                ++gen;
                return 1;
            };
            bool ok = true;
            int more = 1;
            for (int k = 0; k < MD && more == 1; ++k) more = generate();
            if (more < 0) ok = false;
            uint32_t it = 0;  // stages published
            while (ok && it < gen) {
                // stage it's metadata group: at most gen - it - 1 younger groups may stay pending
                if (gen - it - 1 >= (uint32_t)(MD - 1))
                    cp_wait<MD - 1>();
                else
                    cp_wait<0>();
                __syncwarp();  // every lane's copies (and tail fills) of the stage are in place
                if (lane == 0) {
                    __threadfence_block();
                    *pub = (int)(it + 1);
                }
                __syncwarp();
                ++it;
                if (more == 1) {
                    more = generate();
                    if (more < 0) ok = false;
                }
            }
            // nothing of this warp may be in flight when the CTA tears down
            cp_wait<0>();
            __syncwarp();
            if (lane == 0) {  // *pub is now the number of stages; the gather warps add the end marker
                __threadfence_block();
                *fin = 1;
            }
            if (!ok) {
                *abort = 1;
                if (lane == 0) atomicAdd(&p.flags[2], 1);
            }
        } else if (warp == WM) {
            // ------------------------------------------------------------------ MMA issuer
            if (lane == 0) {
                const int ng_mma = FUSED ? p.ng + 16 : p.ng;
                const uint32_t idesc_g = F8 ? idesc_e4m3(128, ng_mma, true, true)
                                            : idesc_bf16(128, ng_mma, true, true);
                const uint32_t idesc_r = F8 ? idesc_e4m3(128, 16, true, false)
                                            : idesc_bf16(128, 16, true, false);
                const uint32_t ring_s = smem_u32(ring);
                uint32_t it = 0, acc_it = 0, buf = 0;
                bool ok = true;
                auto take_buffer = [&]() -> bool {  // wait until accumulator acc_it % nbuf is free
                    buf = acc_it % nbuf;
                    const uint32_t use = acc_it / nbuf;
                    if (use >= 1 &&
                        !mbar_wait(smem_u32(&acc_empty[buf]), (use - 1) & 1, abort, p.wait_ns))
                        return false;
                    tc_fence_after();
                    return true;
                };
                for (;;) {
                    const int s = it % NSTAGE;
                    // (every writer of the stage's operands fenced its generic stores into the async
                    // proxy before it arrived: the acquire of this wait is all the MMA needs)
                    if (!mbar_wait(smem_u32(FUSED ? &ready[s] : &full[s]), (it / NSTAGE) & 1, abort,
                                   p.wait_ns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const Meta m = smeta[s];
                    if (m.row < 0) {  // end of work: one end marker per solver warpgroup
                        for (int g = 0; g < NEPI && ok; ++g) {
                            if (!take_buffer()) { ok = false; break; }
                            ameta[buf] = m;
                            mbar_arrive(smem_u32(&acc_meta[buf]));
                            ++acc_it;
                        }
                        break;
                    }
                    if ((m.flags & 1) && !take_buffer()) { ok = false; break; }
                    const uint32_t dg = tmem_base + buf * p.acc_stride;
                    const uint32_t db = dg + p.ng;
                    const uint32_t tile_s = ring_s + s * SBYTES;
                    if constexpr (F8) {
                        // K = 32 ratings (four 8-rating groups, 4 KB of the one-atom panel) and the
                        // matching 32 bytes of the rating tile's row per MMA
                        const int nk = (m.cnt + F8_K - 1) / F8_K;
                        for (int kk = 0; kk < nk; ++kk) {
                            const uint64_t ad =
                                sdesc(tile_s + kk * 4 * ATOM_BYTES, ATOM_STRIDE, ATOM_BYTES);
                            const uint32_t accum = ((m.flags & 1) && kk == 0) ? 0u : 1u;
                            mma_e4m3(dg, ad, ad, idesc_g, accum);
                            if (!FUSED) {
                                const uint64_t rd = sdesc(tile_s + TBYTES + kk * 32, 16, ATOM_BYTES);
                                mma_e4m3(db, ad, rd, idesc_r, accum);
                            }
                        }
                    } else {
                        const int nk = (m.cnt + 15) >> 4;
                        for (int kk = 0; kk < nk; ++kk) {
                            const uint64_t ad =
                                sdesc(tile_s + kk * 2 * ATOM_BYTES, ATOM_STRIDE, ATOM_BYTES);
                            const uint32_t accum = ((m.flags & 1) && kk == 0) ? 0u : 1u;
                            mma_bf16(dg, ad, ad, idesc_g, accum);
                            if (!FUSED) {
                                const uint64_t rd =
                                    sdesc(tile_s + TBYTES + kk * 32, 16, ATOM_BYTES);
                                mma_bf16(db, ad, rd, idesc_r, accum);
                            }
                        }
                    }
                    mma_commit(smem_u32(&empty[s]));
                    if (m.flags & 2) {
                        ameta[buf] = m;
                        // committed for empty rows too, so buffer b's phase count is its use count
                        mma_commit(smem_u32(&acc_full[buf]));
                        mbar_arrive(smem_u32(&acc_meta[buf]));
                        ++acc_it;
                    }
                    ++it;
                }
                // drain: every MMA issued so far has completed before TMEM is released
                mma_commit(smem_u32(drain));
                if (!mbar_wait(smem_u32(drain), 0, nullptr, WAIT_NS)) ok = false;
                if (!ok) {
                    *abort = 1;
                    atomicAdd(&p.flags[2], 1);
                }
            }
            __syncwarp();
        } else {
            // ------------------------------------------------------------------ gather warps
            // Warp h takes every NGATHER-th stage from t = h once the producer has published it:
            // it waits for the stage's ring slot, writes the rating tile, reads the column ids and
            // Meta out of the metadata slot (handing the slot back), arms the stage's full barrier
            // with the byte count and issues one tile::gather4 per lane (4 ratings x 64 features).
            // The warp whose turn comes after the last stage writes the end marker (row = -1).
            const int h = warp - WG;
            const int natoms = F8 ? 1 : (p.fst > 64 ? 2 : 1);
            const int gq = lane & 15, ga = lane >> 4;  // this lane's 4-rating quad, atom
            const uint64_t keep = l2_evict_last_policy();
            bool ok = true;
            for (uint32_t t = (uint32_t)h;; t += NGATHER) {
                int go = 0;  // 1: stage t is published, 0: no more stages, -1: timed out or aborted
                uint32_t total = 0;
                if (lane == 0) {
                    const unsigned long long t0 = now_ns();
                    for (uint32_t k = 0;; ++k) {
                        if ((uint32_t)*pub > t) { go = 1; break; }
                        if (*fin) {
                            total = (uint32_t)*pub;
                            go = total > t ? 1 : 0;
                            break;
                        }
                        if ((k & 255) == 255 && (*abort || now_ns() - t0 > p.wait_ns)) {
                            go = -1;
                            break;
                        }
                    }
                    __threadfence_block();
                }
                go = __shfl_sync(0xffffffffu, go, 0);
                total = __shfl_sync(0xffffffffu, total, 0);
                __syncwarp();  // the lanes' reads of the stage's metadata follow lane 0's acquire
                if (go < 0) {
                    ok = false;
                    break;
                }
                if (go == 0 && t != total) break;  // another warp writes the end marker
                const int s = t % NSTAGE;
                if (t >= NSTAGE) {
                    // the slot's previous stage (another warp's) is armed first: then the slot's
                    // empty barrier is at most one phase behind the one waited for below, so its
                    // parity cannot match an older phase
                    int armed_ok = 1;
                    if (lane == 0) {
                        const unsigned long long t0 = now_ns();
                        for (uint32_t k = 0;; ++k) {
                            if (armed[s] >= (int)(t - NSTAGE)) break;
                            if ((k & 255) == 255 && (*abort || now_ns() - t0 > p.wait_ns)) {
                                armed_ok = 0;
                                break;
                            }
                            }
                        __threadfence_block();
                    }
                    if (!__shfl_sync(0xffffffffu, armed_ok, 0)) {
                        ok = false;
                        break;
                    }
                }
                if (t >= NSTAGE &&
                    !mbar_wait_warp(smem_u32(&empty[s]), ((t / NSTAGE) - 1) & 1, abort, p.wait_ns)) {
                    ok = false;
                    break;
                }
                if (go == 0) {  // t == total: the end marker, one stage with row = -1
                    if (lane == 0) {
                        Meta m;
                        m.row = -1;
                        m.cnt = 0;
                        m.flags = 3;
                        m.nu = 0;
                        smeta[s] = m;
                        armed[s] = (int)t;  // (its phase completes on this arrive: no bytes)
                        mbar_arrive(smem_u32(&full[s]));
                        if (FUSED) mbar_arrive(smem_u32(&ready[s]));
                    }
                    __syncwarp();
                    break;
                }
                const int slot = (int)(t % MR);
                Meta m;  // read by lane 0 (which saw the stage published), handed to the warp
                {
                    int4 w = make_int4(0, 0, 0, 0);
                    if (lane == 0) w = *reinterpret_cast<const int4 *>(&mmeta[slot]);
                    m.row = __shfl_sync(0xffffffffu, w.x, 0);
                    m.cnt = __shfl_sync(0xffffffffu, w.y, 0);
                    m.flags = __shfl_sync(0xffffffffu, w.z, 0);
                    m.nu = __shfl_sync(0xffffffffu, w.w, 0);
                }
                uint8_t *tile = ring + s * SBYTES;
                __nv_bfloat16 *rt = reinterpret_cast<__nv_bfloat16 *>(tile + TBYTES);
                if constexpr (F8) {  // e4m3 ratings (star ratings are exact), bytes 0..63 of row 0
                    uint8_t *rt8 = tile + TBYTES;
                    rt8[lane] = __nv_cvt_float_to_fp8(mval[slot * KC + lane], __NV_SATFINITE, __NV_E4M3);
                    rt8[lane + 32] =
                        __nv_cvt_float_to_fp8(mval[slot * KC + lane + 32], __NV_SATFINITE, __NV_E4M3);
                } else {
                    rt[lane] = __float2bfloat16_rn(mval[slot * KC + lane]);
                    rt[lane + 32] = __float2bfloat16_rn(mval[slot * KC + lane + 32]);
                }
                // the MMA reads ratings [0, 16 nk) (FP8: [0, 32 nk)): gather their quads (the ragged
                // tail's column ids point at the zero row), 512 bytes per quad and atom
                const int nq = F8 ? ((m.cnt + F8_K - 1) / F8_K) * (F8_K / 4) : ((m.cnt + 15) >> 4) * 4;
                const bool mine = gq < nq && ga < natoms;
                int32_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
                if (mine) {
                    const int32_t *q = mcol + slot * KC + 4 * gq;
                    r0 = q[0];
                    r1 = q[1];
                    r2 = q[2];
                    r3 = q[3];
                }
                // the rating tile is a generic store: visible to the tensor core (async proxy)
                // before the stage can complete
                fence_async_smem();
                __syncwarp();  // every lane has read the metadata slot and written its ratings
                if (lane == 0) {
                    __threadfence_block();
                    done[h] = (int)(t + 1);  // the metadata slot may be refilled
                    smeta[s] = m;
                    armed[s] = (int)t;
                    mbar_arrive_expect_tx(smem_u32(&full[s]), (uint32_t)(nq * natoms * 512));
                }
                __syncwarp();
                if (mine) {
                    const uint32_t dst = smem_u32(tile) + ga * ATOM_STRIDE + (gq >> 1) * ATOM_BYTES +
                                         (gq & 1) * 512;
                    tma_gather4(dst, &p.tmap, 64 * ga, r0, r1, r2, r3, smem_u32(&full[s]), keep);
                }
                __syncwarp();
                if constexpr (FUSED) {
                    // the stage's ratings into feature column ng, once its gathered rows have landed
                    if (!mbar_wait_warp(smem_u32(&full[s]), (t / NSTAGE) & 1, abort, p.wait_ns)) {
                        ok = false;
                        break;
                    }
                    if constexpr (F8) {
                        // one 128-feature atom of bytes: column ng (a multiple of 16) starts
                        // 16-byte chunk ng / 16 of each row, before the 128-byte swizzle
                        const int rc = p.ng >> 4;
                        const uint8_t *rt8 = tile + TBYTES;
                        for (int k = lane; k < 4 * nq; k += 32)
                            tile[(k >> 3) * ATOM_BYTES + (k & 7) * 128 + ((rc ^ (k & 7)) << 4)] =
                                rt8[k];
                    } else {
                        const int ra = p.ng >> 6, rc = (p.ng & 63) >> 3;  // column ng: atom, chunk
                        for (int k = lane; k < 4 * nq; k += 32)
                            *reinterpret_cast<__nv_bfloat16 *>(tile + ra * ATOM_STRIDE +
                                                               (k >> 3) * ATOM_BYTES + (k & 7) * 128 +
                                                               ((rc ^ (k & 7)) << 4)) = rt[k];
                    }
                    fence_async_smem();  // generic stores, read by the tensor core
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(&ready[s]));
                }
            }
            if (!ok) {
                *abort = 1;
                if (lane == 0) atomicAdd(&p.flags[2], 1);
            }
            // no gather may be in flight when the CTA tears down: once every gather warp is done,
            // wait for the last stage armed in each ring slot (a slot is re-armed only after the
            // MMA consumed its previous stage, so only the last can still be landing; bounded)
            asm volatile("bar.sync %0, %1;" ::"r"(15), "r"(32 * NGATHER) : "memory");
            if (h == 0 && lane == 0) {
                for (int u = 0; u < NSTAGE; ++u) {
                    const int a = armed[u];
                    if (a >= 0)
                        mbar_wait(smem_u32(&full[u]), (uint32_t)(a / NSTAGE) & 1, nullptr, WAIT_NS);
                }
            }
            __syncwarp();
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == WM)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                     "r"(p.tmem_cols)
                     : "memory");
}

// Per padded size FP and operand type (one translation unit each, compiled in parallel): set the
// shared-memory limit of the four solver variants and launch the selected one.
template <int FP, bool F8>
cudaError_t configure_fp(size_t smem) {
    // the host's geometry and the kernel's per-group layout agree
    static_assert(group_floats(FP, SOLVER_CG) == GroupLayout<FP, SOLVER_CG>::floats, "");
    static_assert(group_floats(FP, SOLVER_CHOL) == GroupLayout<FP, SOLVER_CHOL>::floats, "");
    static_assert(group_floats(FP, SOLVER_LU) == GroupLayout<FP, SOLVER_LU>::floats, "");
    static_assert(group_floats(FP, SOLVER_CGTC) == GroupLayout<FP, SOLVER_CGTC>::floats, "");
    static_assert(GroupLayout<FP, SOLVER_CGTC>::floats % 32 == 0, "");
    // every variant may use up to the device's opt-in maximum; each launch asks for its own size
    int dev = 0, maxsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if ((size_t)maxsm < smem) return cudaErrorInvalidValue;
    if (regsplit_of(SOLVER_CG, FP)) {
        // the split's setmaxnreg.inc waits for registers the launch must hold: refuse a build
        // whose compiled register count differs from the one the split was sized for
        cudaFuncAttributes fa;
        cudaError_t ea = cudaFuncGetAttributes(&fa, sweep_tc_kernel<FP, SOLVER_CG, F8>);
        if (ea != cudaSuccess) return ea;
        if (fa.numRegs != launch_regs_of(SOLVER_CG, FP)) return cudaErrorInvalidKernelImage;
    }
    cudaError_t e = cudaFuncSetAttribute(sweep_tc_kernel<FP, SOLVER_CG, F8>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sweep_tc_kernel<FP, SOLVER_CHOL, F8>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sweep_tc_kernel<FP, SOLVER_LU, F8>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sweep_tc_kernel<FP, SOLVER_CGTC, F8>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
    return e;
}

template <int FP, bool F8>
void launch_fp(const Params &p, const Geometry &g, int grid, cudaStream_t st) {
    switch (p.solve) {
    case SOLVER_CG: sweep_tc_kernel<FP, SOLVER_CG, F8><<<grid, g.nthreads, g.smem, st>>>(p); break;
    case SOLVER_LU: sweep_tc_kernel<FP, SOLVER_LU, F8><<<grid, g.nthreads, g.smem, st>>>(p); break;
    case SOLVER_CGTC:
        sweep_tc_kernel<FP, SOLVER_CGTC, F8><<<grid, g.nthreads, g.smem, st>>>(p);
        break;
    default: sweep_tc_kernel<FP, SOLVER_CHOL, F8><<<grid, g.nthreads, g.smem, st>>>(p); break;
    }
}

#define ALS_TC_DECLARE(FP)                                                                 \
    cudaError_t configure_##FP(size_t smem);                                               \
    void launch_##FP(const Params &p, const Geometry &g, int grid, cudaStream_t st);       \
    cudaError_t configure_##FP##_e4m3(size_t smem);                                        \
    void launch_##FP##_e4m3(const Params &p, const Geometry &g, int grid, cudaStream_t st);
ALS_TC_DECLARE(32)
ALS_TC_DECLARE(64)
ALS_TC_DECLARE(112)
ALS_TC_DECLARE(128)

}  // namespace tcg
}  // namespace als
