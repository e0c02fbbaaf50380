// Split-precision tensor-core path: digit slicing, rotational-dipole band construction,
// the persistent tcgen05 digit-product GEMM and the FP64 refinement kernels.
#include "split.h"

#include <atomic>

#include <cuda_bf16.h>

#include "gain_internal.h"

namespace gain {
namespace split {
namespace {

constexpr uint32_t BOX_A = BM * BK * 2;     // bytes of one A k-block box (16 KB)
constexpr uint32_t BOX_B = BN * BK * 2;     // bytes of one B k-block box (16 KB)
constexpr uint32_t STAGE_A = KSTEP * BOX_A; // bytes per A stage
constexpr uint32_t STAGE_B = KSTEP * BOX_B; // bytes per B stage
// Warp 0 issues the TMA copies, warp 1 the MMAs, warps 2.. are the epilogue: EPI_WARPS
// warps, two per TMEM lane quadrant, each draining and finalising half of the tile's
// columns (so the finalisation, which holds the next tile's first drain back, is short).
constexpr int EPI_WARPS = 8;
constexpr int NTHREADS = 64 + 32 * EPI_WARPS;
constexpr int EPI_HALVES = EPI_WARPS / 4;     // column parts of a tile
constexpr int EPI_GROUPS = BN / 32 / EPI_HALVES;   // 32-column groups per epilogue warp
// shared memory of the GEMM after its stage ring (the larger, the pair's) and the barriers:
// the current tile's column statistics, five floats per column
constexpr uint32_t COLSTAT_OFF = STAGES * 3 * (BOX_A + BOX_B / 2) + 256;
constexpr uint32_t COLSTAT_BYTES = 5 * BN * 4;
// then (grouped launch) the arguments of the epilogue's current tile
constexpr uint32_t GARGS_OFF = COLSTAT_OFF + COLSTAT_BYTES;
constexpr uint32_t GARGS_BYTES = (sizeof(GemmArgs) + 15) / 16 * 16;
constexpr uint32_t TMEM_COLS = 512;         // acc0 [0,128) acc1 [128,256) hi [256,384) lo [384,512)
constexpr unsigned long long kWaitNs = 2000000000ull;   // 2 s per wait before giving up

// ------------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Probe with a zero suspend-time hint: the caller loops (with its own time limit), and a
// probe that does not offer to suspend costs the MMA-issuing thread less time per stage.
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(0)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait on a barrier phase.  Gives up when another role raised the CTA abort flag
// (unless ignore_abort) or after kWaitNs, raising the flag and the device error word.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                          int code, bool ignore_abort = false, unsigned long long limit_ns = kWaitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 127u) == 0) {
            if (!ignore_abort && *abort_flag) return false;
            if (globaltimer() - t0 > limit_ns) {
                *abort_flag = 1;
                atomicCAS(err, 0, code);
                return false;
            }
        }
    }
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar,
                                            int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}
// ---- CTA-pair (cta_group::2) forms: the two CTAs of a cluster share each MMA (M = 256)
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_map(uint32_t addr, uint32_t rank) {   // peer's address
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}
__device__ __forceinline__ void tma_load_3d_pair(uint32_t dst, const CUtensorMap* map, uint32_t bar_cluster, int c0,
                                                 int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(bar_cluster), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}
__device__ __forceinline__ void tmem_alloc_pair(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on the barrier at this offset in each CTA of mask (bit r = cluster rank r)
__device__ __forceinline__ void mma_commit_pair(uint32_t bar, uint16_t mask) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(bar), "h"(mask)
                 : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

#define GAIN_R8(b) "=r"(r[b + 0]), "=r"(r[b + 1]), "=r"(r[b + 2]), "=r"(r[b + 3]), \
                   "=r"(r[b + 4]), "=r"(r[b + 5]), "=r"(r[b + 6]), "=r"(r[b + 7])
#define GAIN_W8(b) "r"(r[b + 0]), "r"(r[b + 1]), "r"(r[b + 2]), "r"(r[b + 3]), \
                   "r"(r[b + 4]), "r"(r[b + 5]), "r"(r[b + 6]), "r"(r[b + 7])

// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : GAIN_R8(0), GAIN_R8(8), GAIN_R8(16), GAIN_R8(24)
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : GAIN_R8(0), GAIN_R8(8)
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
        "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
        GAIN_W8(0), GAIN_W8(8), GAIN_W8(16), GAIN_W8(24)
        : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr),
        GAIN_W8(0), GAIN_W8(8)
        : "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with 128-byte swizzle:
// rows of 128 bytes, 8-row groups 1024 bytes apart (SBO), base 1024-byte aligned.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);       // start address
    d |= (uint64_t)1 << 16;                        // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset
    d |= (uint64_t)1 << 46;                        // descriptor version
    d |= (uint64_t)2 << 61;                        // 128-byte swizzle
    return d;
}
// Instruction descriptor: BF16 x BF16 -> F32, A and B K-major, M = BM, N = BN.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);
// the same for a CTA pair: M = 2 BM rows, each CTA holding BM rows of A and BN/2 rows of B
constexpr uint32_t kIdescPair = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                ((uint32_t)((2 * BM) >> 4) << 24);

__device__ __forceinline__ float pow2f(int e) {   // exact 2^e for -126 <= e <= 127
    return __int_as_float((e + 127) << 23);
}
__device__ __forceinline__ double pow2d(int e) {
    if (e >= -1022 && e <= 1023) return __longlong_as_double((long long)(e + 1023) << 52);
    return ldexp(1.0, e);
}
// Bits of the double nearest (ties to even) to run 2^E, by integer operations only (the FP64
// units are slow on this part); *mag = |run| 2^-kFixTotal as a float, truncated.  Results
// outside the normal range take the FP64 route.
__device__ __forceinline__ unsigned long long scaled_bits(long long run, int E, float* mag) {
    if (run == 0) {
        *mag = 0.0f;
        return 0ull;
    }
    const unsigned long long sign = run < 0 ? (1ull << 63) : 0ull;
    unsigned long long m = run < 0 ? 0ull - (unsigned long long)run : (unsigned long long)run;
    int msb = 63 - __clzll((long long)m);
    if (msb > 52) {
        const int k = msb - 52;
        const unsigned long long q = m >> k;
        const unsigned long long rem = m & ((1ull << k) - 1ull);
        const unsigned long long half = 1ull << (k - 1);
        m = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
        if (m >> 53) {   // rounded up to 2^53
            m >>= 1;
            ++msb;
        }
    } else {
        m <<= (52 - msb);
    }
    *mag = __uint_as_float(((unsigned)(msb - kFixTotal + 127) << 23) | (unsigned)((m >> 29) & 0x7FFFFFull));
    const int be = msb + E + 1023;
    if (be <= 0 || be >= 2047) return (unsigned long long)__double_as_longlong((double)run * pow2d(E));
    return sign | ((unsigned long long)be << 52) | (m & 0xFFFFFFFFFFFFFull);
}

__device__ __forceinline__ void chunk_range(int nkb, int nch, int c, int* lo, int* hi) {
    *lo = (int)(((long)c * nkb) / nch);
    *hi = (int)(((long)(c + 1) * nkb) / nch);
}

// Barriers of the epilogue warps (named barrier 1); the second form also takes their vote:
// true when any of them passes `fail`.  Every epilogue warp reaches each of these barriers
// (its waits are bounded), and all of them leave the tile loop together at a vote when one
// gave up on a drain, so no warp is left waiting at a barrier the others will not reach.
// Both order the shared-memory writes before them with the reads after them.
__device__ __forceinline__ void epilogue_sync() { asm volatile("bar.sync 1, %0;" ::"n"(32 * EPI_WARPS) : "memory"); }
__device__ __forceinline__ bool epilogue_sync_any(bool fail) {
    uint32_t any;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(any)
        : "r"((uint32_t)fail), "n"(32 * EPI_WARPS)
        : "memory");
    return any != 0;
}

// The arguments of a tile: the launch's own, or (grouped launch) those of the tile's group.
template <bool G>
__device__ __forceinline__ const GemmArgs& group_args(const GemmArgs& a, const Tile& tl) {
    if constexpr (G) return a.groups[tl.group].args;
    else return a;
}

// ------------------------------------------------------------------- the GEMM kernel
// SMAX / CMAX: compile-time bounds of the slices and chunks a launch may use (register arrays
// of the epilogue are sized by them).  PAIR: the two CTAs of a cluster compute one 256 x 128
// tile together -- each loads its 128 rows of A and 64 of the 128 rows of B, the first CTA
// (rank 0) issues the M = 256 MMAs for both, and each CTA's epilogue reads its own TMEM rows.
// Every shared-memory operand byte then serves twice the MMA work of the single-CTA form.
template <int SMAX, int CMAX, bool PAIR, bool GROUPED>
__global__ void __launch_bounds__(NTHREADS, 1)
k_digit_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
             const GemmArgs a) {
    // stages: single CTA 3 x 2 k-blocks (32 KB A + 32 KB B); pair 3 x 3 k-blocks (48 KB A +
    // 24 KB B), i.e. one barrier wait per 8 (single) or 12 (pair) MMAs
    constexpr int KS = PAIR ? 3 : KSTEP;
    constexpr int NST = STAGES;
    constexpr uint32_t BOXB = PAIR ? BOX_B / 2 : BOX_B;
    constexpr uint32_t STA = KS * BOX_A;
    constexpr uint32_t STB = KS * BOXB;
    static_assert(NST * (STA + STB) + 256 <= COLSTAT_OFF, "stage ring");
    static_assert(GARGS_OFF + GARGS_BYTES + 1024 <= 227 * 1024, "shared memory");
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem;
    uint8_t* sB = smem + NST * STA;
    uint64_t* bars = (uint64_t*)(sB + NST * STB);
    uint64_t* full = bars;
    uint64_t* empty = bars + NST;
    uint64_t* accfull = bars + 2 * NST;
    uint64_t* accempty = bars + 2 * NST + 2;
    uint64_t* drain = bars + 2 * NST + 4;
    uint32_t* tmem_holder = (uint32_t*)(bars + 2 * NST + 5);
    volatile int* abort_flag = (volatile int*)(tmem_holder + 1);
    // column statistics of the epilogue's current tile: e (as int bits), ||y^||, rho, sB, max_c ||d_c(y)||
    float* s_col = (float*)(smem + COLSTAT_OFF);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = PAIR ? cluster_rank() : 0u;
    // work unit: a CTA, or a CTA pair (consecutive blocks of a cluster)
    const int unit = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int nunits = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&accfull[b]), 1);
            mbar_init(smem_u32(&accempty[b]), (PAIR ? 64 : 32) * EPI_WARPS);   // both CTAs' epilogues drain
        }
        mbar_init(smem_u32(drain), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (!GROUPED && warp == 0 && lane == 0) {
        asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmB) : "memory");
    }
    if (warp == 1) {
        if (PAIR) {
            tmem_alloc_pair(smem_u32(tmem_holder), TMEM_COLS);   // both CTAs, same columns
        } else {
            tmem_alloc(smem_u32(tmem_holder), TMEM_COLS);
            tmem_relinquish();
        }
    }
    tc_fence_before();
    if (PAIR) cluster_sync_all();   // the peer's barriers are initialised before any remote use
    else __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            uint32_t stage = 0, phase = 0;
            uint32_t issued_mask = 0, last_par = 0;
            bool ok = true;
            for (int t = unit; t < a.ntiles && ok; t += nunits) {
                const Tile tl = a.tiles[t];
                if (tl.group < 0) continue;   // an empty slot of the schedule
                const GemmArgs& g = group_args<GROUPED>(a, tl);
                const CUtensorMap* mapA = GROUPED ? &a.groups[tl.group].tmA : &tmA;
                const CUtensorMap* mapB = GROUPED ? &a.groups[tl.group].tmB : &tmB;
                if (GROUPED) {   // the tile's tensor maps live in global memory: fetch them early
                    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)mapA) : "memory");
                    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)mapB) : "memory");
                }
                const Prod* prods = g.prods;
                const int nprods = g.nprods, nchunks = g.nchunks;
                for (int p = 0; p < nprods && ok; ++p) {
                    const Prod pr = prods[p];
                    int lo, hi;
                    chunk_range(tl.nkb, nchunks, pr.chunk, &lo, &hi);
                    // one stage holds up to KS consecutive k-blocks of the pass
                    for (int kb = lo; kb < hi; kb += KS) {
                        const int nk = hi - kb < KS ? hi - kb : KS;
                        if (!mbar_wait(smem_u32(&empty[stage]), phase ^ 1, abort_flag, a.err, 1)) {
                            ok = false;
                            break;
                        }
                        if (PAIR) {
                            // both CTAs' copies complete on the first CTA's barrier, which expects
                            // the bytes of both
                            const uint32_t fb = cluster_map(smem_u32(&full[stage]), 0);
                            if (rank == 0) mbar_expect_tx(smem_u32(&full[stage]), 2u * (uint32_t)nk * (BOX_A + BOXB));
                            for (int h = 0; h < nk; ++h) {
                                tma_load_3d_pair(smem_u32(sA + stage * STA + h * BOX_A), mapA, fb,
                                                 tl.a_k0 + (kb + h) * BK, tl.m0 + (int)rank * BM, pr.ia);
                                tma_load_3d_pair(smem_u32(sB + stage * STB + h * BOXB), mapB, fb,
                                                 tl.b_k0 + (kb + h) * BK, tl.n0 + (int)rank * (BN / 2), pr.ib);
                            }
                        } else {
                            const uint32_t fb = smem_u32(&full[stage]);
                            mbar_expect_tx(fb, (uint32_t)nk * (BOX_A + BOX_B));
                            for (int h = 0; h < nk; ++h) {
                                tma_load_3d(smem_u32(sA + stage * STA + h * BOX_A), mapA, fb,
                                            tl.a_k0 + (kb + h) * BK, tl.m0, pr.ia);
                                tma_load_3d(smem_u32(sB + stage * STB + h * BOXB), mapB, fb,
                                            tl.b_k0 + (kb + h) * BK, tl.n0, pr.ib);
                            }
                        }
                        issued_mask |= 1u << stage;
                        last_par = (last_par & ~(1u << stage)) | (phase << stage);
                        if (++stage == NST) { stage = 0; phase ^= 1; }
                    }
                }
            }
            if (!ok) {
                // let the copies already issued land before the CTA leaves (the second CTA of a
                // pair cannot observe the first's barrier: it allows them 100 us)
                if (!PAIR || rank == 0) {
                    for (int s = 0; s < NST; ++s)
                        if (issued_mask & (1u << s))
                            mbar_wait(smem_u32(&full[s]), (last_par >> s) & 1, abort_flag, a.err, 1, true);
                } else {
                    const unsigned long long t0 = globaltimer();
                    while (globaltimer() - t0 < 100000ull) {
                    }
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer (one thread; of the first CTA of a pair)
        if (lane == 0 && rank == 0) {
            uint32_t stage = 0, phase = 0, acc_cnt = 0;
            bool ok = true, any = false;
            for (int t = unit; t < a.ntiles && ok; t += nunits) {
                const Tile tl = a.tiles[t];
                if (tl.group < 0) continue;   // an empty slot of the schedule
                const GemmArgs& g = group_args<GROUPED>(a, tl);
                const Prod* prods = g.prods;
                const int nprods = g.nprods, nchunks = g.nchunks;
                for (int p = 0; p < nprods && ok; ++p) {
                    const Prod pr = prods[p];
                    int lo, hi;
                    chunk_range(tl.nkb, nchunks, pr.chunk, &lo, &hi);
                    if (hi <= lo) continue;
                    const uint32_t b = acc_cnt & 1, aphase = (acc_cnt >> 1) & 1;
                    if (pr.open) {   // a new accumulator: wait until the epilogue drained it
                        if (!mbar_wait(smem_u32(&accempty[b]), aphase ^ 1, abort_flag, a.err, 2)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    const uint32_t d = tmem + b * BN;
                    for (int kb = lo; kb < hi; kb += KS) {
                        const int nk = hi - kb < KS ? hi - kb : KS;
                        if (!mbar_wait(smem_u32(&full[stage]), phase, abort_flag, a.err, 3)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint64_t ad = smem_desc(smem_u32(sA + stage * STA));
                        const uint64_t bd = smem_desc(smem_u32(sB + stage * STB));
                        // second k-block of a stage: its boxes start BOX_A / BOXB bytes further
                        // (descriptor address units of 16 B)
#pragma unroll
                        for (int h = 0; h < KS; ++h) {
                            if (h < nk) {
#pragma unroll
                                for (int kk = 0; kk < BK / 16; ++kk) {
                                    const uint32_t acc = (!pr.open || kb > lo || h > 0 || kk > 0) ? 1u : 0u;
                                    const uint64_t a2 = ad + h * (BOX_A >> 4) + 2 * kk;
                                    const uint64_t b2 = bd + h * (BOXB >> 4) + 2 * kk;
                                    if (PAIR) mma_bf16_pair(d, a2, b2, kIdescPair, acc);
                                    else mma_bf16(d, a2, b2, kIdesc, acc);
                                }
                            }
                        }
                        any = true;
                        if (PAIR) mma_commit_pair(smem_u32(&empty[stage]), (uint16_t)3);
                        else mma_commit(smem_u32(&empty[stage]));
                        if (++stage == NST) { stage = 0; phase ^= 1; }
                    }
                    if (!ok) break;
                    if (pr.close) {   // the group is complete: hand the accumulator over
                        if (PAIR) mma_commit_pair(smem_u32(&accfull[b]), (uint16_t)3);
                        else mma_commit(smem_u32(&accfull[b]));
                        ++acc_cnt;
                    }
                }
            }
            if (any) {
                // all MMAs of this CTA (pair) complete before TMEM is released
                if (PAIR) mma_commit_pair(smem_u32(drain), (uint16_t)1);
                else mma_commit(smem_u32(drain));
                mbar_wait(smem_u32(drain), 0, abort_flag, a.err, 4, true);
            }
        }
    } else {
        // ---------------- epilogue: warps 2.., one TMEM lane (output row) per thread, each
        // warp half of the tile's columns (c0: its first 32-column group)
        // Each digit product arrives as an FP32 accumulator holding an exact integer (|acc| <
        // 2^24 where certified).  It is added, shifted to its weight, into an int64 fixed-point
        // running sum (TMEM columns 256..383 low words, 384..511 high words); only the
        // weights below 2^{-kFixTotal} are truncated (floor), at most one unit per product.
        const int q = warp & 3;
        const int row_in_tile = q * 32 + lane;
        const int c0 = ((warp - 2) / 4) * EPI_GROUPS;   // this warp's first 32-column group
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        const float two24 = 16777216.0f;
        uint32_t acc_cnt = 0;
        bool ok = true;
        for (int t = unit; t < a.ntiles && ok; t += nunits) {
            const Tile tl = a.tiles[t];
            if (tl.group < 0) continue;   // an empty slot of the schedule
            // the previous tile's finalisation has read its shared-memory statistics (every
            // epilogue warp gets here: none has left since the vote before that finalisation,
            // which has no waits)
            epilogue_sync();
            const Prod* prods;
            int nprods, nchunks, beta;
            {
                const GemmArgs& g = group_args<GROUPED>(a, tl);
                prods = g.prods;
                nprods = g.nprods;
                nchunks = g.nchunks;
                beta = g.beta;
                // The tile's column statistics, one column per epilogue thread, into shared
                // memory (computed while the tile's first products run; the finalisation reads
                // them as broadcasts).
                if constexpr (GROUPED) {   // the tile's arguments for the finalisation
                    static_assert(sizeof(GemmArgs) % 4 == 0, "word copy");
                    const uint32_t* src = reinterpret_cast<const uint32_t*>(&a.groups[tl.group].args);
                    uint32_t* dst = reinterpret_cast<uint32_t*>(smem + GARGS_OFF);
                    for (int w = (warp - 2) * 32 + lane; w < (int)(sizeof(GemmArgs) / 4); w += 32 * EPI_WARPS)
                        dst[w] = src[w];
                }
                if (c0 == 0) {
                    const int ncol = tl.n0 + row_in_tile;
                    const int sl = g.slices;
                    const float* dvB = g.B.dnv + (long)ncol * MAX_SLICES;
                    const float* rvB = g.B.rnv + (long)ncol * MAX_SLICES;
                    float crho = 0.0f, csB = 0.0f, cdnmax = 0.0f;
                    for (int k = 0; k < sl; ++k) {
                        crho = fmaxf(crho, __fmul_ru(__ldg(&rvB[k]), pow2f((k + 1) * beta)));
                        csB = __fadd_ru(csB, __fmul_ru(pow2f(-(k + 1) * beta), __ldg(&dvB[k])));
                    }
                    for (int cc = 0; cc < nchunks; ++cc)
                        cdnmax = fmaxf(cdnmax, __ldg(&g.B.dn[(long)ncol * nchunks + cc]));
                    s_col[0 * BN + row_in_tile] = __int_as_float(__ldg(&g.B.e[ncol]));
                    s_col[1 * BN + row_in_tile] = __ldg(&g.B.l2[ncol]);   // 0 exactly for an all-zero column
                    s_col[2 * BN + row_in_tile] = crho;
                    s_col[3 * BN + row_in_tile] = csB;
                    s_col[4 * BN + row_in_tile] = cdnmax;
                }
            }
            bool first = true;
            for (int p = 0; p < nprods && ok; ++p) {
                const Prod pr = prods[p];
                int lo, hi;
                chunk_range(tl.nkb, nchunks, pr.chunk, &lo, &hi);
                if (hi <= lo || !pr.close) continue;   // drained once per (fused) group
                const uint32_t b = acc_cnt & 1, aphase = (acc_cnt >> 1) & 1;
                if (!mbar_wait(smem_u32(&accfull[b]), aphase, abort_flag, a.err, 5)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int sh = fix_bits(beta) - pr.t * beta;
#pragma unroll 1
                for (int c = 2 * c0; c < 2 * (c0 + EPI_GROUPS); ++c) {   // 16-column pieces
                    uint32_t acc[16], lo_r[16], hi_r[16];
                    tmem_ld16(tmem + lane_off + b * BN + c * 16, acc);
                    if (!first) {
                        tmem_ld16(tmem + lane_off + 256 + c * 16, lo_r);
                        tmem_ld16(tmem + lane_off + 384 + c * 16, hi_r);
                    }
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const long long ai = (long long)__float2int_rz(__uint_as_float(acc[j]));
                        const long long v = sh >= 0 ? (ai << sh) : (ai >> (-sh));
                        long long run = first ? 0ll
                                              : (long long)(((unsigned long long)hi_r[j] << 32) | lo_r[j]);
                        run += v;
                        lo_r[j] = (uint32_t)(unsigned long long)run;
                        hi_r[j] = (uint32_t)((unsigned long long)run >> 32);
                    }
                    tmem_st16(tmem + lane_off + 256 + c * 16, lo_r);
                    tmem_st16(tmem + lane_off + 384 + c * 16, hi_r);
                }
                tmem_wait_st();
                tc_fence_before();
                if (PAIR && rank != 0) mbar_arrive_cluster(cluster_map(smem_u32(&accempty[b]), 0));
                else mbar_arrive(smem_u32(&accempty[b]));
                ++acc_cnt;
                first = false;
            }
            // every column's statistics are in place; all epilogue warps leave together if any
            // of them gave up on a drain
            if (epilogue_sync_any(!ok)) {
                ok = false;
                break;
            }
            // The finalisation reads many of the tile's arguments for every output.  A grouped
            // launch keeps them in global memory, where any store of an output might alias them
            // and force them to be read again: it reads the copy in shared memory.
            const GemmArgs& g = GROUPED ? *reinterpret_cast<const GemmArgs*>(smem + GARGS_OFF) : a;
            const int s = g.slices;
            // ---- finalize the tile: value, certified bound (Cauchy-Schwarz), flags.
            // Row terms live in registers; the column statistics come from shared memory.
            const int r = tl.m0 + (int)rank * BM + row_in_tile;
            const bool rvalid = r < g.rows_valid;
            // products summed in one accumulator: every partial sum of up to `fuse` exact
            // integer dot products stays below 2^24 when fuse max_c ||d_c(x)|| ||d_c(y)|| does
            const float fuse = g.fuse > 1 ? (float)g.fuse : 1.0f;
            const int eA = g.A.e[r];
            const int nnzA = g.A.nnz[r];
            const float l2A = g.A.l2[r];
            const float inA = g.A.inerr ? g.A.inerr[r] : 0.0f;
            const float* dvA = g.A.dnv + (long)r * MAX_SLICES;
            const float* rvA = g.A.rnv + (long)r * MAX_SLICES;
            const float rlastA = rvA[s - 1];
            // Row terms of the certificates.  The cheap forms need one value per column (all
            // rounded up):
            //   exactness   max_c ||d_c(x)|| max_c ||d_c(y)|| < 2^24 implies every chunk's test;
            //   error       sum_i 2^{-(i+1)b} ||d_i(x)|| ||y^ - Y^(s-1-i)|| <= sigA rhoB with
            //               sigA = 2^{-(s+1)b} sum_i ||d_i(x)||, rhoB = max_k ||y^ - Y^(k)|| 2^{(k+1)b},
            // so rlastA l2B + sigA rhoB bounds the first of the two operand orders.  Outputs
            // that fail a cheap test are checked again with the exact per-chunk and two-order
            // forms, which read the column's statistics directly.
            float dnAmax = 0.0f, sA = 0.0f, sumdA = 0.0f;
            for (int c = 0; c < g.nchunks; ++c) dnAmax = fmaxf(dnAmax, g.A.dn[(long)r * g.nchunks + c]);
            for (int i = 0; i < s; ++i) {
                const float dv = dvA[i];
                // |running sum| <= 2^kFixTotal SA SB, S = sum_i 2^{-(i+1) beta} ||d_i||: below 2^62
                // (SA SB < 2^12) the int64 recombination cannot overflow
                sA = __fmaf_ru(pow2f(-(i + 1) * g.beta), dv, sA);
                sumdA = __fadd_ru(sumdA, dv);
            }
            const float sigA = __fmul_ru(sumdA, pow2f(-(s + 1) * g.beta));
            const float cf64A = __fmul_ru(g.c_f64, l2A);
            float rowerr2 = 0.0f;
            unsigned long long vmax = 0ull;
            double* orow = g.out + (long)r * g.ldo;
            float* brow = g.bnd ? g.bnd + (long)r * g.ldb : nullptr;
#pragma unroll 1
            for (int c = c0; c < c0 + EPI_GROUPS; ++c) {
#pragma unroll 1
                for (int h = 0; h < 2; ++h) {
                    // this thread's 16 outputs leave as eight 16-byte stores (and four for the
                    // bounds) instead of sixteen 8-byte ones
                    double2* o2 = reinterpret_cast<double2*>(orow + tl.n0 + c * 32 + h * 16);
                    float4* b4 = brow ? reinterpret_cast<float4*>(brow + tl.n0 + c * 32 + h * 16) : nullptr;
                    unsigned long long vout[16];
                    float bout[16];
                    uint32_t lo_r[16], hi_r[16];
                    if (!first) {
                        tmem_ld16(tmem + lane_off + 256 + c * 32 + h * 16, lo_r);
                        tmem_ld16(tmem + lane_off + 384 + c * 32 + h * 16, hi_r);
                        tmem_wait_ld();
                    } else {
#pragma unroll
                        for (int j = 0; j < 16; ++j) { lo_r[j] = 0u; hi_r[j] = 0u; }
                    }
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int cl = c * 32 + h * 16 + j;   // the column within the tile
                        const int col = tl.n0 + cl;
                        const long long run = (long long)(((unsigned long long)hi_r[j] << 32) | lo_r[j]);
                        const int eB = __float_as_int(s_col[0 * BN + cl]);
                        const float l2B = s_col[1 * BN + cl];
                        const float rhoB = s_col[2 * BN + cl];
                        const float sB = s_col[3 * BN + cl];
                        const float dnBmax = s_col[4 * BN + cl];
                        float av;
                        const unsigned long long vbits = scaled_bits(run, eA + eB - kFixTotal, &av);
                        vout[j] = vbits;
                        bout[j] = 0.0f;
                        // the row's 16 columns are contiguous and 16-byte aligned (the leading
                        // dimensions are multiples of 128 columns): pairs of values and quads of
                        // bounds leave as 16-byte stores once complete
                        if (j & 1)
                            o2[j >> 1] = make_double2(__longlong_as_double((long long)vout[j - 1]),
                                                      __longlong_as_double((long long)vbits));
                        if (nnzA == 0 || l2B == 0.0f) {   // an exact zero
                            if (b4 && (j & 3) == 3) b4[j >> 2] = make_float4(bout[j - 3], bout[j - 2], bout[j - 1], 0.0f);
                            continue;
                        }
                        bool exact = __fmul_ru(sA, sB) < 4096.0f;
                        if (exact && __fmul_ru(__fmul_ru(dnAmax, dnBmax), fuse) >= two24) {
                            for (int cc = 0; cc < g.nchunks; ++cc)
                                if (__fmul_ru(__fmul_ru(g.A.dn[(long)r * g.nchunks + cc],
                                                        __ldg(&g.B.dn[(long)col * g.nchunks + cc])),
                                              fuse) >= two24)
                                    exact = false;
                        }
                        const float f64b = __fmul_ru(cf64A, l2B);
                        const float limit = g.flag_mode == 1 ? fmaxf(g.tol * av, f64b) : f64b;
                        float bound = __fadd_ru(__fmaf_ru(rlastA, l2B, __fmul_ru(sigA, rhoB)), g.c_fix);
                        bound = __fmaf_ru(inA, l2B, bound);
                        if (g.flag_mode != 0 && bound > limit) {
                            // |x^ y^ - C| <= ||x^ - X|| ||y^|| + sum_i 2^{-(i+1)b} ||d_i(x)|| ||y^ - Y^(s-1-i)||
                            // and the same with x and y exchanged; the smaller of the two holds
                            const float* cdv = g.B.dnv + (long)col * MAX_SLICES;
                            const float* crv = g.B.rnv + (long)col * MAX_SLICES;
                            float bA = __fmul_ru(rlastA, l2B);
                            float bB = __fmul_ru(__ldg(&crv[s - 1]), l2A);
                            for (int i = 0; i < s; ++i) {
                                const float w = pow2f(-(i + 1) * g.beta);
                                bA = __fmaf_ru(__fmul_ru(w, dvA[i]), __ldg(&crv[s - 1 - i]), bA);
                                bB = __fmaf_ru(__fmul_ru(w, __ldg(&cdv[i])), rvA[s - 1 - i], bB);
                            }
                            bound = __fmaf_ru(inA, l2B, __fadd_ru(fminf(bA, bB), g.c_fix));
                        }
                        if (exact && rvalid && col < g.cols_valid) {
                            const unsigned long long vb = vbits & 0x7FFFFFFFFFFFFFFFull;
                            vmax = vb > vmax ? vb : vmax;
                        }
                        {
                            // absolute bound: units 2^{eA+eB}; below float's normal range the
                            // smallest normal scale over-states it (still a bound)
                            const int es = eA + eB;
                            bout[j] = !exact || es > 127 ? __int_as_float(0x7f800000)
                                                         : __fmul_ru(bound, pow2f(max(es, -126)));
                            if (b4 && (j & 3) == 3) b4[j >> 2] = make_float4(bout[j - 3], bout[j - 2], bout[j - 1], bout[j]);
                        }
                        if (g.rowerr2) {
                            const float bb = __fmul_ru(bound, pow2f(max(-126, min(127, eB))));
                            rowerr2 = __fmaf_ru(bb, bb, rowerr2);
                        }
                        // certification: flag_mode 1 -> within max(tol |value|, FP64 bound of the
                        // same dot product); flag_mode 2 -> within the FP64 bound (FP64-grade)
                        const bool flag = !exact || (g.flag_mode != 0 && bound > limit);
                        if (flag && rvalid && col < g.cols_valid) {
                            const unsigned int idx = atomicAdd(g.nflags, 1u);
                            if ((int)idx < g.max_flags) g.flags[idx] = make_int2(r, col);
                        }
                    }
                }
            }
            if (g.absmax && vmax) atomicMax(g.absmax, vmax);
            if (g.rowerr2 && rvalid && rowerr2 > 0.0f) atomicAdd(&g.rowerr2[r], rowerr2);
            // make sure TMEM reads finished before the next tile overwrites the running sums
            tc_fence_before();
        }
    }
    tc_fence_before();
    // a pair stays together until the first CTA's MMAs (which read the second's shared memory
    // and write its TMEM) have drained
    if (PAIR) cluster_sync_all();
    else __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        if (PAIR) tmem_dealloc_pair(tmem, TMEM_COLS);
        else tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ------------------------------------------------------------------- slicing
__device__ __forceinline__ unsigned long long rne_shr(unsigned long long m, int k) {
    if (k <= 0) return m;
    if (k > 55) return 0ull;
    const unsigned long long q = m >> k;
    const unsigned long long rem = m & ((1ull << k) - 1ull);
    const unsigned long long half = 1ull << (k - 1);
    return (rem > half || (rem == half && (q & 1ull))) ? q + 1ull : q;
}

// Rows of at most kShortRow destination columns are sliced by 128 threads (flag
// kShortRowKernel in the kernel code), longer ones by 256.
constexpr int kShortRow = 4096;
constexpr int kShortRowKernel = 16;

// The slicing of output row `flat` of a grouped launch: the block copies that slicing's
// arguments to shared memory (in global memory any digit store might alias them, and copies
// in registers would cost the kernel half its resident blocks) and returns the row within it.
// The caller's previous row has passed its closing barrier.
__device__ __forceinline__ int slice_group_row(const SliceGroups& gs, int flat, SliceArgs* sa) {
    int lo = 0, hi = gs.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (gs.offs[mid] <= flat) lo = mid;
        else hi = mid - 1;
    }
    static_assert(sizeof(SliceArgs) % 4 == 0, "word copy");
    const uint32_t* src = reinterpret_cast<const uint32_t*>(gs.args + lo);
    uint32_t* dst = reinterpret_cast<uint32_t*>(sa);
    for (int w = threadIdx.x; w < (int)(sizeof(SliceArgs) / 4); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    return flat - gs.offs[lo];
}

template <bool G, int NT>
__device__ __forceinline__ void slice_rows(const SliceArgs& a0, const SliceGroups& gs) {
    const int tid = threadIdx.x;
    // one row per iteration; the grid may be smaller than the row count (a capped grid
    // leaves room on every SM for a concurrent kernel)
    __shared__ SliceArgs sa;   // grouped launch: the current row's slicing
    const int nflat = G ? gs.rows : a0.nrows;
    for (int flat = blockIdx.x; flat < nflat; flat += gridDim.x) {
        const int row = G ? slice_group_row(gs, flat, &sa) : flat;
        const SliceArgs& a = G ? sa : a0;
        const long srow = a.src_rows ? (long)a.src_rows[row] : (long)row;
        const unsigned long long* src = (const unsigned long long*)(a.src + srow * a.ld_src);
        __shared__ unsigned long long red_u[NT / 32];
        __shared__ float red_f[NT / 32];
        __shared__ int red_i[NT / 32];
        __shared__ float red_t[NT / 32][MAX_SLICES];
        __shared__ unsigned int red_d[NT / 32][MAX_SLICES * MAX_CHUNKS];

        // pass 1: max |x| through the IEEE bit pattern (integer compares only)
        unsigned long long mx = 0;
        for (int c = tid; c < a.ncols; c += NT) {
            const unsigned long long b = src[c] & 0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
            mx = y > mx ? y : mx;
        }
        if ((tid & 31) == 0) red_u[tid >> 5] = mx;
        __syncthreads();
        mx = 0;
        for (int w = 0; w < NT / 32; ++w) mx = red_u[w] > mx ? red_u[w] : mx;
        if (mx >= 0x7FF0000000000000ull) mx = 0x7FEFFFFFFFFFFFFFull;   // non-finite input: clamp scale
        const int Emax = (int)(mx >> 52);
        const bool zero_row = (mx == 0);
        const int e = zero_row ? 0 : (Emax > 0 ? Emax - 1022 : -1022);
        const int s = a.slices, beta = a.beta;
        const int q = s * beta;
        const long sstride = a.slice_stride;
        __nv_bfloat16* drow = a.digits + (long)row * a.kpad;

        int nnz = 0;
        float l2sq = 0.0f;
        float tsq[MAX_SLICES];
    #pragma unroll
        for (int i = 0; i < MAX_SLICES; ++i) tsq[i] = 0.0f;
        const long mask = (1l << beta) - 1l, halfb = 1l << (beta - 1);
        const float inv2q = pow2f(-q);
        // source columns come in chunk order (the column map is increasing): chunk ch covers
        // src_chunk[ch] .. src_chunk[ch+1]
        for (int ch = 0; ch < a.nchunks; ++ch) {
        unsigned int dsq[MAX_SLICES];
    #pragma unroll
        for (int i = 0; i < MAX_SLICES; ++i) dsq[i] = 0u;
        const int cend = a.src_chunk[ch + 1];
        for (int c = a.src_chunk[ch] + tid; c < cend; c += NT) {
            const unsigned long long bits = src[c];
            const int dc = a.col_map ? a.col_map[c] : c;
            const unsigned long long ab = bits & 0x7FFFFFFFFFFFFFFFull;
            long long I = 0;
            if (!zero_row && ab != 0 && ab < 0x7FF0000000000000ull) {
                const int E = (int)(ab >> 52);
                unsigned long long mant = ab & 0xFFFFFFFFFFFFFull;
                int ex;
                if (E > 0) { mant |= 1ull << 52; ex = E - 1075; }
                else ex = -1074;
                const int sh = ex + q - e;
                const unsigned long long m = sh >= 0 ? (mant << sh) : rne_shr(mant, -sh);
                I = (bits >> 63) ? -(long long)m : (long long)m;
            }
            long long v = I;
            int d[MAX_SLICES];
    #pragma unroll
            for (int i = MAX_SLICES - 1; i >= 1; --i) {
                if (i < s) {
                    long r = (long)(v & mask);
                    if (r > halfb) r -= (1l << beta);
                    d[i] = (int)r;
                    v = (v - r) >> beta;
                } else {
                    d[i] = 0;
                }
            }
            d[0] = (int)v;
            // tails x^(rounded) - X^(n) = sum_{i>n} d_i 2^{-(i+1) beta}, squared into tsq[n]
            float tail = 0.0f;
    #pragma unroll
            for (int i = MAX_SLICES - 1; i >= 1; --i) {
                if (i < s) {
                    tail = __fadd_rn(tail, (float)d[i] * pow2f(-(i + 1) * beta));
                    tsq[i - 1] = __fmaf_ru(tail, tail, tsq[i - 1]);
                }
            }
    #pragma unroll
            for (int i = 0; i < MAX_SLICES; ++i) {
                if (i < s) {
                    drow[i * sstride + dc] = __float2bfloat16_rn((float)d[i]);
                    dsq[i] += (unsigned int)(d[i] * d[i]);
                }
            }
            if (I != 0) {
                ++nnz;
                const unsigned long long aI = (unsigned long long)(I < 0 ? -I : I);
                const float xv = __fmul_ru(__ull2float_ru(aI), inv2q);
                l2sq = __fmaf_ru(xv, xv, l2sq);
            }
        }
        // this chunk's digit sums of squares: warp partials into shared memory
    #pragma unroll
        for (int i = 0; i < MAX_SLICES; ++i) {
            for (int o = 16; o > 0; o >>= 1) dsq[i] += __shfl_xor_sync(0xffffffffu, dsq[i], o);
            if ((tid & 31) == 0) red_d[tid >> 5][i * MAX_CHUNKS + ch] = dsq[i];
        }
        }
        // block reductions
        for (int o = 16; o > 0; o >>= 1) {
            l2sq = __fadd_ru(l2sq, __shfl_xor_sync(0xffffffffu, l2sq, o));
            nnz += __shfl_xor_sync(0xffffffffu, nnz, o);
        }
    #pragma unroll
        for (int i = 0; i < MAX_SLICES; ++i)
            for (int o = 16; o > 0; o >>= 1) tsq[i] = __fadd_ru(tsq[i], __shfl_xor_sync(0xffffffffu, tsq[i], o));
        if ((tid & 31) == 0) {
            red_f[tid >> 5] = l2sq;
            red_i[tid >> 5] = nnz;
    #pragma unroll
            for (int i = 0; i < MAX_SLICES; ++i) red_t[tid >> 5][i] = tsq[i];
        }
        __syncthreads();
        if (tid == 0) {
            float L2 = 0.0f;
            int N = 0;
            for (int w = 0; w < NT / 32; ++w) { L2 = __fadd_ru(L2, red_f[w]); N += red_i[w]; }
            // rounding of x^ to q fractional bits: |delta| <= 2^{-q-1} per non-zero entry
            const float dq = __fmul_ru(__fsqrt_ru((float)N), pow2f(-q - 1));
            const float slack = 1.0f + 1.0e-6f;   // FP32 evaluation of the tails and sums
            a.st.e[row] = e;
            a.st.nnz[row] = N;
            a.st.l2[row] = __fadd_ru(__fmul_ru(__fsqrt_ru(L2), slack), dq);
            for (int i = 0; i < MAX_SLICES; ++i) {
                float tq = 0.0f;
                unsigned long long dd = 0;
                if (i < s) {
                    for (int w = 0; w < NT / 32; ++w) {
                        tq = __fadd_ru(tq, red_t[w][i]);
                        for (int c = 0; c < a.nchunks; ++c) dd += red_d[w][i * MAX_CHUNKS + c];
                    }
                }
                a.st.dnv[(long)row * MAX_SLICES + i] = i < s ? __fsqrt_ru(__ull2float_ru(dd)) : 0.0f;
                a.st.rnv[(long)row * MAX_SLICES + i] =
                    i < s ? __fadd_ru(__fmul_ru(__fsqrt_ru(tq), slack), dq) : 0.0f;
            }
            for (int c = 0; c < a.nchunks; ++c) {
                unsigned long long m = 0;
                for (int i = 0; i < s; ++i) {
                    unsigned long long t = 0;
                    for (int w = 0; w < NT / 32; ++w) t += red_d[w][i * MAX_CHUNKS + c];
                    m = t > m ? t : m;
                }
                a.st.dn[(long)row * a.nchunks + c] = __fsqrt_ru(__ull2float_ru(m));
            }
            if (a.st.inerr) {
                float v = 0.0f;
                if (a.inerr2_prev && !zero_row) {
                    const int de = a.e_prev[row] - e;
                    v = __fmul_ru(__fmul_ru(__fsqrt_ru(a.inerr2_prev[row]), 1.0001f), pow2f(max(-126, min(127, de))));
                    if (de > 127) v = __int_as_float(0x7f800000);   // cannot certify: infinite bound
                }
                a.st.inerr[row] = v;
            }
        }
        __syncthreads();   // the shared reduction buffers are reused by the next row
    }
}

// The same digits and row statistics as k_slice for a compile-time slice count S, walking
// the destination columns four at a time: col_inv gives each destination column's source
// column (-1: padding, stored as zero digits), each slice's four digits leave as one 8-byte
// store, and a chunk is a plain range of destination columns (the GEMM's k-block split).
//
// Digits: the balanced digits of the fixed-point integer I (d_i in [1 - 2^(beta-1), 2^(beta-1)]
// below the top one) are the plain base-2^beta digits of u = I + C, C = (2^(beta-1) - 1) times
// the sum of the lower digit weights, each shifted down by 2^(beta-1) - 1; the top digit is
// u >> beta (S - 1).  Every digit has at most 8 significant bits (|d| <= 2^beta <= 256), so its
// float is exact in BF16 and the BF16 bits are the float's upper half.
template <int S, bool G, int NT>
__device__ __forceinline__ void slice4_rows(const SliceArgs& a0, const SliceGroups& gs) {
    const int tid = threadIdx.x;
    __shared__ unsigned long long red_u[NT / 32];
    __shared__ float red_f[NT / 32];
    __shared__ int red_i[NT / 32];
    __shared__ float red_t[NT / 32][S];
    __shared__ unsigned int red_d[NT / 32][S * MAX_CHUNKS];
    __shared__ unsigned long long dsum[S * MAX_CHUNKS];   // per (slice, chunk): sum over the row
    __shared__ SliceArgs sa;   // grouped launch: the current row's slicing
    const int nflat = G ? gs.rows : a0.nrows;
    for (int flat = blockIdx.x; flat < nflat; flat += gridDim.x) {
        const int row = G ? slice_group_row(gs, flat, &sa) : flat;
        const SliceArgs& a = G ? sa : a0;
        const int nkb = a.kpad / BK;
        const int beta = a.beta;
        const int q = S * beta;
        const long long mask = (1ll << beta) - 1ll;
        const int off = (1 << (beta - 1)) - 1;
        long long C = 0;
#pragma unroll
        for (int k = 0; k < S - 1; ++k) C += (long long)off << (beta * k);
        const float inv2q = pow2f(-q);
        float w2[S];   // 2^{-(i+1) beta}
#pragma unroll
        for (int i = 0; i < S; ++i) w2[i] = pow2f(-(i + 1) * beta);
        const long srow = a.src_rows ? (long)a.src_rows[row] : (long)row;
        const unsigned long long* src = (const unsigned long long*)(a.src + srow * a.ld_src);

        // pass 1: max |x| through the IEEE bit pattern (integer compares only)
        unsigned long long mx = 0;
#pragma unroll 4
        for (int c = tid; c < a.ncols; c += NT) {
            const unsigned long long b = src[c] & 0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
            mx = y > mx ? y : mx;
        }
        if ((tid & 31) == 0) red_u[tid >> 5] = mx;
        __syncthreads();
        mx = 0;
        for (int w = 0; w < NT / 32; ++w) mx = red_u[w] > mx ? red_u[w] : mx;
        if (mx >= 0x7FF0000000000000ull) mx = 0x7FEFFFFFFFFFFFFFull;   // non-finite input: clamp scale
        const int Emax = (int)(mx >> 52);
        const bool zero_row = (mx == 0);
        const int e = zero_row ? 0 : (Emax > 0 ? Emax - 1022 : -1022);
        const long sstride = a.slice_stride;
        __nv_bfloat16* drow = a.digits + (long)row * a.kpad;

        int nnz = 0;
        float l2sq = 0.0f;
        float tsq[S];
#pragma unroll
        for (int i = 0; i < S; ++i) tsq[i] = 0.0f;
        for (int ch = 0; ch < a.nchunks; ++ch) {
            unsigned int dsq[S];
#pragma unroll
            for (int i = 0; i < S; ++i) dsq[i] = 0u;
            const int d0 = (int)(((long)ch * nkb) / a.nchunks) * BK;
            const int d1 = (int)(((long)(ch + 1) * nkb) / a.nchunks) * BK;
            for (int dc = d0 + 4 * tid; dc < d1; dc += 4 * NT) {
                uint32_t pk[S][2];
                uint32_t even[S];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int col = dc + u;
                    const int sc = a.col_inv ? a.col_inv[col] : (col < a.ncols ? col : -1);
                    const unsigned long long bits = sc >= 0 ? src[sc] : 0ull;
                    const unsigned long long ab = bits & 0x7FFFFFFFFFFFFFFFull;
                    long long I = 0;
                    if (!zero_row && ab != 0 && ab < 0x7FF0000000000000ull) {
                        const int E = (int)(ab >> 52);
                        unsigned long long mant = ab & 0xFFFFFFFFFFFFFull;
                        int ex;
                        if (E > 0) { mant |= 1ull << 52; ex = E - 1075; }
                        else ex = -1074;
                        const int sh = ex + q - e;
                        const unsigned long long m = sh >= 0 ? (mant << sh) : rne_shr(mant, -sh);
                        I = (bits >> 63) ? -(long long)m : (long long)m;
                    }
                    const long long uo = I + C;
                    int d[S];
#pragma unroll
                    for (int i = S - 1; i >= 1; --i)
                        d[i] = (int)(((unsigned long long)uo >> (beta * (S - 1 - i))) & mask) - off;
                    d[0] = (int)(uo >> (beta * (S - 1)));
                    // tails x^(rounded) - X^(n) = sum_{i>n} d_i 2^{-(i+1) beta}, squared into tsq[n]
                    float tail = 0.0f;
#pragma unroll
                    for (int i = S - 1; i >= 1; --i) {
                        tail = __fadd_rn(tail, (float)d[i] * w2[i]);
                        tsq[i - 1] = __fmaf_ru(tail, tail, tsq[i - 1]);
                    }
#pragma unroll
                    for (int i = 0; i < S; ++i) {
                        dsq[i] += (unsigned int)(d[i] * d[i]);
                        const uint32_t fb = __float_as_uint((float)d[i]);   // exact: BF16 = upper half
                        if (u & 1) pk[i][u >> 1] = __byte_perm(even[i], fb, 0x7632);
                        else even[i] = fb;
                    }
                    if (I != 0) {
                        ++nnz;
                        const unsigned long long aI = (unsigned long long)(I < 0 ? -I : I);
                        const float xv = __fmul_ru(__ull2float_ru(aI), inv2q);
                        l2sq = __fmaf_ru(xv, xv, l2sq);
                    }
                }
#pragma unroll
                for (int i = 0; i < S; ++i)
                    *reinterpret_cast<uint2*>(drow + i * sstride + dc) = make_uint2(pk[i][0], pk[i][1]);
            }
            // this chunk's digit sums of squares: warp partials into shared memory
#pragma unroll
            for (int i = 0; i < S; ++i) {
                for (int o = 16; o > 0; o >>= 1) dsq[i] += __shfl_xor_sync(0xffffffffu, dsq[i], o);
                if ((tid & 31) == 0) red_d[tid >> 5][i * MAX_CHUNKS + ch] = dsq[i];
            }
        }
        // block reductions
        for (int o = 16; o > 0; o >>= 1) {
            l2sq = __fadd_ru(l2sq, __shfl_xor_sync(0xffffffffu, l2sq, o));
            nnz += __shfl_xor_sync(0xffffffffu, nnz, o);
        }
#pragma unroll
        for (int i = 0; i < S; ++i)
            for (int o = 16; o > 0; o >>= 1) tsq[i] = __fadd_ru(tsq[i], __shfl_xor_sync(0xffffffffu, tsq[i], o));
        if ((tid & 31) == 0) {
            red_f[tid >> 5] = l2sq;
            red_i[tid >> 5] = nnz;
#pragma unroll
            for (int i = 0; i < S; ++i) red_t[tid >> 5][i] = tsq[i];
        }
        __syncthreads();
        // per (slice, chunk) sums over the warps, one thread each (integer: any order)
        if (tid < S * a.nchunks) {
            const int i = tid / a.nchunks, c = tid - i * a.nchunks;
            unsigned long long t = 0;
            for (int w = 0; w < NT / 32; ++w) t += red_d[w][i * MAX_CHUNKS + c];
            dsum[i * MAX_CHUNKS + c] = t;
        }
        __syncthreads();
        // rounding of x^ to q fractional bits: |delta| <= 2^{-q-1} per non-zero entry
        const float slack = 1.0f + 1.0e-6f;   // FP32 evaluation of the tails and sums
        if (tid < MAX_SLICES) {   // one slice per thread; tq in warp order as before
            const int i = tid;
            int N = 0;
            for (int w = 0; w < NT / 32; ++w) N += red_i[w];
            const float dq = __fmul_ru(__fsqrt_ru((float)N), pow2f(-q - 1));
            float tq = 0.0f;
            unsigned long long dd = 0;
            if (i < S) {
                for (int w = 0; w < NT / 32; ++w) tq = __fadd_ru(tq, red_t[w][i]);
                for (int c = 0; c < a.nchunks; ++c) dd += dsum[i * MAX_CHUNKS + c];
            }
            a.st.dnv[(long)row * MAX_SLICES + i] = i < S ? __fsqrt_ru(__ull2float_ru(dd)) : 0.0f;
            a.st.rnv[(long)row * MAX_SLICES + i] = i < S ? __fadd_ru(__fmul_ru(__fsqrt_ru(tq), slack), dq) : 0.0f;
        } else if (tid >= 32 && tid < 32 + a.nchunks) {   // one chunk per thread: the largest digit norm
            const int c = tid - 32;
            unsigned long long m = 0;
            for (int i = 0; i < S; ++i) m = dsum[i * MAX_CHUNKS + c] > m ? dsum[i * MAX_CHUNKS + c] : m;
            a.st.dn[(long)row * a.nchunks + c] = __fsqrt_ru(__ull2float_ru(m));
        } else if (tid == 64) {
            float L2 = 0.0f;
            int N = 0;
            for (int w = 0; w < NT / 32; ++w) { L2 = __fadd_ru(L2, red_f[w]); N += red_i[w]; }
            const float dq = __fmul_ru(__fsqrt_ru((float)N), pow2f(-q - 1));
            a.st.e[row] = e;
            a.st.nnz[row] = N;
            a.st.l2[row] = __fadd_ru(__fmul_ru(__fsqrt_ru(L2), slack), dq);
            if (a.st.inerr) {
                float v = 0.0f;
                if (a.inerr2_prev && !zero_row) {
                    const int de = a.e_prev[row] - e;
                    v = __fmul_ru(__fmul_ru(__fsqrt_ru(a.inerr2_prev[row]), 1.0001f), pow2f(max(-126, min(127, de))));
                    if (de > 127) v = __int_as_float(0x7f800000);   // cannot certify: infinite bound
                }
                a.st.inerr[row] = v;
            }
        }
        __syncthreads();   // the shared reduction buffers are reused by the next row
    }
}

// The slicing kernels: one slicing (its arguments in the parameter space), or a grouped
// launch of several, capped at 64 registers so that it keeps four resident blocks per SM (a
// row's work is short and latency-bound).  NT threads per row: 256, or 128 for rows of at
// most kShortRow destination columns (twice the rows in flight for the same threads).  The
// single and the grouped form pick NT the same way, so both produce the same statistics.
template <int NT>
__global__ void __launch_bounds__(NT) k_slice(const SliceArgs a) { slice_rows<false, NT>(a, SliceGroups{}); }
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_slice_grouped(const SliceGroups gs) {
    slice_rows<true, NT>(SliceArgs{}, gs);
}
template <int S, int NT>
__global__ void __launch_bounds__(NT) k_slice4(const SliceArgs a) { slice4_rows<S, false, NT>(a, SliceGroups{}); }
template <int S, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_slice4_grouped(const SliceGroups gs) {
    slice4_rows<S, true, NT>(SliceArgs{}, gs);
}

// ------------------------------------------------------------------- band builder
__device__ __forceinline__ double parity_sign(int x) { return (x & 1) ? -1.0 : 1.0; }

// The band entry of one (upper primitive rF, lower primitive rI) pair without coefficients
// (0 outside the dipole piece or the selection rules).
__device__ __forceinline__ double band_elem(const BandArgs& a, int rF, int rI) {
    const int vF = a.vibF[rF];
    if (vF < a.startF || vF >= a.endF) return 0.0;
    if (a.wigner) {
        const long d = (long)(vF - a.startF) + (long)a.vibI[rI] * a.ncontrF, ds = (long)a.dipN * a.ncontrF;
        const long wi = 3 * ((long)a.tauI[rI] + (long)a.nlevelI *
                             ((long)a.tauF[rF] + (long)a.nlevelF * ((long)a.KI[rI] + (long)a.maxdeg * a.KF[rF])));
        return __fma_rn(a.wigner[wi + 2], a.dipole[d + 2 * ds],
                        __fma_rn(a.wigner[wi], a.dipole[d], __dmul_rn(a.wigner[wi + 1], a.dipole[d + ds])));
    }
    const int kI = a.KI[rI], kF = a.KF[rF];
    if (abs(kI - kF) > 1) return 0.0;
    const int tI = a.tauI[rI], tF = a.tauF[rF] & 1;
    const int eq = (kF == kI), neq = !eq, tneq = (tF != tI);
    const int didx = 2 * eq + neq * (!tneq);
    const int c = (tF - tI) * eq + (tF - tI) * (kF - kI) * neq * tneq - neq * (!tneq);
    if (c == 0) return 0.0;
    const int n = a.jmax + 1;
    double m = a.threej[a.jI + kI * n + (a.jF - a.jI + 1) * n * n + (kF - kI + 1) * n * n * 3];
    if (kI != kF && kI * kF != 0) m = __dmul_rn(m, kSqrt2Ref);
    m = __dmul_rn(m, (double)c * parity_sign((kI % 3) * tI + kI) * parity_sign((kF % 3) * tF));
    const double mu = a.dipole[(long)(vF - a.startF) + (long)a.vibI[rI] * a.ncontrF + (long)didx * a.dipN * a.ncontrF];
    return __dmul_rn(m, mu);
}

__global__ void k_band(const BandArgs a) {
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)a.fpad * a.W) return;
    const int row = (int)(idx / a.W), w = (int)(idx - (long)row * a.W);
    const int kc = a.band_k0[row] + w;
    double val = 0.0;
    if (kc < a.kpadI) {
        if (a.f_ptr) {   // symmetric functions combining primitives: sum over both expansions
            for (int q = a.f_ptr[row]; q < a.f_ptr[row + 1]; ++q)
                for (int t = a.i_ptr[kc]; t < a.i_ptr[kc + 1]; ++t) {
                    const double e = band_elem(a, a.f_col[q], a.i_col[t]);
                    if (e != 0.0) val = __fma_rn(__dmul_rn(a.f_val[q], a.i_val[t]), e, val);
                }
        } else {
            const int rF = a.f_prim[row], rI = a.i_prim[kc];
            if (rF >= 0 && rI >= 0) {
                const double e = band_elem(a, rF, rI);
                if (e != 0.0) val = __dmul_rn(e, __dmul_rn(a.i_coef[kc], a.f_coef[row]));
            }
        }
    }
    a.band[idx] = val;
}

// Self-test of the bounded wait: an mbarrier nothing arrives on; the wait gives up after
// limit_ns, raises the abort flag and writes code 9 to err.
__global__ void k_wait_selftest(unsigned long long limit_ns, int* err) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait(smem_u32(&bar), 0, &abort_flag, err, 9, false, limit_ns);
    __syncthreads();
}

// ------------------------------------------------------------------- refinement
__global__ void k_refine_h(const RefineHArgs a) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = min((int)*a.nflags, a.max_flags);
    for (int f = gw; f < n; f += nw) {
        const int2 rc = a.flags[f];
        const int r = rc.x, c = rc.y;
        const double* v = a.vecs + (long)a.row_level[r] * a.nsize;
        const double* b = a.band + (long)c * a.W;
        const int k0 = a.band_k0[c], len = a.band_len[c];
        double acc = 0.0, aacc = 0.0;
        for (int w = lane; w < len; w += 32) {
            const int s = a.i_sym[k0 + w];
            if (s < 0) continue;
            const double p = v[s] * b[w];
            acc = __fma_rn(v[s], b[w], acc);
            aacc += fabs(p);
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
            aacc += __shfl_xor_sync(0xffffffffu, aacc, o);
        }
        if (lane == 0) {
            a.H[(long)r * a.ldh + c] = acc;
            // rounding error of this FP64 sum (gamma_n with n <= len + 32), in units of 2^{eA},
            // added to the row's sum of squared element bounds
            const double err = aacc * (double)(len + 64) * 1.1102230246251565e-16 * 1.01;
            const float u = __double2float_ru(err * pow2d(-a.eA[r]));
            atomicAdd(&a.rowerr2[r], __fmul_ru(u, u));
        }
    }
}

__global__ void k_refine_amp(const RefineAmpArgs a) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = min((int)*a.nflags, a.max_flags);
    for (int f = gw; f < n; f += nw) {
        const int2 rc = a.flags[f];
        const int r = rc.x, c = rc.y;
        const double* u = a.U + (long)a.col_level[c] * a.nsize;
        const double* h = a.H + (long)r * a.ldh;
        double acc = 0.0, aacc = 0.0, l2 = 0.0;
        for (int s = lane; s < a.nsize; s += 32) {
            const double uv = u[s], hv = h[a.colpos[s]];
            acc = __fma_rn(uv, hv, acc);
            aacc += fabs(uv * hv);
            l2 = __fma_rn(uv, uv, l2);
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(0xffffffffu, acc, o);
            aacc += __shfl_xor_sync(0xffffffffu, aacc, o);
            l2 += __shfl_xor_sync(0xffffffffu, l2, o);
        }
        if (lane == 0) {
            a.amp[(long)r * a.lda + c] = acc;
            // The recomputed amplitude now carries the FP64 method's own bound: the rounding
            // of this dot product plus the H error, which the first GEMM certified FP64-grade.
            // Lines where even that bound exceeds tol |amp| are counted (information only).
            const double f64b = aacc * (double)(a.nsize + 64) * 1.1102230246251565e-16 * 1.01;
            if (a.bnd) {
                const double herr = a.h_inerr ? (double)a.h_inerr[r] * pow2d(a.eH[r]) * sqrt(l2) * 1.01 : 0.0;
                a.bnd[(long)r * a.ldb + c] = __double2float_ru(f64b + herr);
            }
            if (!(f64b <= a.tol * fabs(acc))) {
                const double amax = __longlong_as_double((long long)*a.absmax);
                atomicAdd(fabs(acc) >= a.amp_floor * amax ? a.uncertified : a.uncertified_weak, 1ull);
            }
        }
    }
}

}  // namespace

size_t gemm_smem_bytes() {   // the larger of the two stage rings (the pair's three 72 KB stages)
    return (size_t)GARGS_OFF + GARGS_BYTES + 1024 /* align slack */;
}

// Kernel instances by (max slices, max chunks, pair): the two common configurations (first
// GEMM: up to 8 slices in one chunk; second GEMM: up to 6 slices in up to 8 chunks) and a
// general one, each as a single CTA and as a CTA pair.
typedef void (*GemmKernel)(const CUtensorMap, const CUtensorMap, const GemmArgs);
template <bool G>
static GemmKernel gemm_kernel_of(int slices, int chunks, bool pair) {
    if (slices <= 8 && chunks <= 1) return pair ? k_digit_gemm<8, 1, true, G> : k_digit_gemm<8, 1, false, G>;
    if (slices <= 6 && chunks <= MAX_CHUNKS)
        return pair ? k_digit_gemm<6, MAX_CHUNKS, true, G> : k_digit_gemm<6, MAX_CHUNKS, false, G>;
    return pair ? k_digit_gemm<MAX_SLICES, MAX_CHUNKS, true, G> : k_digit_gemm<MAX_SLICES, MAX_CHUNKS, false, G>;
}
static GemmKernel gemm_kernel_for(int slices, int chunks, bool pair, bool grouped = false) {
    return grouped ? gemm_kernel_of<true>(slices, chunks, pair) : gemm_kernel_of<false>(slices, chunks, pair);
}

// Function attributes are per device: set them once on each device that launches.
// All kernels ask for the largest shared-memory carveout.
static cudaError_t set_attributes_once() {
    static std::atomic<unsigned long long> done{0};   // bit per device ordinal (< 64)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return cudaSuccess;
    GemmKernel ks[12];
    const int cfg[3][2] = {{8, 1}, {6, MAX_CHUNKS}, {MAX_SLICES, MAX_CHUNKS}};
    for (int i = 0; i < 12; ++i)
        ks[i] = gemm_kernel_for(cfg[i % 3][0], cfg[i % 3][1], (i / 3) & 1, i >= 6);
    for (GemmKernel k : ks) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes());
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
    const void* slicers[] = {
        (const void*)k_slice<256>,             (const void*)k_slice<128>,
        (const void*)k_slice_grouped<256>,     (const void*)k_slice_grouped<128>,
        (const void*)k_slice4<6, 256>,         (const void*)k_slice4<6, 128>,
        (const void*)k_slice4<7, 256>,         (const void*)k_slice4<7, 128>,
        (const void*)k_slice4<8, 256>,         (const void*)k_slice4<8, 128>,
        (const void*)k_slice4_grouped<6, 256>, (const void*)k_slice4_grouped<6, 128>,
        (const void*)k_slice4_grouped<7, 256>, (const void*)k_slice4_grouped<7, 128>,
        (const void*)k_slice4_grouped<8, 256>, (const void*)k_slice4_grouped<8, 128>};
    for (const void* f : slicers)
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    done.fetch_or(bit);
    return cudaSuccess;
}

cudaError_t prepare_device() { return set_attributes_once(); }

cudaError_t launch_gemm(const CUtensorMap& tmA, const CUtensorMap& tmB, const GemmArgs& a, int num_sms,
                        cudaStream_t st, bool pair) {
    const size_t smem = gemm_smem_bytes();
    cudaError_t e = set_attributes_once();
    if (e != cudaSuccess) return e;
    if (a.ntiles <= 0) return cudaSuccess;
    if (a.slices < 1 || a.slices > MAX_SLICES || a.nchunks < 1 || a.nchunks > MAX_CHUNKS)
        return cudaErrorInvalidValue;
    GemmKernel k = gemm_kernel_for(a.slices, a.nchunks, pair);
    if (!pair) {
        const int grid = a.ntiles < num_sms ? a.ntiles : num_sms;
        k<<<grid, NTHREADS, smem, st>>>(tmA, tmB, a);
        return cudaGetLastError();
    }
    // pairs of CTAs (clusters of two), one pair per tile at most
    const int pairs = a.ntiles < num_sms / 2 ? a.ntiles : num_sms / 2;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(2 * pairs));
    cfg.blockDim = dim3(NTHREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, tmA, tmB, a);
}

cudaError_t launch_gemm_grouped(const GemmArgs& a, int units, int max_slices, int max_chunks, cudaStream_t st,
                                bool pair) {
    const size_t smem = gemm_smem_bytes();
    cudaError_t e = set_attributes_once();
    if (e != cudaSuccess) return e;
    if (a.ntiles <= 0 || units <= 0) return cudaSuccess;
    if (!a.groups || a.ntiles % units) return cudaErrorInvalidValue;
    if (max_slices < 1 || max_slices > MAX_SLICES || max_chunks < 1 || max_chunks > MAX_CHUNKS)
        return cudaErrorInvalidValue;
    GemmKernel k = gemm_kernel_for(max_slices, max_chunks, pair, true);
    const CUtensorMap unused = {};   // every tile's maps come from its group
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(pair ? 2 * units : units));
    cfg.blockDim = dim3(NTHREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = pair ? 2 : 1;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pair ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, unused, unused, a);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

bool make_digit_map(CUtensorMap* map, void* base, int kpad, int rows_pad, int slices, int box_rows) {
    // looked up once (thread-safe initialisation of a function-local static)
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult qr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) !=
                cudaSuccess || qr != cudaDriverEntryPointSuccess || !p)
            return nullptr;
        return (EncodeTiledFn)p;
    }();
    if (!fn) return false;
    if (((uintptr_t)base & 15) || (kpad % BK) || (rows_pad % BM)) return false;
    cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rows_pad, (cuuint64_t)slices};
    cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)kpad * 2 * (cuuint64_t)rows_pad};
    if (box_rows != BM && box_rows != BN / 2) return false;
    cuuint32_t box[3] = {BK, (cuuint32_t)box_rows, 1};
    cuuint32_t es[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_slice(const SliceArgs& a, cudaStream_t st) {
    if (a.nrows <= 0) return cudaSuccess;
    cudaError_t e = set_attributes_once();
    if (e != cudaSuccess) return e;
    const int grid = (a.grid_limit > 0 && a.grid_limit < a.nrows) ? a.grid_limit : a.nrows;
    const int k = slice_kernel_of(a);
    if (k & kShortRowKernel) {
        switch (k & 15) {
            case 6: k_slice4<6, 128><<<grid, 128, 0, st>>>(a); break;
            case 7: k_slice4<7, 128><<<grid, 128, 0, st>>>(a); break;
            case 8: k_slice4<8, 128><<<grid, 128, 0, st>>>(a); break;
            default: k_slice<128><<<grid, 128, 0, st>>>(a); break;
        }
    } else {
        switch (k) {
            case 6: k_slice4<6, 256><<<grid, 256, 0, st>>>(a); break;
            case 7: k_slice4<7, 256><<<grid, 256, 0, st>>>(a); break;
            case 8: k_slice4<8, 256><<<grid, 256, 0, st>>>(a); break;
            default: k_slice<256><<<grid, 256, 0, st>>>(a); break;
        }
    }
    return cudaGetLastError();
}

int slice_kernel_of(const SliceArgs& a) {
    // the four-column kernel needs the destination map (or the identity) and whole k-blocks
    const bool four = (a.col_inv || !a.col_map) && (a.kpad % BK) == 0;
    const int k = four && a.slices >= 6 && a.slices <= 8 ? a.slices : 0;
    return a.kpad <= kShortRow ? (k | kShortRowKernel) : k;
}

cudaError_t launch_slice_grouped(const SliceGroups& g, int kernel, cudaStream_t st) {
    if (g.rows <= 0 || g.n <= 0) return cudaSuccess;
    cudaError_t e = set_attributes_once();
    if (e != cudaSuccess) return e;
    if (kernel & kShortRowKernel) {
        switch (kernel & 15) {
            case 6: k_slice4_grouped<6, 128><<<g.rows, 128, 0, st>>>(g); break;
            case 7: k_slice4_grouped<7, 128><<<g.rows, 128, 0, st>>>(g); break;
            case 8: k_slice4_grouped<8, 128><<<g.rows, 128, 0, st>>>(g); break;
            default: k_slice_grouped<128><<<g.rows, 128, 0, st>>>(g); break;
        }
    } else {
        switch (kernel) {
            case 6: k_slice4_grouped<6, 256><<<g.rows, 256, 0, st>>>(g); break;
            case 7: k_slice4_grouped<7, 256><<<g.rows, 256, 0, st>>>(g); break;
            case 8: k_slice4_grouped<8, 256><<<g.rows, 256, 0, st>>>(g); break;
            default: k_slice_grouped<256><<<g.rows, 256, 0, st>>>(g); break;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_band(const BandArgs& a, cudaStream_t st) {
    const long total = (long)a.fpad * a.W;
    if (total <= 0) return cudaSuccess;
    k_band<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_refine_h(const RefineHArgs& a, int max_blocks, cudaStream_t st) {
    k_refine_h<<<max_blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_wait_selftest(unsigned long long limit_ns, int* err, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(limit_ns, err);
    return cudaGetLastError();
}

cudaError_t launch_refine_amp(const RefineAmpArgs& a, int max_blocks, cudaStream_t st) {
    k_refine_amp<<<max_blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace split
}  // namespace gain
