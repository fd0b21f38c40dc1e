// (c) Cross-covariance GEMMs on the 5th-generation tensor cores: tcgen05.mma
// (kind::f16, float32 accumulation) with TMEM accumulators, operands staged by
// TMA (cp.async.bulk.tensor, 128-byte swizzle). Float32 accuracy comes from a
// two-term float16 split of power-of-two-scaled operands,
//   a * b ~ ah*bh + ah*bl + al*bh,   ah = f16(s a), al = f16(s a - ah),
// which carries 22 significand bits like a two-term tf32 split, at twice the
// tf32 tensor rate and half the operand bytes. Power-of-two scales bring the
// largest entry of every operand row (A) and column (B) to at most 2^14, so the
// float16 subnormal floor sits about 2^-38 below it; the epilogue multiplies
// each output by row_mul[i] * col_mul[j] to undo them.
//
//   forward  V = Kc L^-T   (B operand stored as L^-1, K-major; k < n0 + BN)
//   adjoint  D = H  L^-1   (B operand stored as L^-T, K-major; k >= n0)
//
// Two forms share one kernel body. PAIR = 2 (the default): a cluster of two CTAs
// on two SMs computes a 256 x 256 tile of C with tcgen05.mma.cta_group::2
// (M = 256), each CTA staging its own 128 rows of A and 128 of the 256 rows of B,
// so each SM's shared memory feeds half of B per MMA; three stages of 64 KB.
// PAIR = 1: one CTA per 128 x 256 tile, two stages of 96 KB. Warp roles: warp 0
// issues the TMA loads (one elected lane; in the pair, each CTA its own rows,
// completing on the leader CTA's barrier), warp 1 owns the TMEM allocation and
// (leader CTA only) issues the MMAs, warps 2-9 drain the accumulators and store
// C through shared memory with TMA. The kernel is persistent: one CTA (cluster)
// per SM (pair) walks a static, work-balanced schedule of tiles, keeping TMEM
// and the pipeline across tiles.
//
// Accumulation: the K range is cut into chunks of TC_FLUSH k-blocks; each chunk
// is accumulated in one of two TMEM accumulators (ping-pong, 2 x 256 columns)
// while the epilogue warps add the previous chunk into float32 registers
// (round-to-nearest). Keeping each tensor-core accumulation short holds the
// split product to float32 accuracy over long K.
//
// Every mbarrier wait is bounded in time; on expiry the CTA records an error
// code, stops issuing work, waits (bounded) for its copies in flight, frees
// its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 64;  // BK: float16 elements (128 bytes)
constexpr int TC_UMMA_K = 16;                         // float16 K per tcgen05.mma
constexpr uint32_t A_TILE = TC_BM * TC_BK * 2;        // 16 KB
constexpr int TC_THREADS = 320;                       // 10 warps
constexpr int TC_FLUSH = 1;                           // k-blocks per TMEM accumulation chunk
constexpr uint32_t TMEM_COLS = 512;                   // two 128 x 256 float32 accumulators
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

// Tile geometry of the two forms. PAIR = 1: one CTA computes a 128 x 256 tile
// (B tile 256 rows), two stages of 96 KB. PAIR = 2 (cta_group::2): a cluster
// of two CTAs on two SMs computes a 256 x 256 tile with one M = 256 MMA; each
// CTA stages its own 128 rows of A and 128 of the 256 B rows, so the shared
// memory each SM reads per MMA halves; three stages of 64 KB. Both keep one
// 32 x 32 float32 staging tile per epilogue warp for the TMA stores of C.
template <int PAIR>
struct TcCfg {
    static constexpr int STAGES = PAIR == 2 ? 3 : 2;
    static constexpr int B_ROWS = TC_BN / PAIR;
    static constexpr uint32_t B_TILE = (uint32_t)B_ROWS * TC_BK * 2;
    static constexpr uint32_t STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
    static constexpr uint32_t TX_BYTES = STAGE_BYTES * PAIR;  // bytes that complete one stage
    static constexpr uint32_t STAGING = 8 * 32 * 32 * 4;      // 8 epilogue warps x 4 KB
    static constexpr size_t SMEM = STAGES * STAGE_BYTES + STAGING + 1024 /*align*/ + 256 /*barriers*/;
    // instruction descriptor (kind::f16): D f32, A/B f16, both K-major, N = 256, M = 128 PAIR
    static constexpr uint32_t IDESC = (1u << 4) | (0u << 7) | (0u << 10) |
                                      ((uint32_t)(TC_BN >> 3) << 17) |
                                      ((uint32_t)((TC_BM * PAIR) >> 4) << 24);
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t peer_addr(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}

__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Arrive on barrier `bar` of CTA `rank` of the cluster (PAIR = 2) or of this CTA.
// The arrival orders this thread's completed tcgen05.ld (after wait::ld and a
// tcgen05 fence) before the MMAs the waiting thread issues next; no
// cluster-scope memory fence is needed for that (one per arrival stalled the
// epilogue warps measurably).
template <int PAIR>
__device__ __forceinline__ void mbar_arrive(uint64_t* bar, uint32_t rank) {
    if constexpr (PAIR == 2) {
        asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(
                         peer_addr(smem_u32(bar), rank))
                     : "memory");
    } else {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
    }
}

// Wait for the phase with parity `phase` to complete; false after kWaitNs or
// as soon as another role of the CTA has recorded a failure in *fail.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase,
                                          const int* fail = nullptr) {
    const uint32_t addr = smem_u32(bar);
    const unsigned long long t0 = global_ns();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
        if (fail != nullptr && *(volatile const int*)fail != 0) return false;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

// 2-D tile load into this CTA's shared memory; completion is counted on the
// mbarrier at shared::cluster address `bar` (PAIR = 2: the leader CTA's).
template <int PAIR>
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint32_t bar, int x,
                                            int y) {
    if constexpr (PAIR == 2) {
        asm volatile(
            "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
            "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
            : "memory");
    } else {
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
            "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
            : "memory");
    }
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of 1024 bytes.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;                      // leading byte offset (unused here)
    d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;  // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1u << 46;                      // descriptor version
    d |= (uint64_t)2u << 61;                      // SWIZZLE_128B
    return d;
}

template <int PAIR>
__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
    if constexpr (PAIR == 2) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(TcCfg<2>::IDESC), "r"(accumulate));
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(TcCfg<1>::IDESC), "r"(accumulate));
    }
}

// Arrive on `bar` once the MMAs issued so far have completed; PAIR = 2: on the
// barrier at the same offset in both CTAs of the pair.
template <int PAIR>
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    if constexpr (PAIR == 2) {
        asm volatile(
            "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
            "[%0], %1;" ::"r"(smem_u32(bar)),
            "h"((uint16_t)3)
            : "memory");
    } else {
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(bar))
            : "memory");
    }
}

// TMEM allocation: with cta_group::2, one warp of each CTA of the pair takes
// part in the allocation and in the release.
template <int PAIR>
__device__ __forceinline__ void tmem_alloc(uint32_t* slot) {
    if constexpr (PAIR == 2) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    } else {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
}

template <int PAIR>
__device__ __forceinline__ void tmem_dealloc(uint32_t tmem) {
    if constexpr (PAIR == 2) {
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
    } else {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
    }
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// t[v] += r[v] (v < 32, round-to-nearest) as 16 packed float32-pair adds.
__device__ __forceinline__ void add_f32x2_32(float* t, const uint32_t (&r)[32]) {
#pragma unroll
    for (int v = 0; v < 32; v += 2) {
        asm("{\n\t.reg .b64 x, y;\n\t"
            "mov.b64 x, {%0, %1};\n\t"
            "mov.b64 y, {%2, %3};\n\t"
            "add.rn.f32x2 x, x, y;\n\t"
            "mov.b64 {%0, %1}, x;\n\t}"
            : "+f"(t[v]), "+f"(t[v + 1])
            : "r"(r[v]), "r"(r[v + 1]));
    }
}

struct TcMaps {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
    CUtensorMap c;  // float32 output, 32 x 32 boxes, 128-byte swizzle
};

// 2-D tile store from this CTA's shared memory (bulk async group).
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
            reinterpret_cast<uint64_t>(map)),
        "r"(smem_u32(src)), "r"(x), "r"(y)
        : "memory");
}

// Static schedule shared by every role of a CTA (no broadcast needed): super-tile
// s = (row block, p) holds the output column blocks p and n_tiles - 1 - p of one
// row block. Their triangular k ranges add up to the same length for every p, so
// a round-robin of super-tiles over the clusters balances the work; consecutive
// super-tiles share the row block, so the A rows in flight stay in L2. The longer
// k range of the two runs first.
struct TileSched {
    int n_tiles, P, total, kmode;
    __host__ __device__ TileSched(int m_tiles, int n_tiles_, int kmode_)
        : n_tiles(n_tiles_), P((n_tiles_ + 1) / 2), total(m_tiles * ((n_tiles_ + 1) / 2)),
          kmode(kmode_) {}
    // tile h (0, 1) of super-tile s; false when s holds a single (middle) column block
    __host__ __device__ bool tile(int s, int h, int& m_tile, int& n_tile) const {
        const int p = s % P;
        m_tile = s / P;
        const int lo = p, hi = n_tiles - 1 - p;
        if (h == 1 && hi == lo) return false;
        const bool hi_first = (kmode != KB_LOWER);  // KB_UPPER: k range grows with the block
        n_tile = ((h == 0) == hi_first) ? hi : lo;
        return true;
    }
    __host__ __device__ void k_range(int n_tile, int K, int& kbeg, int& nkb) const {
        const int n0 = n_tile * TC_BN;
        int kend = K;
        kbeg = 0;
        if (kmode == KB_UPPER) kend = K < n0 + TC_BN ? K : n0 + TC_BN;
        else if (kmode == KB_LOWER) kbeg = (n0 / TC_BK) * TC_BK;
        nkb = kend > kbeg ? (kend - kbeg + TC_BK - 1) / TC_BK : 0;
    }
};

// The last rounds of the round-robin leave clusters idle while others finish
// (1024 super-tiles on 76 clusters: 40 clusters wait out the 14th round). So
// only the first static_rounds rounds are round-robin; the tiles of the
// remaining one to two rounds' super-tiles (all from the last few row blocks,
// whose A rows stay in L2) are dealt out largest first to the least-loaded
// cluster (LPT), computed on the host and passed as a kernel parameter:
// cluster c then runs tiles[off[c] .. off[c + 1]) in that order.
constexpr int TC_MAX_CLUSTERS = 160;
constexpr int TC_MAX_TAIL = 640;
struct TcTail {
    int static_rounds;
    uint16_t off[TC_MAX_CLUSTERS + 1];
    uint32_t tiles[TC_MAX_TAIL];  // m_tile << 8 | n_tile
};

// One GEMM of a launch: its operand maps, sizes and scale vectors. A single
// GEMM's record is a kernel parameter; a group's records sit in device memory.
struct TcProblem {
    const TcMaps* maps;
    const float* row_mul;  // nullptr: row_mul_const for every row
    const float* col_mul;
    float row_mul_const;
    int M, N, K, kmode;
};

// k-blocks of column block n_tile of a problem (its kmode's triangular range)
__device__ __forceinline__ void problem_k_range(const TcProblem* p, int n_tile, int& kbeg,
                                                int& nkb) {
    const TileSched ks(1, 1, p->kmode);
    ks.k_range(n_tile, p->K, kbeg, nkb);
}

// The tiles of one cluster of a single GEMM, in order: the static rounds (both
// tiles of each super-tile), then the cluster's share of the tail.
struct SingleIter {
    const TileSched& sched;
    const TcTail& tail;
    const TcProblem* prob;
    int cluster, ncl, i;
    __device__ SingleIter(const TileSched& s, const TcTail& t, const TcProblem* p, int c, int n)
        : sched(s), tail(t), prob(p), cluster(c), ncl(n), i(0) {}
    __device__ bool next(int& m_tile, int& n_tile, const TcProblem*& p) {
        p = prob;
        const int nst = 2 * tail.static_rounds;
        while (i < nst) {
            const int r = i >> 1, h = i & 1;
            ++i;
            const int s = cluster + r * ncl;
            if (s < sched.total && sched.tile(s, h, m_tile, n_tile)) return true;
        }
        const int e = (int)tail.off[cluster] + (i - nst);
        if (e >= (int)tail.off[cluster + 1]) return false;
        ++i;
        const uint32_t t = tail.tiles[e];
        m_tile = (int)(t >> 8);
        n_tile = (int)(t & 255u);
        return true;
    }
};

// A group of independent GEMMs in one launch (many models of uneven size): the
// host deals every (problem, row block, column block) tile out to the clusters
// (largest k range first, to the least-loaded cluster); cluster c runs
// tiles[off[c] .. off[c + 1]).
struct TcGroupEntry {
    TcMaps maps;
    TcProblem p;  // p.maps points at this entry's maps
};
struct TcGroupDev {
    const TcGroupEntry* entries;
    const int* off;
    const uint64_t* tiles;  // problem << 40 | m_tile << 16 | n_tile
};

struct GroupIter {
    const TcGroupDev& g;
    int e, end;
    int last = -1;
    __device__ GroupIter(const TcGroupDev& gd, int c) : g(gd), e(gd.off[c]), end(gd.off[c + 1]) {}
    __device__ bool next(int& m_tile, int& n_tile, const TcProblem*& p) {
        if (e >= end) return false;
        const uint64_t t = g.tiles[e++];
        const int prob = (int)(t >> 40);
        m_tile = (int)((t >> 16) & 0xFFFFFFull);
        n_tile = (int)(t & 0xFFFFull);
        p = &g.entries[prob].p;
        if (prob != last) {
            // the maps were written through the generic proxy (a copy from the host)
            const TcMaps* mp = &g.entries[prob].maps;
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&mp->a_hi)
                         : "memory");
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&mp->a_lo)
                         : "memory");
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&mp->b_hi)
                         : "memory");
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&mp->b_lo)
                         : "memory");
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&mp->c)
                         : "memory");
            last = prob;
        }
        return true;
    }
};

// kmode: KB_UPPER (forward, k < n0 + BN), KB_LOWER (adjoint, k >= n0) or KFULL.
// Persistent: each CTA (PAIR = 2: each cluster of two CTAs, rank 0 issuing the
// MMAs) walks the tiles of the static schedule above. TMEM is allocated once;
// the stage and accumulator counters run on across tiles, so the next tile's
// loads and MMAs proceed while the epilogue warps store the previous tile.
template <int PAIR, class MakeIter>
__device__ __forceinline__ void tc_gemm_body(const MakeIter& make_iter, int* __restrict__ err) {
    using Cfg = TcCfg<PAIR>;
    constexpr int STAGES = Cfg::STAGES;
    extern __shared__ __align__(1024) uint8_t smraw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) &
                                               ~(uintptr_t)1023);
    float* staging = reinterpret_cast<float*>(base + STAGES * Cfg::STAGE_BYTES);  // 1024-aligned
    uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * Cfg::STAGE_BYTES + Cfg::STAGING);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;  // accumulator a holds a finished chunk
    uint64_t* acce = accf + 2;        // accumulator a has been drained
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
    int* fail = reinterpret_cast<int*>(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t rank = (PAIR == 2) ? cluster_rank() : 0u;
    const bool leader = (rank == 0);
    const int cluster = blockIdx.x / PAIR;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&accf[a], 1);
            mbar_init(&acce[a], 8 * PAIR);  // one arrival per epilogue warp of the pair
        }
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc<PAIR>(tmem_slot);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if constexpr (PAIR == 2) cluster_sync();  // the peer's barriers exist before any remote use
    else __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer (each CTA loads its own rows of A and of B)
        int g = 0;  // k-blocks issued by this CTA
        bool stop = false;
        auto it = make_iter(cluster);
        int m_tile, n_tile;
        const TcProblem* pr;
        while (!stop && it.next(m_tile, n_tile, pr)) {
            {
                int kbeg, nkb;
                problem_k_range(pr, n_tile, kbeg, nkb);
                const int arow = m_tile * TC_BM * PAIR + (int)rank * TC_BM;
                const int brow = n_tile * TC_BN + (int)rank * Cfg::B_ROWS;
                for (int kb = 0; kb < nkb; ++kb, ++g) {
                    const int st = g % STAGES;
                    if (g >= STAGES && !mbar_wait(&empty[st], ((g / STAGES) - 1) & 1, fail)) {
                        atomicExch(fail, 1);
                        stop = true;
                        break;
                    }
                    if (*(volatile int*)fail) {
                        stop = true;
                        break;
                    }
                    uint8_t* sp = base + st * Cfg::STAGE_BYTES;
                    const int k = kbeg + kb * TC_BK;
                    // the stage completes on the leader's barrier once both CTAs' bytes landed
                    if (leader) mbar_expect_tx(&full[st], Cfg::TX_BYTES);
                    const uint32_t bar =
                        (PAIR == 2) ? peer_addr(smem_u32(&full[st]), 0) : smem_u32(&full[st]);
                    const TcMaps* mp = pr->maps;
                    tma_load_2d<PAIR>(sp, &mp->a_hi, bar, k, arow);
                    tma_load_2d<PAIR>(sp + A_TILE, &mp->a_lo, bar, k, arow);
                    tma_load_2d<PAIR>(sp + 2 * A_TILE, &mp->b_hi, bar, k, brow);
                    tma_load_2d<PAIR>(sp + 2 * A_TILE + Cfg::B_TILE, &mp->b_lo, bar, k, brow);
                }
            }
        }
        // copies in flight must land before the CTA may exit: the leader waits for
        // the last phase armed on each stage (bounded); the peer cannot wait on the
        // leader's barrier and relies on the delay before the final cluster barrier
        if (*(volatile int*)fail && leader) {
            for (int gg = g - STAGES < 0 ? 0 : g - STAGES; gg < g; ++gg)
                mbar_wait(&full[gg % STAGES], (gg / STAGES) & 1);
        }
    } else if (warp == 1 && lane == 0 && leader) {
        // ---------------- MMA issuer (the leader CTA of the pair)
        int g = 0, cg = 0;  // k-blocks consumed, accumulator chunks started
        bool stop = false;
        auto it = make_iter(cluster);
        int m_tile, n_tile;
        const TcProblem* pr;
        while (!stop && it.next(m_tile, n_tile, pr)) {
            {
                int kbeg, nkb;
                problem_k_range(pr, n_tile, kbeg, nkb);
                const int nch = (nkb + TC_FLUSH - 1) / TC_FLUSH;
                for (int c = 0; c < nch && !stop; ++c, ++cg) {
                    const int a = cg & 1;
                    if (cg >= 2 && !mbar_wait(&acce[a], ((cg >> 1) - 1) & 1, fail)) {
                        atomicCAS(fail, 0, 4);
                        stop = true;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t tacc = tmem + (uint32_t)(a * TC_BN);
                    const int kb_end = min(nkb, (c + 1) * TC_FLUSH);
                    for (int kb = c * TC_FLUSH; kb < kb_end; ++kb, ++g) {
                        const int st = g % STAGES;
                        if (!mbar_wait(&full[st], (g / STAGES) & 1, fail)) {
                            atomicCAS(fail, 0, 2);
                            stop = true;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t sa = smem_u32(base + st * Cfg::STAGE_BYTES);
                        const uint32_t a_hi = sa, a_lo = sa + A_TILE, b_hi = sa + 2 * A_TILE,
                                       b_lo = sa + 2 * A_TILE + Cfg::B_TILE;
                        // the two small cross products first, the hi x hi product last:
                        // each MMA truncates its sum to the accumulator's scale, so
                        // issuing the small terms while the accumulator is still small
                        // leaves fewer full-scale truncations per chunk
#pragma unroll
                        for (int kk = 0; kk < TC_BK / TC_UMMA_K; ++kk) {
                            const uint32_t off = kk * TC_UMMA_K * 2;  // bytes along K in the 128-B row
                            const uint32_t acc = (kb > c * TC_FLUSH || kk > 0) ? 1u : 0u;
                            umma_f16<PAIR>(tacc, sdesc(a_lo + off), sdesc(b_hi + off), acc);
                            umma_f16<PAIR>(tacc, sdesc(a_hi + off), sdesc(b_lo + off), 1u);
                        }
#pragma unroll
                        for (int kk = 0; kk < TC_BK / TC_UMMA_K; ++kk) {
                            const uint32_t off = kk * TC_UMMA_K * 2;
                            umma_f16<PAIR>(tacc, sdesc(a_hi + off), sdesc(b_hi + off), 1u);
                        }
                        umma_commit<PAIR>(&empty[st]);
                    }
                    umma_commit<PAIR>(&accf[a]);
                }
            }
        }
    } else if (warp >= 2) {
        // ---------------- epilogue: drain chunks into float32 registers, then store C
        const int quarter = warp % 4;          // TMEM lanes 32*quarter .. +31
        const int half = (warp - 2) / 4;       // columns 128*half .. +127
        float* stg = staging + (warp - 2) * 32 * 32;
        int cg = 0;
        bool good = true;
        auto it = make_iter(cluster);
        int m_tile, n_tile;
        const TcProblem* pr;
        while (good && it.next(m_tile, n_tile, pr)) {
            {
                int kbeg, nkb;
                problem_k_range(pr, n_tile, kbeg, nkb);
                const int nch = (nkb + TC_FLUSH - 1) / TC_FLUSH;
                const int row0 = m_tile * TC_BM * PAIR + (int)rank * TC_BM + quarter * 32;
                const int row = row0 + lane;
                float tot[TC_BN / 2];
#pragma unroll
                for (int j = 0; j < TC_BN / 2; ++j) tot[j] = 0.f;
                for (int c = 0; c < nch; ++c, ++cg) {
                    const int a = cg & 1;
                    const bool ok = mbar_wait(&accf[a], (cg >> 1) & 1, fail);
                    // warp-uniform decision: tcgen05.ld is a .sync.aligned warp instruction
                    const int drain =
                        __shfl_sync(0xffffffffu, (ok && *(volatile int*)fail == 0) ? 1 : 0, 0);
                    if (!drain) {
                        if (lane == 0) atomicCAS(fail, 0, 3);
                        good = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) +
                                           (uint32_t)(a * TC_BN + half * (TC_BN / 2));
                    // the adds sit on the path from one chunk's completion to the MMAs
                    // that reuse its accumulator, so they run as packed float32 pairs
                    // and the last group's adds follow the release of the accumulator
                    uint32_t r[32];
#pragma unroll
                    for (int j = 0; j < TC_BN / 2 / 32 - 1; ++j) {
                        tmem_ld32(tbase + (uint32_t)(j * 32), r);
                        add_f32x2_32(tot + j * 32, r);
                    }
                    tmem_ld32(tbase + (uint32_t)((TC_BN / 2 / 32 - 1) * 32), r);
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive<PAIR>(&acce[a], 0);
                    add_f32x2_32(tot + (TC_BN / 2 / 32 - 1) * 32, r);
                }
                if (!good) break;
                // undo the operand scales (row multiplier times column multiplier) and
                // store through shared memory: per 32-column group the warp writes its
                // 32 x 32 tile (row = lane, 128-byte swizzle: 16-byte chunk v of row i at
                // v ^ (i % 8)) and one lane issues a TMA store of it, so global writes are
                // whole 128-byte row segments; the TMA clips rows >= M and columns >= N
                const int c0 = n_tile * TC_BN + half * (TC_BN / 2);
                const int M = pr->M, N = pr->N;
                const float* row_mul = pr->row_mul;
                const float* col_mul = pr->col_mul;
                const float rm = row < M ? (row_mul != nullptr ? row_mul[row] : pr->row_mul_const) : 0.f;
#pragma unroll
                for (int j = 0; j < TC_BN / 2 / 32; ++j) {
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    __syncwarp();
#pragma unroll
                    for (int v = 0; v < 8; ++v) {
                        const int col = c0 + j * 32 + 4 * v;
                        float4 cm;
                        if (col + 3 < N) {
                            cm = *reinterpret_cast<const float4*>(col_mul + col);
                        } else {
                            cm.x = col < N ? col_mul[col] : 0.f;
                            cm.y = col + 1 < N ? col_mul[col + 1] : 0.f;
                            cm.z = col + 2 < N ? col_mul[col + 2] : 0.f;
                            cm.w = 0.f;
                        }
                        const float* t = tot + j * 32 + 4 * v;
                        *reinterpret_cast<float4*>(stg + lane * 32 + ((v ^ (lane & 7)) * 4)) =
                            make_float4(t[0] * rm * cm.x, t[1] * rm * cm.y, t[2] * rm * cm.z,
                                        t[3] * rm * cm.w);
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) {
                        tma_store_2d(&pr->maps->c, stg, c0 + j * 32, row0);
                        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    }
                }
            }
        }
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if constexpr (PAIR == 2) {
        // after a failure, give bulk copies still in flight (which count on the
        // leader's barriers) time to land before either CTA of the pair exits
        if (*(volatile int*)fail) {
            const unsigned long long t0 = global_ns();
            while (global_ns() - t0 < 50000ull) {
            }
        }
        cluster_sync();
    } else {
        __syncthreads();
    }
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tmem_dealloc<PAIR>(tmem);
    }
    if (threadIdx.x == 0 && *fail) atomicExch(err, *fail);
}

// One GEMM: the maps, the tail schedule and the problem record are parameters.
template <int PAIR>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ TcMaps maps, const __grid_constant__ TcTail tail,
                   int M, int N, int K, int kmode, int m_tiles, int n_tiles,
                   const float* __restrict__ row_mul, float row_mul_const,
                   const float* __restrict__ col_mul, int* __restrict__ err) {
    const TileSched sched(m_tiles, n_tiles, kmode);
    const TcProblem prob{&maps, row_mul, col_mul, row_mul_const, M, N, K, kmode};
    const int ncl = gridDim.x / PAIR;
    auto make_iter = [&](int cluster) { return SingleIter(sched, tail, &prob, cluster, ncl); };
    tc_gemm_body<PAIR>(make_iter, err);
}

// A group of GEMMs: records, maps and the tile list in device memory.
template <int PAIR>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_group_kernel(const __grid_constant__ TcGroupDev grp, int* __restrict__ err) {
    auto make_iter = [&](int cluster) { return GroupIter(grp, cluster); };
    tc_gemm_body<PAIR>(make_iter, err);
}

// Power-of-two scale that brings the largest magnitude m of a row to at most
// 2^14: s = 2^(14 - e) with m = f 2^e, f in [0.5, 1); s = 1 for m = 0 or non-finite m.
__device__ __forceinline__ float pow2_scale(double m) {
    if (!(m > 0.0) || isinf(m)) return 1.f;
    int e;
    frexp(m, &e);
    return ldexpf(1.f, 14 - e);
}

// Per storage row i of src (or of its transpose): scale s_i = pow2_scale(max_j |x_ij|)
// and the float16 split hi = f16(s_i x), lo = f16(s_i x - hi) into ldd-strided
// rows (columns >= cols are 0); mul[i] = 1 / s_i. One warp per row.
__global__ void split_f64_f16_kernel(const double* __restrict__ src, int64_t rows, int64_t cols,
                                     int64_t lds, int transpose, __half* __restrict__ hi,
                                     __half* __restrict__ lo, int64_t ldd, float* __restrict__ mul) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (i >= rows) return;
    auto at = [&](int64_t j) { return transpose ? src[j * lds + i] : src[i * lds + j]; };
    double m = 0.0;
    for (int64_t j = lane; j < cols; j += 32) m = fmax(m, fabs(at(j)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    const float sc = pow2_scale(m);
    for (int64_t j = lane; j < ldd; j += 32) {
        const float x = (j < cols) ? (float)(at(j) * (double)sc) : 0.f;
        const __half h = __float2half_rn(x);
        hi[i * ldd + j] = h;
        lo[i * ldd + j] = __float2half_rn(x - __half2float(h));
    }
    if (lane == 0) mul[i] = 1.f / sc;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (fn == nullptr) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// 2-D row-major float16 matrix (rows x cols, leading dimension ld) as a TMA map
// with a 64-column x box_rows box and 128-byte swizzle; out-of-range reads are 0.
bool make_map(CUtensorMap* map, const __half* ptr, int64_t rows, int64_t cols, int64_t ld,
              int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (fn == nullptr) return false;
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) != 0 || (ld * 2) % 16 != 0) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half*>(ptr), dims, strides,
                    box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// 2-D row-major float32 matrix (rows x cols, leading dimension ld) as a TMA map
// with 32 x 32 boxes and 128-byte swizzle: the epilogue's stores of C.
bool make_map_f32(CUtensorMap* map, const float* ptr, int64_t rows, int64_t cols, int64_t ld) {
    EncodeTiledFn fn = encode_fn();
    if (fn == nullptr) return false;
    if ((reinterpret_cast<uintptr_t>(ptr) & 15) != 0 || (ld * 4) % 16 != 0) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(ptr), dims, strides,
                    box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Clusters of form PAIR that can be resident at once (one CTA per SM), per device.
template <int PAIR>
int resident_clusters() {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kNumSMs / PAIR;
    if (cached[dev] == 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(PAIR * 64);
        cfg.blockDim = dim3(TC_THREADS);
        cfg.dynamicSmemBytes = TcCfg<PAIR>::SMEM;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = PAIR;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, tc_gemm_kernel<PAIR>, &cfg) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = kNumSMs / PAIR;
        }
        cached[dev] = n;
    }
    return cached[dev];
}

// Tail schedule for ncl clusters (see TcTail). Without room for it (more
// clusters or tail tiles than the parameter holds, or n_tiles > 256) every
// round is round-robin.
void build_tail(int m_tiles, int n_tiles, int K, int kmode, int ncl, TcTail& t) {
    const TileSched sched(m_tiles, n_tiles, kmode);
    memset(&t, 0, sizeof(t));
    t.static_rounds = (sched.total + ncl - 1) / ncl;
    if (ncl <= 0 || ncl > TC_MAX_CLUSTERS || n_tiles > 256 || m_tiles >= (1 << 24)) return;
    const int rounds = sched.total / ncl;
    const int rs = rounds >= 2 ? rounds - 1 : 0;
    struct Item { int nkb, m, n; };
    std::vector<Item> items;
    for (int sidx = rs * ncl; sidx < sched.total; ++sidx) {
        for (int h = 0; h < 2; ++h) {
            int m, n, kbeg, nkb;
            if (!sched.tile(sidx, h, m, n)) continue;
            sched.k_range(n, K, kbeg, nkb);
            items.push_back({nkb, m, n});
        }
    }
    if ((int)items.size() > TC_MAX_TAIL) return;
    std::stable_sort(items.begin(), items.end(),
                     [](const Item& a, const Item& b) { return a.nkb > b.nkb; });
    // a tile costs its k-blocks plus about two k-blocks of exposed epilogue
    constexpr int kTileCost = 2;
    std::vector<long> load(ncl, 0);
    std::vector<std::vector<uint32_t>> lists(ncl);
    for (const Item& it : items) {
        int c = 0;
        for (int j = 1; j < ncl; ++j)
            if (load[j] < load[c]) c = j;
        lists[c].push_back(((uint32_t)it.m << 8) | (uint32_t)it.n);
        load[c] += it.nkb + kTileCost;
    }
    t.static_rounds = rs;
    int e = 0;
    for (int c = 0; c < ncl; ++c) {
        t.off[c] = (uint16_t)e;
        for (uint32_t v : lists[c]) t.tiles[e++] = v;
    }
    t.off[ncl] = (uint16_t)e;
}

// build_tail, memoised over the last few shapes (the schedule is a pure function
// of its arguments; graph capture and repeated calls reuse it).
void tail_for(int m_tiles, int n_tiles, int K, int kmode, int ncl, TcTail& out) {
    struct Entry { int key[5]; TcTail tail; };
    static std::mutex mu;
    static Entry cache[8];
    static int used = 0, next = 0;
    const int key[5] = {m_tiles, n_tiles, K, kmode, ncl};
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < used; ++i) {
        if (memcmp(cache[i].key, key, sizeof(key)) == 0) {
            out = cache[i].tail;
            return;
        }
    }
    Entry& en = cache[next];
    next = (next + 1) % 8;
    if (used < 8) ++used;
    memcpy(en.key, key, sizeof(key));
    build_tail(m_tiles, n_tiles, K, kmode, ncl, en.tail);
    out = en.tail;
}

// One persistent launch of the GEMM in form PAIR over m_tiles x n_tiles tiles:
// as many clusters of PAIR CTAs as are resident at once, or fewer when there are
// fewer super-tiles (pairs of column blocks of one row block).
template <int PAIR>
int launch_tc(const TcMaps& maps, int64_t M, int64_t N, int64_t K, int kmode, int m_tiles,
              int n_tiles, const float* row_mul, float row_mul_const, const float* col_mul,
              int* err, cudaStream_t stream) {
    // the shared-memory opt-in is a per-device function attribute
    static bool attr_set[64] = {};
    int dev = 0;
    BGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        BGB_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel<PAIR>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)TcCfg<PAIR>::SMEM));
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    const int64_t super_tiles = (int64_t)m_tiles * ((n_tiles + 1) / 2);
    const int64_t resident = resident_clusters<PAIR>();
    const int64_t clusters = super_tiles < resident ? super_tiles : resident;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(clusters * PAIR));
    cfg.blockDim = dim3(TC_THREADS);
    cfg.dynamicSmemBytes = TcCfg<PAIR>::SMEM;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = PAIR;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TcTail tail;
    tail_for(m_tiles, n_tiles, (int)K, kmode, (int)clusters, tail);
    BGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, tc_gemm_kernel<PAIR>, maps, tail, (int)M, (int)N, (int)K,
                                    kmode, m_tiles, n_tiles, row_mul, row_mul_const, col_mul, err));
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

// Clusters of two that can be resident at once for the grouped kernel, per device
// (after its shared-memory opt-in).
int group_resident_clusters() {
    static int cached[64] = {};
    static bool attr_set[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kNumSMs / 2;
    if (!attr_set[dev]) {
        if (cudaFuncSetAttribute(tc_gemm_group_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)TcCfg<2>::SMEM) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        attr_set[dev] = true;
    }
    if (cached[dev] == 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * 64);
        cfg.blockDim = dim3(TC_THREADS);
        cfg.dynamicSmemBytes = TcCfg<2>::SMEM;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, tc_gemm_group_kernel<2>, &cfg) != cudaSuccess ||
            n <= 0) {
            cudaGetLastError();
            n = kNumSMs / 2;
        }
        cached[dev] = n;
    }
    return cached[dev];
}

}  // namespace

size_t tc_group_entry_bytes() { return sizeof(TcGroupEntry); }

int64_t tc_group_tiles(int64_t M, int64_t N) {
    return ceil_div(M, (int64_t)TC_BM * 2) * ceil_div(N, (int64_t)TC_BN);
}

// Device tables of a grouped launch (two-SM form) into host buffers: one entry
// per GEMM (its maps and record; the record's maps pointer is the entry's
// address in dev_entries), and every (GEMM, row block, column block) tile dealt
// out largest k range first to the least-loaded of `clusters` clusters.
int tc_group_build(const TcGroupGemm* gemms, int count, uintptr_t dev_entries,
                   std::vector<unsigned char>& entries, std::vector<int>& off,
                   std::vector<uint64_t>& tiles, int& clusters) {
    if (count <= 0 || count >= (1 << 23)) return BGB_ERR_ARG;
    if (!tc_gemm_available()) return BGB_ERR_UNSUPPORTED;
    std::vector<TcGroupEntry> ent((size_t)count);
    struct Item { int nkb; uint64_t code; };
    std::vector<Item> items;
    for (int i = 0; i < count; ++i) {
        const TcGroupGemm& g = gemms[i];
        if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.col_mul == nullptr ||
            (reinterpret_cast<uintptr_t>(g.col_mul) & 15) != 0)
            return BGB_ERR_ARG;
        if (g.kmode != KB_UPPER && g.kmode != KB_LOWER && g.kmode != KFULL) return BGB_ERR_ARG;
        TcMaps& mp = ent[i].maps;
        const int b_rows = TC_BN / 2;
        if (!make_map(&mp.a_hi, g.A_hi, g.M, g.K, g.lda, TC_BM) ||
            !make_map(&mp.a_lo, g.A_lo, g.M, g.K, g.lda, TC_BM) ||
            !make_map(&mp.b_hi, g.B_hi, g.N, g.K, g.ldbs, b_rows) ||
            !make_map(&mp.b_lo, g.B_lo, g.N, g.K, g.ldbs, b_rows) ||
            !make_map_f32(&mp.c, g.C, g.M, g.N, g.ldc))
            return BGB_ERR_UNSUPPORTED;
        ent[i].p = TcProblem{reinterpret_cast<const TcMaps*>(dev_entries + (uintptr_t)i * sizeof(TcGroupEntry)),
                             g.row_mul, g.col_mul, g.row_mul_const, (int)g.M, (int)g.N, (int)g.K,
                             g.kmode};
        const int64_t m_tiles = ceil_div(g.M, (int64_t)TC_BM * 2);
        const int64_t n_tiles = ceil_div(g.N, (int64_t)TC_BN);
        if (m_tiles >= (1 << 24) || n_tiles >= (1 << 16)) return BGB_ERR_UNSUPPORTED;
        const TileSched ks(1, 1, g.kmode);
        for (int64_t mt = 0; mt < m_tiles; ++mt) {
            for (int64_t nt = 0; nt < n_tiles; ++nt) {
                int kbeg, nkb;
                ks.k_range((int)nt, (int)g.K, kbeg, nkb);
                items.push_back({nkb, ((uint64_t)i << 40) | ((uint64_t)mt << 16) | (uint64_t)nt});
            }
        }
    }
    const int resident = group_resident_clusters();
    if (resident <= 0) return BGB_ERR_UNSUPPORTED;
    clusters = (int)items.size() < resident ? (int)items.size() : resident;
    std::stable_sort(items.begin(), items.end(),
                     [](const Item& a, const Item& b) { return a.nkb > b.nkb; });
    constexpr int kTileCost = 2;  // about two k-blocks of exposed epilogue per tile
    std::vector<long> load((size_t)clusters, 0);
    std::vector<std::vector<uint64_t>> lists((size_t)clusters);
    for (const Item& it : items) {
        int c = 0;
        for (int j = 1; j < clusters; ++j)
            if (load[j] < load[c]) c = j;
        lists[c].push_back(it.code);
        load[c] += it.nkb + kTileCost;
    }
    off.assign((size_t)clusters + 1, 0);
    tiles.clear();
    for (int c = 0; c < clusters; ++c) {
        off[c] = (int)tiles.size();
        tiles.insert(tiles.end(), lists[c].begin(), lists[c].end());
    }
    off[clusters] = (int)tiles.size();
    entries.resize(sizeof(TcGroupEntry) * (size_t)count);
    memcpy(entries.data(), ent.data(), entries.size());
    return BGB_OK;
}

int tc_group_launch(const void* dev_entries, const int* dev_off, const uint64_t* dev_tiles,
                    int clusters, int* err, cudaStream_t stream) {
    if (clusters <= 0) return BGB_OK;
    if (dev_entries == nullptr || dev_off == nullptr || dev_tiles == nullptr ||
        (reinterpret_cast<uintptr_t>(dev_entries) & 63) != 0)
        return BGB_ERR_ARG;
    if (group_resident_clusters() <= 0) return BGB_ERR_UNSUPPORTED;
    TcGroupDev grp{static_cast<const TcGroupEntry*>(dev_entries), dev_off, dev_tiles};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(clusters * 2));
    cfg.blockDim = dim3(TC_THREADS);
    cfg.dynamicSmemBytes = TcCfg<2>::SMEM;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    BGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, tc_gemm_group_kernel<2>, grp, err));
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

bool tc_gemm_available() { return encode_fn() != nullptr; }

int split_f64_f16(const double* src, int64_t rows, int64_t cols, int64_t lds, int transpose,
                  __half* hi, __half* lo, int64_t ldd, float* mul, cudaStream_t stream) {
    if (rows <= 0 || cols <= 0) return BGB_OK;
    if (ldd < cols) return BGB_ERR_ARG;
    split_f64_f16_kernel<<<(unsigned)ceil_div(rows * 32, 256), 256, 0, stream>>>(
        src, rows, cols, lds, transpose, hi, lo, ldd, mul);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

// C (M x N) = diag(row_mul) (A (M x K) * op(B)) diag(col_mul), A given as its
// float16 split hi/lo (lda), B as its K-major storage Bs (N x K, hi/lo, ldbs):
// op(B)[k][j] = Bs[j][k]. row_mul: M multipliers, or nullptr for row_mul_const.
// kmode KB_UPPER or KB_LOWER.
int tc_gemm_f16x3(int64_t M, int64_t N, int64_t K, const __half* A_hi, const __half* A_lo,
                  int64_t lda, const __half* B_hi, const __half* B_lo, int64_t ldbs, float* C,
                  int64_t ldc, int kmode, const float* row_mul, float row_mul_const,
                  const float* col_mul, int* err, cudaStream_t stream) {
    if (M <= 0 || N <= 0) return BGB_OK;
    if (col_mul == nullptr || (reinterpret_cast<uintptr_t>(col_mul) & 15) != 0) return BGB_ERR_ARG;
    // form: the two-SM pair (default) or, with BGB_TC_PAIR=1 in the environment, the
    // single-SM form (a comparison aid)
    static const int pair = [] {
        const char* e = getenv("BGB_TC_PAIR");
        return (e != nullptr && e[0] == '1') ? 1 : 2;
    }();
    TcMaps maps;
    const int b_rows = TC_BN / pair;
    if (!make_map(&maps.a_hi, A_hi, M, K, lda, TC_BM) || !make_map(&maps.a_lo, A_lo, M, K, lda, TC_BM) ||
        !make_map(&maps.b_hi, B_hi, N, K, ldbs, b_rows) || !make_map(&maps.b_lo, B_lo, N, K, ldbs, b_rows) ||
        !make_map_f32(&maps.c, C, M, N, ldc))
        return BGB_ERR_UNSUPPORTED;
    const int m_tiles = (int)ceil_div(M, (int64_t)TC_BM * pair), n_tiles = (int)ceil_div(N, TC_BN);
    return pair == 2 ? launch_tc<2>(maps, M, N, K, kmode, m_tiles, n_tiles, row_mul, row_mul_const,
                                    col_mul, err, stream)
                     : launch_tc<1>(maps, M, N, K, kmode, m_tiles, n_tiles, row_mul, row_mul_const,
                                    col_mul, err, stream);
}

}  // namespace bgb
