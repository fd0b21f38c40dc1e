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
// One CTA computes a 128 x 256 tile of C. Warp roles: warp 0 issues the TMA
// loads (one elected lane), warp 1 owns the TMEM allocation and issues the
// MMAs (one elected lane), warps 2-9 drain the accumulators. Two shared-memory
// stages of {A_hi, A_lo, B_hi, B_lo} (96 KB each, 64 K-elements deep).
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

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 64;  // BK: float16 elements (128 bytes)
constexpr int TC_STAGES = 2;
constexpr int TC_UMMA_K = 16;                         // float16 K per tcgen05.mma
constexpr uint32_t A_TILE = TC_BM * TC_BK * 2;        // 16 KB
constexpr uint32_t B_TILE = TC_BN * TC_BK * 2;        // 32 KB
constexpr uint32_t STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int TC_THREADS = 320;                       // 10 warps
constexpr int TC_FLUSH = 1;                           // k-blocks per TMEM accumulation chunk
constexpr uint32_t TMEM_COLS = 512;                   // two 128 x 256 float32 accumulators
constexpr size_t TC_SMEM = TC_STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

// instruction descriptor (kind::f16): D f32, A/B f16, both K-major, N = 256, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                            ((uint32_t)(TC_BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
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

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
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

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
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

struct TcMaps {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
};

// kmode: KB_UPPER (forward, k < n0 + BN) or KB_LOWER (adjoint, k >= n0).
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ TcMaps maps, float* __restrict__ C, int64_t ldc,
                   int M, int N, int K, int kmode, int n_tiles, const float* __restrict__ row_mul,
                   float row_mul_const, const float* __restrict__ col_mul, int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smraw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smraw) + 1023) &
                                               ~(uintptr_t)1023);
    uint64_t* full = reinterpret_cast<uint64_t*>(base + TC_STAGES * STAGE_BYTES);
    uint64_t* empty = full + TC_STAGES;
    uint64_t* accf = empty + TC_STAGES;  // accumulator a holds a finished chunk
    uint64_t* acce = accf + 2;           // accumulator a has been drained
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
    int* fail = reinterpret_cast<int*>(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    // tile order: consecutive CTAs share the A row-block (all n-tiles of one m-tile),
    // and within it the longest k range comes first (KB_UPPER: the last column
    // blocks, KB_LOWER: the first), so the final wave holds the short tiles
    const int m_tile = blockIdx.x / n_tiles;
    const int n_idx = blockIdx.x % n_tiles;
    const int n_tile = (kmode == KB_UPPER) ? n_tiles - 1 - n_idx : n_idx;
    const int m0 = m_tile * TC_BM, n0 = n_tile * TC_BN;
    int kbeg = 0, kend = K;
    if (kmode == KB_UPPER) kend = min(K, n0 + TC_BN);
    else if (kmode == KB_LOWER) kbeg = (n0 / TC_BK) * TC_BK;
    const int nkb = (kend - kbeg + TC_BK - 1) / TC_BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&accf[a], 1);
            mbar_init(&acce[a], 8);  // one arrival per epilogue warp
        }
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % TC_STAGES;
            if (kb >= TC_STAGES && !mbar_wait(&empty[s], ((kb / TC_STAGES) - 1) & 1, fail)) {
                atomicExch(fail, 1);
                break;
            }
            if (*(volatile int*)fail) break;
            uint8_t* st = base + s * STAGE_BYTES;
            const int k = kbeg + kb * TC_BK;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_load_2d(st, &maps.a_hi, &full[s], k, m0);
            tma_load_2d(st + A_TILE, &maps.a_lo, &full[s], k, m0);
            tma_load_2d(st + 2 * A_TILE, &maps.b_hi, &full[s], k, n0);
            tma_load_2d(st + 2 * A_TILE + B_TILE, &maps.b_lo, &full[s], k, n0);
            issued = kb + 1;
        }
        // copies in flight must land before the CTA may exit: wait for the last
        // phase armed on each stage (bounded)
        if (*(volatile int*)fail) {
            for (int kb = issued - TC_STAGES < 0 ? 0 : issued - TC_STAGES; kb < issued; ++kb)
                mbar_wait(&full[kb % TC_STAGES], (kb / TC_STAGES) & 1);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        const int nch = (nkb + TC_FLUSH - 1) / TC_FLUSH;
        for (int c = 0; c < nch; ++c) {
            const int a = c & 1;
            if (c >= 2 && !mbar_wait(&acce[a], ((c >> 1) - 1) & 1, fail)) {
                atomicCAS(fail, 0, 4);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t tacc = tmem + (uint32_t)(a * TC_BN);
            const int kb_end = min(nkb, (c + 1) * TC_FLUSH);
            bool ok = true;
            for (int kb = c * TC_FLUSH; kb < kb_end; ++kb) {
                const int s = kb % TC_STAGES;
                if (!mbar_wait(&full[s], (kb / TC_STAGES) & 1, fail)) {
                    atomicCAS(fail, 0, 2);
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = smem_u32(base + s * STAGE_BYTES);
                const uint32_t a_hi = sa, a_lo = sa + A_TILE, b_hi = sa + 2 * A_TILE,
                               b_lo = sa + 2 * A_TILE + B_TILE;
#pragma unroll
                for (int kk = 0; kk < TC_BK / TC_UMMA_K; ++kk) {
                    const uint32_t off = kk * TC_UMMA_K * 2;  // bytes along K in the 128-B row
                    const uint32_t acc = (kb > c * TC_FLUSH || kk > 0) ? 1u : 0u;
                    umma_f16(tacc, sdesc(a_lo + off), sdesc(b_hi + off), acc);
                    umma_f16(tacc, sdesc(a_hi + off), sdesc(b_lo + off), 1u);
                    umma_f16(tacc, sdesc(a_hi + off), sdesc(b_hi + off), 1u);
                }
                umma_commit(&empty[s]);
            }
            umma_commit(&accf[a]);
            if (!ok) break;
        }
    } else if (warp >= 2) {
        // ---------------- epilogue: drain chunks into float32 registers, then store C
        const int quarter = warp % 4;          // TMEM lanes 32*quarter .. +31
        const int half = (warp - 2) / 4;       // columns 128*half .. +127
        const int row = m0 + quarter * 32 + lane;
        const int nch = (nkb + TC_FLUSH - 1) / TC_FLUSH;
        float tot[TC_BN / 2];
#pragma unroll
        for (int j = 0; j < TC_BN / 2; ++j) tot[j] = 0.f;
        bool good = true;
        for (int c = 0; c < nch; ++c) {
            const int a = c & 1;
            const bool ok = mbar_wait(&accf[a], (c >> 1) & 1, fail);
            // warp-uniform decision: tcgen05.ld is a .sync.aligned warp instruction
            const int drain = __shfl_sync(0xffffffffu, (ok && *(volatile int*)fail == 0) ? 1 : 0, 0);
            if (!drain) {
                if (lane == 0) atomicCAS(fail, 0, 3);
                good = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) +
                                   (uint32_t)(a * TC_BN + half * (TC_BN / 2));
#pragma unroll
            for (int j = 0; j < TC_BN / 2 / 32; ++j) {
                uint32_t r[32];
                tmem_ld32(tbase + (uint32_t)(j * 32), r);
#pragma unroll
                for (int v = 0; v < 32; ++v) tot[j * 32 + v] += __uint_as_float(r[v]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[a]);
        }
        if (good && row < M) {
            // undo the operand scales: row multiplier times column multiplier
            const int c0 = n0 + half * (TC_BN / 2);
            const float rm = row_mul != nullptr ? row_mul[row] : row_mul_const;
            float* dst = C + (int64_t)row * ldc + c0;
            if (c0 + TC_BN / 2 <= N && (ldc % 4) == 0 &&
                (reinterpret_cast<uintptr_t>(col_mul + c0) % 16) == 0) {
                const float4* cm4 = reinterpret_cast<const float4*>(col_mul + c0);
#pragma unroll
                for (int v = 0; v < TC_BN / 2 / 4; ++v) {
                    const float4 cm = cm4[v];
                    reinterpret_cast<float4*>(dst)[v] =
                        make_float4(tot[4 * v] * rm * cm.x, tot[4 * v + 1] * rm * cm.y,
                                    tot[4 * v + 2] * rm * cm.z, tot[4 * v + 3] * rm * cm.w);
                }
            } else {
#pragma unroll
                for (int v = 0; v < TC_BN / 2; ++v)
                    if (c0 + v < N) dst[v] = tot[v] * rm * col_mul[c0 + v];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
    }
    if (threadIdx.x == 0 && *fail) atomicExch(err, *fail);
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

}  // namespace

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
    if (col_mul == nullptr) return BGB_ERR_ARG;
    TcMaps maps;
    if (!make_map(&maps.a_hi, A_hi, M, K, lda, TC_BM) || !make_map(&maps.a_lo, A_lo, M, K, lda, TC_BM) ||
        !make_map(&maps.b_hi, B_hi, N, K, ldbs, TC_BN) || !make_map(&maps.b_lo, B_lo, N, K, ldbs, TC_BN))
        return BGB_ERR_UNSUPPORTED;
    // the shared-memory opt-in is a per-device function attribute
    static bool attr_set[64] = {};
    int dev = 0;
    BGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64 || !attr_set[dev]) {
        BGB_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)TC_SMEM));
        if (dev >= 0 && dev < 64) attr_set[dev] = true;
    }
    const int m_tiles = (int)ceil_div(M, TC_BM), n_tiles = (int)ceil_div(N, TC_BN);
    tc_gemm_kernel<<<(unsigned)(m_tiles * n_tiles), TC_THREADS, TC_SMEM, stream>>>(
        maps, C, ldc, (int)M, (int)N, (int)K, kmode, n_tiles, row_mul, row_mul_const, col_mul, err);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

}  // namespace bgb
