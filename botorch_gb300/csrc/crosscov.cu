// (c) Cross-covariance GEMM, float32 SIMT form: C = Kc * B, where Kc = K(X, Xt)
// (b*q x n) and B = [K^-1 | K^-1 K(Xt, Xb) | alpha] (n x ldb).
//
// 128 x 128 output tile per CTA, k step 8, 256 threads with an 8 x 8
// register micro-tile each, shared-memory double buffering. This is the
// FFMA-bound baseline of the mixed-precision path; the tensor-core form of the
// same product lives in crosscov_tc.cu.
#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int SG_BM = 128, SG_BN = 128, SG_BK = 8;

__global__ void __launch_bounds__(256) sgemm_kernel(int64_t M, int64_t N, int64_t K,
                                                    const float* __restrict__ A, int64_t lda,
                                                    const float* __restrict__ B, int64_t ldb,
                                                    float* __restrict__ C, int64_t ldc, int kmode,
                                                    int64_t n_tri) {
    __shared__ __align__(16) float As[2][SG_BK][SG_BM];
    __shared__ __align__(16) float Bs[2][SG_BK][SG_BN];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int64_t row0 = (int64_t)blockIdx.y * SG_BM, col0 = (int64_t)blockIdx.x * SG_BN;
    // loader coordinates
    const int a_r = tid / 2, a_k = (tid % 2) * 4;
    const int b_k = tid / 32, b_c = (tid % 32) * 4;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    float ra[4], rb[4];
    auto load_regs = [&](int64_t k0) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int64_t gr = row0 + a_r, gk = k0 + a_k + u;
            ra[u] = (gr < M && gk < K) ? A[gr * lda + gk] : 0.f;
            int64_t gk2 = k0 + b_k, gc = col0 + b_c + u;
            rb[u] = (gk2 < K && gc < N) ? B[gk2 * ldb + gc] : 0.f;
        }
    };
    auto store_smem = [&](int buf) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            As[buf][a_k + u][a_r] = ra[u];
            Bs[buf][b_k][b_c + u] = rb[u];
        }
    };
    // triangular right operands: skip the k-range where B is zero
    int64_t kbeg = 0, kend = K;
    if (kmode == KB_LOWER) kbeg = col0;
    else if (kmode == KB_UPPER && col0 + SG_BN <= n_tri) kend = col0 + SG_BN < K ? col0 + SG_BN : K;
    load_regs(kbeg);
    store_smem(0);
    __syncthreads();
    int buf = 0;
    for (int64_t k0 = kbeg; k0 < kend; k0 += SG_BK) {
        const bool more = k0 + SG_BK < kend;
        if (more) load_regs(k0 + SG_BK);
#pragma unroll
        for (int kk = 0; kk < SG_BK; ++kk) {
            float a[8], b[8];
            float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
            float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
            a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
            b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) {
            store_smem(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        int64_t r = row0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int64_t c = col0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
            if (c < N) C[r * ldc + c] = acc[i][j];
        }
    }
}

}  // namespace

int gemm_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
             int64_t ldb, float* C, int64_t ldc, int kmode, int64_t n_tri, cudaStream_t stream) {
    if (M <= 0 || N <= 0) return BGB_OK;
    dim3 grid((unsigned)ceil_div(N, SG_BN), (unsigned)ceil_div(M, SG_BM));
    sgemm_kernel<<<grid, 256, 0, stream>>>(M, N, K, A, lda, B, ldb, C, ldc, kmode, n_tri);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

}  // namespace bgb
