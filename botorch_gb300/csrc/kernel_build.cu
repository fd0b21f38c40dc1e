// (a) Covariance-matrix build: K[i, j] = outputscale * kappa(sum_k ((x1_ik - x2_jk) * il_k)^2).
//
// One CTA computes a 64 x 64 output tile. The two 64-row slabs of inputs
// are staged in shared memory (32 coordinates at a time); each thread owns a
// 4 x 4 micro-tile and forms the squared scaled distances from explicit
// coordinate differences (no |a|^2 + |b|^2 - 2ab expansion, so close points
// keep full relative accuracy). The distance tensor never leaves registers.
// The kernel is HBM-write bound for the matrix it produces: algorithmic bytes
// per output = sizeof(TOut).
#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int KB_TILE = 64;
constexpr int KB_DCHUNK = 32;


// K16 == nullptr: plain output K. Otherwise (float32 arithmetic only) the output
// is the scaled float16 split for the tensor-core GEMM: with w = k16_scale * v,
// K16 = f16(w), K16_lo = f16(w - K16) (K is not written).
template <typename TIn, typename TAcc, typename TOut>
__global__ void __launch_bounds__(256) kernel_matrix_kernel(
    const TIn* __restrict__ X1, int64_t m, const TIn* __restrict__ X2, int64_t n2, int d,
    const double* __restrict__ inv_ls, double outputscale, int kind, double diag_add,
    int same, TOut* __restrict__ K, int64_t ldk, __half* __restrict__ K16,
    __half* __restrict__ K16_lo, float k16_scale, const float* __restrict__ Z1T, int64_t ldz1,
    const float* __restrict__ Z2T, int64_t ldz2) {
    __shared__ TAcc s1[KB_DCHUNK][KB_TILE + 1];
    __shared__ TAcc s2[KB_DCHUNK][KB_TILE + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int64_t row0 = (int64_t)blockIdx.y * KB_TILE, col0 = (int64_t)blockIdx.x * KB_TILE;
    TAcc acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = TAcc(0);
    for (int k0 = 0; k0 < d; k0 += KB_DCHUNK) {
        const int kc = min(KB_DCHUNK, d - k0);
        for (int idx = threadIdx.x; idx < KB_DCHUNK * KB_TILE; idx += blockDim.x) {
            int kk = idx / KB_TILE, rr = idx % KB_TILE;
            TAcc v1 = 0, v2 = 0;
            if (kk < kc && Z1T != nullptr) {  // pre-scaled float32, k-major
                if (row0 + rr < m) v1 = (TAcc)Z1T[(int64_t)(k0 + kk) * ldz1 + row0 + rr];
                if (col0 + rr < n2) v2 = (TAcc)Z2T[(int64_t)(k0 + kk) * ldz2 + col0 + rr];
            } else if (kk < kc) {
                const double il = inv_ls[k0 + kk];
                if (row0 + rr < m) v1 = (TAcc)((double)X1[(row0 + rr) * d + k0 + kk] * il);
                if (col0 + rr < n2) v2 = (TAcc)((double)X2[(col0 + rr) * d + k0 + kk] * il);
            }
            s1[kk][rr] = v1;
            s2[kk][rr] = v2;
        }
        __syncthreads();
        for (int kk = 0; kk < kc; ++kk) {
            TAcc a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = s1[kk][ty + 16 * u];
                b[u] = s2[kk][tx + 16 * u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    TAcc df = a[u] - b[v];
                    acc[u][v] += df * df;
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        int64_t i = row0 + ty + 16 * u;
        if (i >= m) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            int64_t j = col0 + tx + 16 * v;
            if (j >= n2) continue;
            TAcc val = TAcc(outputscale) * kappa<TAcc>(kind, acc[u][v]);
            if (same && i == j) val += TAcc(diag_add);
            if constexpr (sizeof(TAcc) == 4) {
                if (K16 != nullptr) {
                    const float w = (float)val * k16_scale;
                    const __half h = __float2half_rn(w);
                    K16[i * ldk + j] = h;
                    K16_lo[i * ldk + j] = __float2half_rn(w - __half2float(h));
                    continue;
                }
            }
            K[i * ldk + j] = (TOut)val;
        }
    }
}

}  // namespace

template <typename TIn, typename TAcc, typename TOut>
int launch_kernel_matrix(const TIn* X1, int64_t m, const TIn* X2, int64_t n2, int d,
                         const double* inv_ls, double outputscale, int kind, double diag_add,
                         int same, TOut* K, int64_t ldk, cudaStream_t stream) {
    if (m <= 0 || n2 <= 0) return BGB_OK;
    dim3 grid((unsigned)ceil_div(n2, KB_TILE), (unsigned)ceil_div(m, KB_TILE));
    kernel_matrix_kernel<TIn, TAcc, TOut><<<grid, 256, 0, stream>>>(
        X1, m, X2, n2, d, inv_ls, outputscale, kind, diag_add, same, K, ldk, nullptr, nullptr,
        0.f, nullptr, 0, nullptr, 0);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int launch_kernel_matrix_zt(const float* Z1T, int64_t ldz1, int64_t m, const float* Z2T,
                            int64_t ldz2, int64_t n2, int d, double outputscale, int kind,
                            float* K, __half* K16, __half* K16_lo, float k16_scale, int64_t ldk,
                            cudaStream_t stream) {
    if (m <= 0 || n2 <= 0) return BGB_OK;
    if (Z1T == nullptr || Z2T == nullptr || ldz1 < m || ldz2 < n2) return BGB_ERR_ARG;
    if (K == nullptr && (K16 == nullptr || K16_lo == nullptr)) return BGB_ERR_ARG;
    dim3 grid((unsigned)ceil_div(n2, KB_TILE), (unsigned)ceil_div(m, KB_TILE));
    kernel_matrix_kernel<float, float, float><<<grid, 256, 0, stream>>>(
        nullptr, m, nullptr, n2, d, nullptr, outputscale, kind, 0.0, 0, K, ldk, K16, K16_lo,
        k16_scale, Z1T, ldz1, Z2T, ldz2);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

template int launch_kernel_matrix<double, double, double>(const double*, int64_t, const double*,
                                                          int64_t, int, const double*, double,
                                                          int, double, int, double*, int64_t,
                                                          cudaStream_t);
template int launch_kernel_matrix<double, float, float>(const double*, int64_t, const double*,
                                                        int64_t, int, const double*, double, int,
                                                        double, int, float*, int64_t,
                                                        cudaStream_t);

}  // namespace bgb
