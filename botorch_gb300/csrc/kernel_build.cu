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
#include "bgb_qbatch.cuh"

namespace bgb {

namespace {

constexpr int KB_TILE = 64;
constexpr int KB_DCHUNK = 32;


// K16 == nullptr: plain output K. Otherwise (float32 arithmetic only) the output
// is the scaled float16 split for the tensor-core GEMM: with w = k16_scale * v,
// K16 = f16(w), K16_lo = f16(w - K16) (K is not written).
template <typename TIn, typename TAcc, typename TOut>
__device__ __forceinline__ void kernel_matrix_body(
    const TIn* __restrict__ X1, int64_t m, const TIn* __restrict__ X2, int64_t n2, int d,
    const double* __restrict__ inv_ls, double outputscale, int kind, double diag_add,
    int same, TOut* __restrict__ K, int64_t ldk, __half* __restrict__ K16,
    __half* __restrict__ K16_lo, float k16_scale, const float* __restrict__ Z1T, int64_t ldz1,
    const float* __restrict__ Z2T, int64_t ldz2, int64_t bx, int64_t by) {
    __shared__ __align__(16) TAcc s1[KB_DCHUNK][KB_TILE];
    __shared__ __align__(16) TAcc s2[KB_DCHUNK][KB_TILE];
    // thread (tx, ty): rows 4 ty + u, columns 4 tx + v (u, v < 4): the row and
    // column coordinates are 16-byte shared loads per k (broadcast within a
    // half-warp) and the outputs are vector stores of 4 consecutive entries
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int64_t row0 = by * KB_TILE, col0 = bx * KB_TILE;
    TAcc acc[4][4];
    float2 acc2[4][2];  // packed accumulators of the float32 form
#pragma unroll
    for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = TAcc(0);
        acc2[a][0] = acc2[a][1] = make_float2(0.f, 0.f);
    }
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
        if constexpr (sizeof(TAcc) == 4) {
            // packed float32 pairs of columns: the same correctly rounded
            // (a - b) and fma(df, df, acc) as the scalar form, two lanes at a time
            const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll 4
            for (int kk = 0; kk < kc; ++kk) {
                const float4 bv = *reinterpret_cast<const float4*>(&s2[kk][4 * tx]);
                const float4 av = *reinterpret_cast<const float4*>(&s1[kk][4 * ty]);
                const float2 b01 = make_float2(bv.x, bv.y), b23 = make_float2(bv.z, bv.w);
                const float avs[4] = {av.x, av.y, av.z, av.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float au = avs[u];
                    const float2 a2 = make_float2(au, au);
                    const float2 d01 = __ffma2_rn(b01, m1, a2);
                    const float2 d23 = __ffma2_rn(b23, m1, a2);
                    acc2[u][0] = __ffma2_rn(d01, d01, acc2[u][0]);
                    acc2[u][1] = __ffma2_rn(d23, d23, acc2[u][1]);
                }
            }
        } else {
#pragma unroll 4
            for (int kk = 0; kk < kc; ++kk) {
                TAcc a[4], b[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) a[u] = s1[kk][4 * ty + u];
                const double2 b01 = *reinterpret_cast<const double2*>(&s2[kk][4 * tx]);
                const double2 b23 = *reinterpret_cast<const double2*>(&s2[kk][4 * tx + 2]);
                b[0] = b01.x; b[1] = b01.y; b[2] = b23.x; b[3] = b23.y;
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        TAcc df = a[u] - b[v];
                        acc[u][v] += df * df;
                    }
            }
        }
        __syncthreads();
    }
    if constexpr (sizeof(TAcc) == 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            acc[u][0] = acc2[u][0].x;
            acc[u][1] = acc2[u][0].y;
            acc[u][2] = acc2[u][1].x;
            acc[u][3] = acc2[u][1].y;
        }
    }
    const int64_t j0 = col0 + 4 * tx;
    const bool full = (j0 + 3 < n2) && (ldk % 4) == 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t i = row0 + 4 * ty + u;
        if (i >= m) continue;
        TAcc val[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            val[v] = TAcc(outputscale) * kappa<TAcc>(kind, acc[u][v]);
            if (same && i == j0 + v) val[v] += TAcc(diag_add);
        }
        if constexpr (sizeof(TAcc) == 4) {
            if (K16 != nullptr) {
                __half hh[4], ll[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const float w = (float)val[v] * k16_scale;
                    hh[v] = __float2half_rn(w);
                    ll[v] = __float2half_rn(w - __half2float(hh[v]));
                }
                if (full && (reinterpret_cast<uintptr_t>(K16) % 8) == 0 &&
                    (reinterpret_cast<uintptr_t>(K16_lo) % 8) == 0) {
                    *reinterpret_cast<uint2*>(K16 + i * ldk + j0) = *reinterpret_cast<const uint2*>(hh);
                    *reinterpret_cast<uint2*>(K16_lo + i * ldk + j0) = *reinterpret_cast<const uint2*>(ll);
                } else {
#pragma unroll
                    for (int v = 0; v < 4; ++v)
                        if (j0 + v < n2) {
                            K16[i * ldk + j0 + v] = hh[v];
                            K16_lo[i * ldk + j0 + v] = ll[v];
                        }
                }
                continue;
            }
        }
        if (full && sizeof(TOut) == 4 && (reinterpret_cast<uintptr_t>(K) % 16) == 0) {
            *reinterpret_cast<float4*>(K + i * ldk + j0) =
                make_float4((float)val[0], (float)val[1], (float)val[2], (float)val[3]);
        } else {
#pragma unroll
            for (int v = 0; v < 4; ++v)
                if (j0 + v < n2) K[i * ldk + j0 + v] = (TOut)val[v];
        }
    }
}

template <typename TIn, typename TAcc, typename TOut>
__global__ void __launch_bounds__(256) kernel_matrix_kernel(
    const TIn* __restrict__ X1, int64_t m, const TIn* __restrict__ X2, int64_t n2, int d,
    const double* __restrict__ inv_ls, double outputscale, int kind, double diag_add,
    int same, TOut* __restrict__ K, int64_t ldk, __half* __restrict__ K16,
    __half* __restrict__ K16_lo, float k16_scale, const float* __restrict__ Z1T, int64_t ldz1,
    const float* __restrict__ Z2T, int64_t ldz2) {
    kernel_matrix_body<TIn, TAcc, TOut>(X1, m, X2, n2, d, inv_ls, outputscale, kind, diag_add,
                                        same, K, ldk, K16, K16_lo, k16_scale, Z1T, ldz1, Z2T, ldz2,
                                        blockIdx.x, blockIdx.y);
}

// Model of this CTA in a grouped launch: the largest m with off[m] <= blockIdx.x.
__device__ __forceinline__ int km_group_model(const GroupTab& t) {
    int lo = 0, hi = t.nm - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t.off[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// grouped: candidates scaled by 1 / lengthscale into k-major float32 (zt)
__global__ void scale_rows_group_kernel(const GroupTab t) {
    const int m = km_group_model(t);
    const KmG& g = static_cast<const KmG*>(t.args)[m];
    const int64_t idx = ((int64_t)blockIdx.x - t.off[m]) * blockDim.x + threadIdx.x;
    if (idx >= g.rows * g.d) return;
    const int64_t i = idx / g.d;
    const int k = (int)(idx % g.d);
    g.zt[(int64_t)k * g.rows + i] = (float)(g.X[idx] * g.inv_ls[k]);
}

// grouped: K(X, Xt) of every model as its scaled float16 split; model m's CTAs
// cover its (column tile, row tile) grid row-major in row tiles
__global__ void __launch_bounds__(256) kernel_matrix_group_kernel(const GroupTab t) {
    const int m = km_group_model(t);
    const KmG& g = static_cast<const KmG*>(t.args)[m];
    const int64_t lb = (int64_t)blockIdx.x - t.off[m];
    kernel_matrix_body<float, float, float>(nullptr, g.rows, nullptr, g.n, g.d, nullptr,
                                            g.outputscale, g.kind, 0.0, 0, nullptr, g.ldk, g.K16,
                                            g.K16_lo, g.k16_scale, g.zt, g.rows, g.Xs32, g.n,
                                            lb % g.gx, lb / g.gx);
}

}  // namespace

int64_t kernel_matrix_col_tiles(int64_t n) { return ceil_div(n, (int64_t)KB_TILE); }
int64_t kernel_matrix_row_tiles(int64_t m) { return ceil_div(m, (int64_t)KB_TILE); }

int launch_kernel_matrix_group(const GroupTab& t_scale, int64_t total_scale, const GroupTab& t_km,
                               int64_t total_km, cudaStream_t stream) {
    if (total_scale > 0x7fffffff || total_km > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
    if (total_scale > 0) {
        scale_rows_group_kernel<<<(unsigned)total_scale, 256, 0, stream>>>(t_scale);
        BGB_CHECK_LAUNCH();
    }
    if (total_km > 0) {
        kernel_matrix_group_kernel<<<(unsigned)total_km, 256, 0, stream>>>(t_km);
        BGB_CHECK_LAUNCH();
    }
    return BGB_OK;
}

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
