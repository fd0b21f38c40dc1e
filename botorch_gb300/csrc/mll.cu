// (a3) Exact marginal log-likelihood of the training targets and its gradient
// w.r.t. the hyperparameters, float64, from the training cache (L, L^-1, alpha):
// the loss that hyperparameter fitting minimises (fit_gpytorch_mll with
// gpytorch's ExactMarginalLogLikelihood; no priors). With K = s k(X, X) + noise I
// (s the outputscale), y the standardised targets and m the mean constant:
//   mll           = (-1/2 (y - m)^T alpha - sum_i log L_ii - n/2 log 2 pi) / n
//   W             = alpha alpha^T - K^-1,  K^-1 = L^-T L^-1
//   d mll / d s   = (1/2) sum_ij W_ij k_ij / n
//   d mll / d l_k = -(s / l_k) sum_ij W_ij kappa'(r2_ij) dz_ijk^2 / n   (dz = scaled difference)
//   d mll / d noise = (1/2) tr(W) / n,   d mll / d m = sum_i alpha_i / n
// The pair sums run over the lower triangle of 32 x 32 tiles (off-diagonal
// pairs counted twice); each CTA writes its partial sums, and a second pass
// adds them in a fixed order, so the result does not depend on scheduling.
#include <math.h>

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int kMllTile = 32;
constexpr int kMllThreads = 256;

template <int DMAX>
__global__ void __launch_bounds__(kMllThreads) mll_pair_kernel(
    const double* __restrict__ X, int64_t n, int d, const double* __restrict__ inv_ls, int kind,
    const double* __restrict__ alpha, const double* __restrict__ Kinv, double* __restrict__ part) {
    // tile index t -> (ti, tj), tj <= ti, over the lower triangle of tiles
    const int64_t t = blockIdx.x;
    int64_t ti = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) / 2.0);
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    while (ti * (ti + 1) / 2 > t) --ti;
    const int64_t tj = t - ti * (ti + 1) / 2;
    const int64_t i0 = ti * kMllTile, j0 = tj * kMllTile;
    __shared__ double zi[kMllTile][DMAX + 1], zj[kMllTile][DMAX + 1];
    __shared__ double ai[kMllTile], aj[kMllTile];
    __shared__ double red[kMllThreads / 32][DMAX + 1];
    const int tid = threadIdx.x;
    for (int p = tid; p < kMllTile * DMAX; p += kMllThreads) {
        const int r = p / DMAX, k = p % DMAX;
        zi[r][k] = (k < d && i0 + r < n) ? X[(i0 + r) * d + k] * inv_ls[k] : 0.0;
        zj[r][k] = (k < d && j0 + r < n) ? X[(j0 + r) * d + k] * inv_ls[k] : 0.0;
    }
    if (tid < kMllTile) {
        ai[tid] = (i0 + tid < n) ? alpha[i0 + tid] : 0.0;
        aj[tid] = (j0 + tid < n) ? alpha[j0 + tid] : 0.0;
    }
    __syncthreads();
    double acc[DMAX + 1];
#pragma unroll
    for (int k = 0; k <= DMAX; ++k) acc[k] = 0.0;
    for (int p = tid; p < kMllTile * kMllTile; p += kMllThreads) {
        const int r = p / kMllTile, c = p % kMllTile;
        const int64_t i = i0 + r, j = j0 + c;
        if (i >= n || j >= n || j > i) continue;
        const double w = (i == j ? 1.0 : 2.0) * (ai[r] * aj[c] - Kinv[i * n + j]);
        double dz2[DMAX];
        double r2 = 0.0;
#pragma unroll
        for (int k = 0; k < DMAX; ++k) {
            const double df = zi[r][k] - zj[c][k];
            dz2[k] = df * df;
            r2 += dz2[k];
        }
        acc[DMAX] += w * kappa<double>(kind, r2);
        const double wd = w * dkappa_dr2<double>(kind, r2);
#pragma unroll
        for (int k = 0; k < DMAX; ++k) acc[k] += wd * dz2[k];
    }
    const int lane = tid % 32, warp = tid / 32;
#pragma unroll
    for (int k = 0; k <= DMAX; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    for (int k = tid; k <= DMAX; k += kMllThreads) {
        double v = 0.0;
        for (int w = 0; w < kMllThreads / 32; ++w) v += red[w][k];
        part[t * (DMAX + 1) + k] = v;
    }
}

// out[0] = -(1/2) (y - m)^T alpha - sum log L_ii, out[1] = tr(W), out[2] = sum alpha
__global__ void mll_scalars_kernel(const double* __restrict__ y, double m, const double* __restrict__ L,
                                   const double* __restrict__ alpha, const double* __restrict__ Kinv,
                                   int64_t n, double* __restrict__ out) {
    __shared__ double red[3][32];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double a = alpha[i];
        s0 += -0.5 * (y[i] - m) * a - log(L[i * n + i]);
        s1 += a * a - Kinv[i * n + i];
        s2 += a;
    }
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
        red[0][warp] = s0;
        red[1][warp] = s1;
        red[2][warp] = s2;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) v += red[threadIdx.x][w];
        out[threadIdx.x] = v;
    }
}

// out[3 + k] = sum over tiles of part[., k], k <= dmax (fixed order)
__global__ void mll_part_sum_kernel(const double* __restrict__ part, int64_t tiles, int width,
                                    double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= width) return;
    double v = 0.0;
    for (int64_t t = 0; t < tiles; ++t) v += part[t * width + k];
    out[3 + k] = v;
}

int64_t mll_tiles(int64_t n) {
    const int64_t tn = ceil_div(n, kMllTile);
    return tn * (tn + 1) / 2;
}

int mll_dmax(int d) {
    return d <= 8 ? 8 : d <= 16 ? 16 : d <= 24 ? 24 : d <= 32 ? 32 : d <= 64 ? 64 : 0;
}

}  // namespace

size_t mll_workspace_bytes(int64_t n, int d) {
    const int dm = mll_dmax(d);
    if (dm == 0 || n <= 0) return 0;
    return align_up(sizeof(double) * (size_t)n * n) +
           align_up(sizeof(double) * (size_t)mll_tiles(n) * (dm + 1)) +
           align_up(sizeof(double) * (size_t)(dm + 4));
}

int gp_mll(const double* X, int64_t n, int d, const double* inv_ls, double outputscale, int kind,
           double mean_constant, const double* y, const double* L, const double* Linv,
           const double* alpha, double* out_host, void* ws, size_t ws_bytes, cudaStream_t st) {
    const int dm = mll_dmax(d);
    if (dm == 0) return BGB_ERR_UNSUPPORTED;
    if (ws == nullptr || ws_bytes < mll_workspace_bytes(n, d)) return BGB_ERR_WORKSPACE;
    Arena ar{static_cast<char*>(ws), ws_bytes, 0};
    double* Kinv = ar.take<double>(n * n);
    const int64_t tiles = mll_tiles(n);
    double* part = ar.take<double>(tiles * (dm + 1));
    double* sums = ar.take<double>(dm + 4);
    // K^-1 = L^-T L^-1, lower triangle (k >= max(row, col))
    int rc = gemm_f64(n, n, n, 1.0, Linv, n, 1, Linv, n, 0, 0.0, Kinv, n, KAB_LOWER_T, 1, nullptr,
                      st);
    if (rc) return rc;
#define BGB_MLL(DM)                                                                              \
    mll_pair_kernel<DM><<<(unsigned)tiles, kMllThreads, 0, st>>>(X, n, d, inv_ls, kind, alpha,   \
                                                                 Kinv, part)
    if (dm == 8) BGB_MLL(8);
    else if (dm == 16) BGB_MLL(16);
    else if (dm == 24) BGB_MLL(24);
    else if (dm == 32) BGB_MLL(32);
    else BGB_MLL(64);
#undef BGB_MLL
    BGB_CHECK_LAUNCH();
    mll_scalars_kernel<<<1, 1024, 0, st>>>(y, mean_constant, L, alpha, Kinv, n, sums);
    BGB_CHECK_LAUNCH();
    mll_part_sum_kernel<<<1, 128, 0, st>>>(part, tiles, dm + 1, sums);
    BGB_CHECK_LAUNCH();
    double h[68];
    BGB_CUDA_TRY(cudaMemcpyAsync(h, sums, sizeof(double) * (dm + 4), cudaMemcpyDeviceToHost, st));
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    const double nn = (double)n;
    // h[0] = -(1/2)(y-m)^T alpha - sum log L_ii, h[1] = tr(W), h[2] = sum alpha,
    // h[3 + k] = sum W kappa' dz_k^2 (k < d), h[3 + dm] = sum W kappa
    out_host[0] = (h[0] - 0.5 * nn * log(2.0 * M_PI)) / nn;
    for (int k = 0; k < d; ++k) out_host[1 + k] = -outputscale * h[3 + k] / nn;  // times 1 / l_k below
    out_host[1 + d] = 0.5 * h[3 + dm] / nn;
    out_host[2 + d] = 0.5 * h[1] / nn;
    out_host[3 + d] = h[2] / nn;
    return BGB_OK;
}

}  // namespace bgb
