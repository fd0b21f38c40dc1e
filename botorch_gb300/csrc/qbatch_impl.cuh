// (d) + (e) + adjoint: the per-t-batch part of the path.
//
// The cross-covariance enters through V = K(X, Xt) L^-T (the triangular solve
// against the training Cholesky factor, computed by the GEMM before these
// kernels), as in the reference's root-inverse form of the predictive
// covariance:
//  row_dots       mu = m + V beta (beta = L^-1 (y - m)) and P = V Vb^T, one warp per row.
//  sigma_reduce   Sigma_qq = K(X,X) - V V^T, Sigma_qb = K(X,Xb) - P. Reads the q rows of
//                 V of each t-batch once.
//  batch_step     one CTA per t-batch, float64: untransform, bl = Sigma_qb Lb^-T,
//                 br = psd_safe_cholesky(Sigma_qq - bl bl^T) with per-batch jitter
//                 retries, Y = mu + [bl, br] z over the S base samples, the qLogNEI
//                 reduction (log_fatplus, fatmax over q, logmeanexp over S) or the
//                 qEI reduction, and in reverse the seeds of the adjoint
//                 (d value / d Sigma_qq, d Sigma_qb, d mu) through the sample
//                 reduction, the sample step and the q x q Cholesky.
//  mix_rows       H = gmu beta^T - 2 Gqq V - Gqb Vb  (d value / d V), per t-batch.
//  adjoint        d value / d X with dKc = H L^-1 (the second triangular GEMM, D),
//                 contracted with d K(X, Xt) / d X while recomputing
//                 the scaled distances to Xt instead of storing K(X, Xt); plus the
//                 K(X, X) and K(X, Xb) terms.
//
// This file holds the kernels and their launchers. It is compiled as several
// translation units (qbatch_*.cu), each defining one BGB_QB_* selector, so
// that the launchers and the kernel instantiations they pull in are split
// over parallel compiler processes.
#pragma once

#include <math.h>

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"
#include "bgb_qbatch.cuh"

namespace bgb {

// SMs of the current device (defined in the statistics translation unit)
int sm_count();

namespace {

// ---------------------------------------------------------------- sigma_reduce
template <typename T, int QMAX>
__global__ void __launch_bounds__(256) sigma_reduce_kernel(QBatchArgs a, const T* __restrict__ P,
                                                           const T* __restrict__ C, int64_t ldc) {
    constexpr int NP = QMAX * (QMAX + 1) / 2;
    const int q = a.q;
    const int64_t n = a.n;
    const int64_t bidx = blockIdx.x;
    const int64_t rbase = bidx * q;
    // Each thread sums n / blockDim terms per pair in T (float64 for the plain
    // path, float32 for the mixed one); the cross-thread reduction is float64.
    T acc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[p] = T(0);
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
        T w[QMAX], k[QMAX];
#pragma unroll
        for (int i = 0; i < QMAX; ++i) {
            w[i] = (i < q) ? C[(rbase + i) * ldc + c] : T(0);
            k[i] = w[i];
        }
        int p = 0;
#pragma unroll
        for (int i = 0; i < QMAX; ++i)
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                acc[p] = fma(w[i], k[j], acc[p]);
                ++p;
            }
    }
    __shared__ double red[8][NP];
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        double v = (double)acc[p];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][p] = v;
    }
    __syncthreads();
    const int nw = blockDim.x / 32;
    const int d = a.d;
    for (int p = threadIdx.x; p < NP; p += blockDim.x) {
        // p -> (i, j), j <= i
        int i = 0;
        while ((i + 1) * (i + 2) / 2 <= p) ++i;
        int j = p - i * (i + 1) / 2;
        if (i >= q) continue;
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += red[w][p];
        // K(x_i, x_j)
        const double* xi = a.X + (rbase + i) * d;
        const double* xj = a.X + (rbase + j) * d;
        double r2 = 0.0;
        for (int k = 0; k < d; ++k) {
            double df = (xi[k] - xj[k]) * a.inv_ls[k];
            r2 = fma(df, df, r2);
        }
        double kij = a.outputscale * kappa<double>(a.kernel, r2);
        double v = kij - s;
        a.sig[(bidx * q + i) * q + j] = v;
        a.sig[(bidx * q + j) * q + i] = v;
    }
    const int r = a.r;
    for (int p = threadIdx.x; p < q * (r + 1); p += blockDim.x) {
        int i = p / (r + 1), kb = p % (r + 1);
        if (kb < r) {
            const double cval = (double)P[(rbase + i) * r + kb];
            const double* xi = a.X + (rbase + i) * d;
            const double* xb = a.Xb + (int64_t)kb * d;
            double r2 = 0.0;
            for (int k = 0; k < d; ++k) {
                double df = (xi[k] - xb[k]) * a.inv_ls[k];
                r2 = fma(df, df, r2);
            }
            a.sqb[(bidx * q + i) * r + kb] = a.outputscale * kappa<double>(a.kernel, r2) - cval;
        }
    }
}

// Fallback for q > 8: one warp per (t-batch, pair).
template <typename T>
__global__ void sigma_reduce_pairs_kernel(QBatchArgs a, const T* __restrict__ P,
                                          const T* __restrict__ C, int64_t ldc) {
    const int q = a.q;
    const int64_t n = a.n;
    const int64_t warp_id = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    const int64_t npairs = (int64_t)q * q;
    if (warp_id >= a.b * npairs) return;
    const int64_t bidx = warp_id / npairs;
    const int i = (int)((warp_id % npairs) / q), j = (int)(warp_id % q);
    if (j > i) return;
    const int64_t rbase = bidx * q;
    double s = 0.0;
    for (int64_t c = lane; c < n; c += 32)
        s += (double)(C[(rbase + i) * ldc + c] * C[(rbase + j) * ldc + c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane != 0) return;
    const int d = a.d;
    const double* xi = a.X + (rbase + i) * d;
    const double* xj = a.X + (rbase + j) * d;
    double r2 = 0.0;
    for (int k = 0; k < d; ++k) {
        double df = (xi[k] - xj[k]) * a.inv_ls[k];
        r2 = fma(df, df, r2);
    }
    double v = a.outputscale * kappa<double>(a.kernel, r2) - s;
    a.sig[(bidx * q + i) * q + j] = v;
    a.sig[(bidx * q + j) * q + i] = v;
    if (j == 0) {
        const int r = a.r;
        for (int kb = 0; kb < r; ++kb) {
            const double cval = (double)P[(rbase + i) * r + kb];
            {
                const double* xb = a.Xb + (int64_t)kb * d;
                double rb2 = 0.0;
                for (int k = 0; k < d; ++k) {
                    double df = (xi[k] - xb[k]) * a.inv_ls[k];
                    rb2 = fma(df, df, rb2);
                }
                a.sqb[(bidx * q + i) * r + kb] = a.outputscale * kappa<double>(a.kernel, rb2) - cval;
            }
        }
    }
}

// ---------------------------------------------------------------- row_dots
// mu[i] = m + V[i,:] . beta and P[i,k] = V[i,:] . Vb[k,:] (k < r), one warp per
// row of V. float32 inputs use compensated per-lane sums; the cross-lane sum is
// float64. (mu = K(X,Xt) alpha = V beta with beta = L^-1 (y - m): the bounded
// factor avoids the cancellation of K(X,Xt) alpha.)
template <typename T>
__device__ __forceinline__ void comp_add(T& s, T& c, T x) {
    T y = x - c;
    T t = s + y;
    c = (t - s) - y;
    s = t;
}

template <typename T>
__global__ void __launch_bounds__(256) row_dots_kernel(QBatchArgs a, const T* __restrict__ V,
                                                       int64_t ldv, const T* __restrict__ beta,
                                                       const T* __restrict__ Vb, T* __restrict__ P) {
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    const int64_t rows = a.b * a.q, n = a.n;
    if (row >= rows) return;
    const int r = a.r;
    const T* v = V + row * ldv;
    for (int k0 = -1; k0 < r; k0 += 8) {
        // k = -1 is the beta dot product, k >= 0 the baseline rows
        T s[8], c[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) { s[u] = T(0); c[u] = T(0); }
        for (int64_t j = lane; j < n; j += 32) {
            const T vj = v[j];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = k0 + u;
                if (k < r) {
                    const T w = (k < 0) ? beta[j] : Vb[(int64_t)k * n + j];
                    comp_add<T>(s[u], c[u], vj * w);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            double tot = (double)s[u] - (double)c[u];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
            const int k = k0 + u;
            if (lane == 0 && k < r) {
                if (k < 0) a.mu[row] = a.mean_constant + tot;
                else P[row * r + k] = (T)tot;
            }
        }
    }
}

// ---------------------------------------------------------------- qstats
// row_dots + sigma_reduce in one pass over V for q <= 8, r <= 4: one CTA of 256
// threads per t-batch reads its q rows of V once with 16-byte loads and forms
//   G = V V^T (lower triangle), mu = m + V beta, P = V Vb^T,
//   Sigma_qq = K(X,X) - G, Sigma_qb = K(X,Xb) - P.
// Per thread: T sums over n / 256 columns (mu compensated). Across the 32 lanes
// of a warp: a butterfly reduce-scatter of (hi, lo) pairs with error-free
// two-sums, so each lane ends with NPAD / 32 totals and moves only about twice
// that many values. Across the 8 warps: float64.
template <typename T> struct Vec16;
template <> struct Vec16<float> {
    using type = float4;
    static constexpr int E = 4;
    static __device__ __forceinline__ float at(const float4& v, int e) {
        return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
    }
};
template <> struct Vec16<double> {
    using type = double2;
    static constexpr int E = 2;
    static __device__ __forceinline__ double at(const double2& v, int e) { return e == 0 ? v.x : v.y; }
};

// (h, l) += (bh, bl), with the rounding error of h + bh kept in l (Knuth two-sum)
template <typename T>
__device__ __forceinline__ void add_pair(T& h, T& l, T bh, T bl) {
    const T s = h + bh;
    const T bb = s - h;
    const T e = (h - (s - bb)) + (bh - bb);
    h = s;
    l = l + bl + e;
}

// Model of this CTA in a grouped launch: the largest m with off[m] <= blockIdx.x.
__device__ __forceinline__ int group_model(const GroupTab& t) {
    int lo = 0, hi = t.nm - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t.off[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

constexpr int kQstatsThreads = 128;  // 8 columns of 4 per thread at n = 4096: the tail reduction is paid per 128 threads

// outputscale * kappa between row `ri` of X and row `rj` of X (rj >= 0) or
// baseline point `kb` (rj < 0). Float path (T = float with a.zt set): float32
// over the scaled candidate coordinates a.zt, like the float32 kernel build;
// otherwise float64.
// zb: the baseline points' scaled coordinates (float, r x d) when staged by the
// caller, else nullptr.
template <typename T>
__device__ __forceinline__ double kernel_pair(const QBatchArgs& a, int64_t ri, int64_t rj, int kb,
                                              const float* zb = nullptr) {
    const int d = a.d;
    if (sizeof(T) == 4 && a.zt != nullptr) {
        const int64_t rows = a.b * a.q;
        float r2 = 0.f;
        for (int k = 0; k < d; ++k) {
            const float zj = rj >= 0 ? a.zt[(int64_t)k * rows + rj]
                                     : (zb != nullptr ? zb[kb * d + k]
                                                      : (float)(a.Xb[(int64_t)kb * d + k] * a.inv_ls[k]));
            const float df = a.zt[(int64_t)k * rows + ri] - zj;
            r2 = fmaf(df, df, r2);
        }
        return (double)((float)a.outputscale * kappa<float>(a.kernel, r2));
    }
    const double* xi = a.X + ri * d;
    const double* xj = rj >= 0 ? a.X + rj * d : a.Xb + (int64_t)kb * d;
    double r2 = 0.0;
    for (int k = 0; k < d; ++k) {
        const double df = (xi[k] - xj[k]) * a.inv_ls[k];
        r2 = fma(df, df, r2);
    }
    return a.outputscale * kappa<double>(a.kernel, r2);
}

template <int NV>
struct PadPow2 {
    static constexpr int value = NV <= 32 ? 32 : NV <= 64 ? 64 : 128;
};

template <typename T, int QMAX, int RM>
__device__ __forceinline__ void qstats_body(const QBatchArgs& a, const T* __restrict__ V,
                                            int64_t ldv, const T* __restrict__ beta,
                                            const T* __restrict__ Vb, int vec_ok, int64_t bidx_) {
    using VT = typename Vec16<T>::type;
    constexpr int E = Vec16<T>::E;
    constexpr int NG = QMAX * (QMAX + 1) / 2;
    constexpr int NV = NG + QMAX + QMAX * RM;
    constexpr int NPAD = PadPow2<NV>::value;
    constexpr int NPL = NPAD / 32;  // totals per lane after the butterfly
    const int q = a.q, r = a.r, tid = threadIdx.x;
    const int64_t n = a.n, bidx = bidx_, rbase = bidx * q;
    T g[NG], ms[QMAX], mc[QMAX], pv[QMAX * RM];
#pragma unroll
    for (int p = 0; p < NG; ++p) g[p] = T(0);
#pragma unroll
    for (int i = 0; i < QMAX; ++i) { ms[i] = T(0); mc[i] = T(0); }
#pragma unroll
    for (int p = 0; p < QMAX * RM; ++p) pv[p] = T(0);
    // one column's contribution
    auto consume = [&](const T* w, T bt, const T* vb) {
        int p = 0;
#pragma unroll
        for (int i = 0; i < QMAX; ++i) {
#pragma unroll
            for (int j = 0; j <= i; ++j) {
                g[p] = fma(w[i], w[j], g[p]);
                ++p;
            }
            comp_add<T>(ms[i], mc[i], w[i] * bt);
#pragma unroll
            for (int k = 0; k < RM; ++k) pv[i * RM + k] = fma(w[i], vb[k], pv[i * RM + k]);
        }
    };
    const int64_t nvec = vec_ok ? n / E : 0;
    for (int64_t u = tid; u < nvec; u += kQstatsThreads) {
        VT wv[QMAX], bv[RM];
#pragma unroll
        for (int i = 0; i < QMAX; ++i)
            if (i < q) wv[i] = *reinterpret_cast<const VT*>(V + (rbase + i) * ldv + u * E);
        const VT btv = *reinterpret_cast<const VT*>(beta + u * E);
#pragma unroll
        for (int k = 0; k < RM; ++k)
            if (k < r) bv[k] = *reinterpret_cast<const VT*>(Vb + (int64_t)k * n + u * E);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            T w[QMAX], vb[RM];
#pragma unroll
            for (int i = 0; i < QMAX; ++i) w[i] = (i < q) ? Vec16<T>::at(wv[i], e) : T(0);
#pragma unroll
            for (int k = 0; k < RM; ++k) vb[k] = (k < r) ? Vec16<T>::at(bv[k], e) : T(0);
            consume(w, Vec16<T>::at(btv, e), vb);
        }
    }
    for (int64_t c = nvec * E + tid; c < n; c += kQstatsThreads) {
        T w[QMAX], vb[RM];
#pragma unroll
        for (int i = 0; i < QMAX; ++i) w[i] = (i < q) ? V[(rbase + i) * ldv + c] : T(0);
#pragma unroll
        for (int k = 0; k < RM; ++k) vb[k] = (k < r) ? Vb[(int64_t)k * n + c] : T(0);
        consume(w, beta[c], vb);
    }
    // butterfly reduce-scatter over the lanes
    T h[NPAD], l[NPAD];
#pragma unroll
    for (int p = 0; p < NPAD; ++p) {
        if (p < NG) { h[p] = g[p]; l[p] = T(0); }
        else if (p < NG + QMAX) { h[p] = ms[p - NG]; l[p] = -mc[p - NG]; }
        else if (p < NV) { h[p] = pv[p - NG - QMAX]; l[p] = T(0); }
        else { h[p] = T(0); l[p] = T(0); }
    }
    const int lane = tid % 32, warp = tid / 32;
    int base = 0;
#pragma unroll
    for (int lvl = 0; lvl < 5; ++lvl) {
        const int half = NPAD >> (lvl + 1);
        const bool up = (lane >> lvl) & 1;
        if (up) base += half;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const T sh = up ? h[i] : h[i + half], sl = up ? l[i] : l[i + half];
            T kh = up ? h[i + half] : h[i], kl = up ? l[i + half] : l[i];
            const T rh = __shfl_xor_sync(0xffffffffu, sh, 1 << lvl);
            const T rl = __shfl_xor_sync(0xffffffffu, sl, 1 << lvl);
            add_pair<T>(kh, kl, rh, rl);
            h[i] = kh;
            l[i] = kl;
        }
    }
    __shared__ double red[kQstatsThreads / 32][NPAD];
#pragma unroll
    for (int i = 0; i < NPL; ++i) red[warp][base + i] = (double)h[i] + (double)l[i];
    // the baseline's scaled coordinates for the cross terms, computed once across
    // the CTA (float64 products are scarce: a handful of warp instructions in
    // place of d per cross-term lane)
    constexpr int kZb = 4 * 64;
    __shared__ float s_zb[kZb];
    const bool stage_zb = sizeof(T) == 4 && a.zt != nullptr && r * a.d <= kZb;
    if (stage_zb)
        for (int p = tid; p < r * a.d; p += kQstatsThreads)
            s_zb[p] = (float)(a.Xb[p] * a.inv_ls[p % a.d]);
    __syncthreads();
    if (tid >= NV) return;
    double tot = 0.0;
#pragma unroll
    for (int w = 0; w < kQstatsThreads / 32; ++w) tot += red[w][tid];
    if (tid < NG) {
        int i = 0;
        while ((i + 1) * (i + 2) / 2 <= tid) ++i;
        const int j = tid - i * (i + 1) / 2;
        if (i >= q) return;
        const double v = kernel_pair<T>(a, rbase + i, rbase + j, 0) - tot;
        a.sig[(bidx * q + i) * q + j] = v;
        a.sig[(bidx * q + j) * q + i] = v;
    } else if (tid < NG + QMAX) {
        const int i = tid - NG;
        if (i < q) a.mu[rbase + i] = a.mean_constant + tot;
    } else {
        const int i = (tid - NG - QMAX) / RM, kb = (tid - NG - QMAX) % RM;
        if (i >= q || kb >= r) return;
        // P rounded to T as the two-kernel path stores it
        a.sqb[(bidx * q + i) * r + kb] =
            kernel_pair<T>(a, rbase + i, -1, kb, stage_zb ? s_zb : nullptr) - (double)(T)tot;
    }
}

template <typename T, int QMAX, int RM>
__global__ void __launch_bounds__(kQstatsThreads)
    qstats_kernel(const __grid_constant__ QBatchArgs a, const T* __restrict__ V, int64_t ldv,
                  const T* __restrict__ beta, const T* __restrict__ Vb, int vec_ok) {
    qstats_body<T, QMAX, RM>(a, V, ldv, beta, Vb, vec_ok, blockIdx.x);
}

template <typename T, int QMAX, int RM>
__global__ void __launch_bounds__(kQstatsThreads) qstats_group_kernel(const GroupTab t) {
    const int m = group_model(t);
    const QstatsG<T>& g = static_cast<const QstatsG<T>*>(t.args)[m];
    qstats_body<T, QMAX, RM>(g.a, g.V, g.ldv, g.beta, g.Vb, g.vec_ok, blockIdx.x - t.off[m]);
}

// ---------------------------------------------------------------- tiled statistics
// mu, Sigma_qq and Sigma_qb for q up to 32 in one pass over V: one CTA per
// t-batch stages 128-column tiles of its q rows of V, of beta and of the r rows
// of Vb in shared memory; each thread owns up to kQtOut of the q(q+1)/2 + q + q r
// dot products (pairs, mean, cross terms) and sums the tile's columns in four
// chains, starting at a lane-dependent column so the warp reads 32 different
// banks; tile partials add up in float64 (the mean's per tile compensated).
constexpr int kQtThreads = 256, kQtCols = 128, kQtOut = 3;

// With nsplit > 1 (few t-batches), CTA (t-batch, split) takes every nsplit-th
// block of tiles and writes its partial sums to part[(t-batch, split, output)];
// qstats_tile_finish_kernel adds the splits in order and writes the outputs.
template <typename T>
__device__ __forceinline__ void qstats_tile_outputs(const QBatchArgs& a, int q, int r,
                                                    int64_t bidx, int kind, int i, int j,
                                                    double tot);

template <typename T>
__global__ void __launch_bounds__(kQtThreads)
    qstats_tile_kernel(const __grid_constant__ QBatchArgs a, const T* __restrict__ V, int64_t ldv,
                       const T* __restrict__ beta, const T* __restrict__ Vb, int nsplit,
                       double* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char qt_raw[];
    T* S = reinterpret_cast<T*>(qt_raw);  // R x kQtCols, rows: V (q), beta, Vb (r)
    const int q = a.q, r = a.r, R = q + 1 + r;
    const int64_t n = a.n, bidx = blockIdx.x / nsplit, rbase = bidx * q;
    const int split = blockIdx.x % nsplit;
    const int np = q * (q + 1) / 2, nout = np + q + q * r;
    const int tid = threadIdx.x, lane = tid % 32;
    int ra[kQtOut], rb[kQtOut], kind[kQtOut];  // kind: 0 none, 1 pair, 2 mean, 3 cross
    double tot[kQtOut];
#pragma unroll
    for (int k = 0; k < kQtOut; ++k) {
        const int o = tid + k * kQtThreads;
        tot[k] = 0.0;
        ra[k] = rb[k] = 0;
        kind[k] = 0;
        if (o < np) {
            int i = 0;
            while ((i + 1) * (i + 2) / 2 <= o) ++i;
            ra[k] = i;
            rb[k] = o - i * (i + 1) / 2;
            kind[k] = 1;
        } else if (o < np + q) {
            ra[k] = o - np;
            rb[k] = q;
            kind[k] = 2;
        } else if (o < nout) {
            const int p = o - np - q;
            ra[k] = p / r;
            rb[k] = q + 1 + p % r;
            kind[k] = 3;
        }
    }
    for (int64_t c0 = (int64_t)split * kQtCols; c0 < n; c0 += (int64_t)nsplit * kQtCols) {
        const int64_t cw = (n - c0) < kQtCols ? (n - c0) : kQtCols;
        for (int idx = tid; idx < R * kQtCols; idx += kQtThreads) {
            const int row = idx / kQtCols, c = idx % kQtCols;
            T v = T(0);
            if (c < cw) {
                if (row < q) v = V[(rbase + row) * ldv + c0 + c];
                else if (row == q) v = beta[c0 + c];
                else v = Vb[(int64_t)(row - q - 1) * n + c0 + c];
            }
            S[idx] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kQtOut; ++k) {
            if (kind[k] == 0) continue;
            const T* x = S + ra[k] * kQtCols;
            const T* y = S + rb[k] * kQtCols;
            if (kind[k] != 2) {
                T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll 4
                for (int c = 0; c < kQtCols; c += 4) {
                    const int c_a = (c + lane) % kQtCols, c_b = (c + 1 + lane) % kQtCols;
                    const int c_c = (c + 2 + lane) % kQtCols, c_d = (c + 3 + lane) % kQtCols;
                    s0 = fma(x[c_a], y[c_a], s0);
                    s1 = fma(x[c_b], y[c_b], s1);
                    s2 = fma(x[c_c], y[c_c], s2);
                    s3 = fma(x[c_d], y[c_d], s3);
                }
                tot[k] += (double)((s0 + s1) + (s2 + s3));
            } else {
                T sh = T(0), sc = T(0);
                for (int c = 0; c < kQtCols; ++c) {
                    const int cc = (c + lane) % kQtCols;
                    comp_add<T>(sh, sc, x[cc] * y[cc]);
                }
                tot[k] += (double)sh - (double)sc;
            }
        }
        __syncthreads();
    }
    // the zero-padded columns of a partial last tile added nothing
#pragma unroll
    for (int k = 0; k < kQtOut; ++k) {
        if (kind[k] == 0) continue;
        if (nsplit > 1)
            part[((int64_t)bidx * nsplit + split) * nout + tid + k * kQtThreads] = tot[k];
        else
            qstats_tile_outputs<T>(a, q, r, bidx, kind[k], ra[k], rb[k], tot[k]);
    }
}

// sig / mu / sqb of output (kind, i, j) from its float64 sum
template <typename T>
__device__ __forceinline__ void qstats_tile_outputs(const QBatchArgs& a, int q, int r,
                                                    int64_t bidx, int kind, int i, int j,
                                                    double tot) {
    const int64_t rbase = bidx * q;
    if (kind == 1) {
        const double v = kernel_pair<T>(a, rbase + i, rbase + j, 0) - tot;
        a.sig[(bidx * q + i) * q + j] = v;
        a.sig[(bidx * q + j) * q + i] = v;
    } else if (kind == 2) {
        a.mu[rbase + i] = a.mean_constant + tot;
    } else if (kind == 3) {
        const int kb = j - q - 1;
        a.sqb[(bidx * q + i) * r + kb] = kernel_pair<T>(a, rbase + i, -1, kb) - tot;
    }
}

// one CTA per t-batch: the splits' partial sums in split order, then the outputs
template <typename T>
__global__ void __launch_bounds__(kQtThreads)
    qstats_tile_finish_kernel(const __grid_constant__ QBatchArgs a, int nsplit,
                              const double* __restrict__ part) {
    const int q = a.q, r = a.r;
    const int np = q * (q + 1) / 2, nout = np + q + q * r;
    const int64_t bidx = blockIdx.x;
    for (int o = threadIdx.x; o < nout; o += kQtThreads) {
        double tot = 0.0;
        for (int sp = 0; sp < nsplit; ++sp) tot += part[((int64_t)bidx * nsplit + sp) * nout + o];
        int kind, i, j;
        if (o < np) {
            i = 0;
            while ((i + 1) * (i + 2) / 2 <= o) ++i;
            j = o - i * (i + 1) / 2;
            kind = 1;
        } else if (o < np + q) {
            i = o - np;
            j = q;
            kind = 2;
        } else {
            const int p = o - np - q;
            i = p / r;
            j = q + 1 + p % r;
            kind = 3;
        }
        qstats_tile_outputs<T>(a, q, r, bidx, kind, i, j, tot);
    }
}

// ---------------------------------------------------------------- smooth pieces
// softplus with torch's threshold 20 (beta = 1)
__device__ __forceinline__ double softplus_t(double x) { return x > 20.0 ? x : log1p(exp(x)); }
__device__ __forceinline__ double softplus_grad(double x) {
    if (x > 20.0) return 1.0;
    double z = exp(x);
    return z / (z + 1.0);
}
// log_fatplus(u, tau) = log(tau * (softplus(u/tau) + 0.1 / (1 + (u/tau)^2)))
__device__ __forceinline__ double log_fatplus(double u, double tau) {
    double v = u / tau;
    return log(tau * (softplus_t(v) + 0.1 / (1.0 + v * v)));
}
__device__ __forceinline__ double dlog_fatplus(double u, double tau) {
    double v = u / tau;
    double c = 1.0 / (1.0 + v * v);
    double h = softplus_t(v) + 0.1 * c;
    double hp = softplus_grad(v) - 0.2 * v * c * c;
    return hp / (tau * h);
}
// pareto kernel of fatmax (alpha = 2): p(x) = 2 / (2 + 2x + x^2), p'(x) = -4 (1 + x) / (..)^2
__device__ __forceinline__ double pareto2(double x) { return 2.0 / (2.0 + 2.0 * x + x * x); }
__device__ __forceinline__ double dpareto2(double x) {
    double den = 2.0 + 2.0 * x + x * x;
    return -4.0 * (1.0 + x) / (den * den);
}

// float32 forms for the mixed path. One exponential serves softplus and its
// derivative; the divisions and the outer logarithm use the fast intrinsics
// (__fdividef, __logf: a few ulp), far inside the per-sample error budget.
// log_fatplus(u) = log(tau) + log(h(v)), d/du = h'(v) / (tau h(v)), v = u / tau,
// h(v) = softplus(v) + 0.1 / (1 + v^2)
__device__ __forceinline__ void log_fatplus_f(float v, float log_tau, float inv_tau, float& li,
                                              float& dli) {
    const float c = __fdividef(1.f, fmaf(v, v, 1.f));
    float sp, sg;
    if (v > 20.f) {  // torch softplus threshold (beta = 1)
        sp = v;
        sg = 1.f;
    } else {
        const float e = __expf(v);
        sp = log1pf(e);
        sg = __fdividef(e, e + 1.f);
    }
    const float h = fmaf(0.1f, c, sp);
    const float hp = sg - 0.2f * v * c * c;
    li = log_tau + __logf(h);
    dli = __fdividef(hp * inv_tau, h);
}
__device__ __forceinline__ float pareto2_f(float x) {
    return __fdividef(2.f, 2.f + 2.f * x + x * x);
}
__device__ __forceinline__ float dpareto2_f(float x) {
    const float den = 2.f + 2.f * x + x * x;
    return __fdividef(-4.f * (1.f + x), den * den);
}

// In-place Cholesky of a q x q row-major matrix (lower). Returns 0 or pivot+1.
__device__ int chol_small(double* A, int q) {
    for (int j = 0; j < q; ++j) {
        double v = A[j * q + j];
        for (int k = 0; k < j; ++k) v -= A[j * q + k] * A[j * q + k];
        if (!(v > 0.0)) return j + 1;
        double djj = sqrt(v);
        A[j * q + j] = djj;
        for (int i = j + 1; i < q; ++i) {
            double s = A[i * q + j];
            for (int k = 0; k < j; ++k) s -= A[i * q + k] * A[j * q + k];
            A[i * q + j] = s / djj;
        }
        for (int k = j + 1; k < q; ++k) A[j * q + k] = 0.0;
    }
    return 0;
}

// ---------------------------------------------------------------- batch_step
// Shared memory (doubles): Lq q*(r+q) | dLq q*(r+q) | M q*q | gA q*q | mu q | dmu q |
//                          t S | dY SC*q | scratch q*q
constexpr int kSampleChunk = 128;

#if defined(BGB_QB_STEP)
// The float64 path's step (the mixed path's is batch_step_f32_kernel).
__global__ void __launch_bounds__(128) batch_step_kernel(QBatchArgs a, int backward) {
    extern __shared__ double sm[];
    const int q = a.q, r = a.r, S = a.S, D = r + q;
    const int64_t bidx = blockIdx.x;
    double* Lq = sm;
    double* dLq = Lq + q * D;
    double* M = dLq + q * D;
    double* gA = M + q * q;
    double* mu = gA + q * q;
    double* dmu = mu + q;
    double* tS = dmu + q;
    double* dY = tS + S;
    double* scr = dY + kSampleChunk * q;
    __shared__ int s_status;
    __shared__ double s_red[4];
    __shared__ double s_lse;
    const int tid = threadIdx.x;
    const double sy = a.y_std, sy2 = a.y_std * a.y_std;
    if (tid == 0) s_status = (a.dev_err != nullptr && *a.dev_err != 0) ? BGB_DEVICE_TIMEOUT : 0;
    __syncthreads();
    if (s_status != 0) {
        if (tid == 0) {
            a.status[bidx] = s_status;
            a.value[bidx] = NAN;
        }
        return;
    }
    // (1) untransformed mean and covariance blocks
    for (int i = tid; i < q; i += blockDim.x) mu[i] = a.y_mean + sy * a.mu[bidx * q + i];
    for (int p = tid; p < q * q; p += blockDim.x) M[p] = sy2 * a.sig[bidx * q * q + p];
    __syncthreads();
    // (2)-(4) the q new rows [bl, br] of the Cholesky factor of the joint covariance
    //   cached root (joint == 0): bl = Sigma_qb Lb^-T, br = psd_safe_cholesky(Sigma_qq - bl bl^T)
    //   joint sampling: psd_safe_cholesky of the whole (r+q) x (r+q) matrix, blockwise:
    //   at jitter level t, bl = Sigma_qb L_t^-T with L_t = chol(Sigma_bb + j_t I), and
    //   br = chol(Sigma_qq + j_t I - bl bl^T); the first level where both succeed
    __shared__ int s_lv;
    const double* Lbi = a.Lb_inv;
    const int nlv = a.joint ? a.max_tries + 1 : 1;
    if (tid == 0) s_lv = -1;
    __syncthreads();
    for (int lv = 0; lv < nlv; ++lv) {
        if (a.joint) {
            Lbi = a.Lb_inv_lv + (int64_t)lv * r * r;
            if (r > 0 && isnan(Lbi[0])) continue;  // chol(Sigma_bb + j_t I) failed at this level
            if (lv > 0) {  // M holds the previous level's attempt
                for (int p = tid; p < q * q; p += blockDim.x) M[p] = sy2 * a.sig[bidx * q * q + p];
                __syncthreads();
            }
        }
        const double jit = (a.joint && lv > 0) ? a.jitter * pow(10.0, (double)(lv - 1)) : 0.0;
        // (2) bl = Sigma_qb Lb^-T  (Lq[:, :r]);  Lb_inv lower triangular
        for (int p = tid; p < q * r; p += blockDim.x) {
            int i = p / r, k = p % r;
            double s = 0.0;
            for (int kk = 0; kk <= k; ++kk) s += sy2 * a.sqb[(bidx * q + i) * r + kk] * Lbi[k * r + kk];
            Lq[i * D + k] = s;
        }
        __syncthreads();
        // (3) M = Sigma_qq (+ j_t I) - bl bl^T
        for (int p = tid; p < q * q; p += blockDim.x) {
            int i = p / q, j = p % q;
            double s = 0.0;
            for (int k = 0; k < r; ++k) s += Lq[i * D + k] * Lq[j * D + k];
            M[p] += (i == j ? jit : 0.0) - s;
        }
        __syncthreads();
        // (4) cached root: psd_safe_cholesky(M), plain then jitter j * 10^i (i < max_tries)
        // for this batch only; joint: the plain factorisation at this level
        if (tid == 0) {
            int status = 0;
            bool has_nan = false;
            for (int p = 0; p < q * q; ++p) has_nan |= isnan(M[p]);
            for (int p = 0; p < q * q; ++p) scr[p] = M[p];
            int info = has_nan ? 1 : chol_small(scr, q);
            if (info != 0) {
                if (has_nan) {
                    status = BGB_NAN;
                } else {
                    double jprev = 0.0;
                    status = BGB_NOT_PSD;
                    for (int t = 0; t < (a.joint ? 0 : a.max_tries); ++t) {
                        double jnew = a.jitter * pow(10.0, (double)t);
                        for (int i = 0; i < q; ++i) M[i * q + i] += jnew - jprev;
                        jprev = jnew;
                        for (int p = 0; p < q * q; ++p) scr[p] = M[p];
                        if (chol_small(scr, q) == 0) { status = 0; break; }
                    }
                }
            }
            for (int i = 0; i < q; ++i)
                for (int j = 0; j < q; ++j) Lq[i * D + r + j] = (j <= i) ? scr[i * q + j] : 0.0;
            s_status = status;
            if (status == 0) s_lv = lv;
        }
        __syncthreads();
        if (s_status != BGB_NOT_PSD) break;  // factorised, or NaN (no jitter helps)
    }
    if (a.joint && s_lv < 0 && s_status == 0) {  // every level's chol(Sigma_bb + j_t I) failed
        __syncthreads();
        if (tid == 0) s_status = BGB_NOT_PSD;
        __syncthreads();
    }
    if (a.joint && s_lv >= 0) Lbi = a.Lb_inv_lv + (int64_t)s_lv * r * r;
    const double* best_f = (a.joint == 2 && s_lv >= 0) ? a.best_f_lv + (int64_t)s_lv * S : a.best_f;
    if (s_status != 0) {
        if (tid == 0) {
            a.status[bidx] = s_status;
            a.value[bidx] = NAN;
        }
        if (backward) {
            for (int p = tid; p < q * q; p += blockDim.x) a.gqq[bidx * q * q + p] = 0.0;
            for (int p = tid; p < q * r; p += blockDim.x) a.gqb[bidx * q * r + p] = 0.0;
            for (int p = tid; p < q; p += blockDim.x) a.gmu[bidx * q + p] = 0.0;
        }
        return;
    }
    const bool qei = (a.acqf == BGB_ACQF_QEI);
    const double tau = a.tau_relu, taum = a.tau_max;
    // (5) forward over samples: t_s (per-sample reduced utility)
    int local_bad = 0;
    for (int s = tid; s < S; s += blockDim.x) {
        const double* z = a.Z + (int64_t)s * D;
        const double bf = qei ? a.best_f[0] : best_f[s];
        double li[kMaxQ];
        double Mx = -INFINITY;
        for (int i = 0; i < q; ++i) {
            double y = mu[i];
            for (int k = 0; k < r + i + 1; ++k) y += Lq[i * D + k] * z[k];
            if (!isfinite(y)) local_bad = 1;
            if (qei) {
                li[i] = fmax(y - bf, 0.0);
            } else {
                li[i] = log_fatplus(y - bf, tau);
            }
            Mx = fmax(Mx, li[i]);
        }
        double t;
        if (qei) {
            t = Mx;
        } else if (isinf(Mx)) {
            t = Mx;
        } else {
            double P = 0.0;
            for (int i = 0; i < q; ++i) P += pareto2((Mx - li[i]) / taum);
            t = Mx + taum * log(P);
        }
        tS[s] = t;
    }
    if (__syncthreads_or(local_bad)) {
        if (tid == 0) {
            a.status[bidx] = BGB_NAN;
            a.value[bidx] = NAN;
        }
        if (backward) {
            for (int p = tid; p < q * q; p += blockDim.x) a.gqq[bidx * q * q + p] = 0.0;
            for (int p = tid; p < q * r; p += blockDim.x) a.gqb[bidx * q * r + p] = 0.0;
            for (int p = tid; p < q; p += blockDim.x) a.gmu[bidx * q + p] = 0.0;
        }
        return;
    }
    // (6) sample reduction (float64): qEI mean, qLogNEI logmeanexp with inf handling
    const int lane = tid % 32, warp = tid / 32;
    double mx = -INFINITY;
    for (int s = tid; s < S; s += blockDim.x) mx = fmax(mx, tS[s]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_red[warp] = mx;
    __syncthreads();
    mx = fmax(fmax(s_red[0], s_red[1]), fmax(s_red[2], s_red[3]));
    __syncthreads();
    double acc = 0.0;
    for (int s = tid; s < S; s += blockDim.x) {
        if (qei) acc += tS[s];
        else if (!isinf(mx)) acc += exp(tS[s] - mx);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_red[warp] = acc;
    __syncthreads();
    if (tid == 0) {
        double tot = (s_red[0] + s_red[1]) + (s_red[2] + s_red[3]);
        double v, lse;
        if (qei) {
            v = tot / S;
            lse = 0.0;
        } else if (isinf(mx)) {
            v = mx;  // sum of the infinite maxima (same sign) minus log S
            lse = mx;
        } else {
            lse = mx + log(tot);
            v = lse - log((double)S);
        }
        a.value[bidx] = v;
        a.status[bidx] = 0;
        s_lse = lse;
    }
    if (!backward) return;
    for (int p = tid; p < q * D; p += blockDim.x) dLq[p] = 0.0;
    for (int p = tid; p < q; p += blockDim.x) dmu[p] = 0.0;
    __syncthreads();
    const double lse = s_lse;
    // (7) reverse through the sample reduction and the sample step, SC samples at a time
    for (int s0 = 0; s0 < S; s0 += kSampleChunk) {
        const int sc = min(kSampleChunk, S - s0);
        for (int ls = tid; ls < sc; ls += blockDim.x) {
            const int s = s0 + ls;
            const double* z = a.Z + (int64_t)s * D;
            const double bf = qei ? a.best_f[0] : best_f[s];
            double u[kMaxQ], li[kMaxQ], g[kMaxQ];
            double Mx = -INFINITY;
            for (int i = 0; i < q; ++i) {
                double y = mu[i];
                for (int k = 0; k < r + i + 1; ++k) y += Lq[i * D + k] * z[k];
                u[i] = y - bf;
                li[i] = qei ? fmax(u[i], 0.0) : log_fatplus(u[i], tau);
                Mx = fmax(Mx, li[i]);
            }
            int nt = 0;
            for (int i = 0; i < q; ++i) nt += (li[i] == Mx);
            if (qei) {
                const double w = 1.0 / S / nt;
                for (int i = 0; i < q; ++i) g[i] = (li[i] == Mx && u[i] >= 0.0) ? w : 0.0;
            } else {
                const double ws = isinf(mx) ? (tS[s] == mx ? 1.0 : 0.0) : exp(tS[s] - lse);
                if (isinf(Mx)) {
                    for (int i = 0; i < q; ++i) g[i] = (li[i] == Mx) ? ws : 0.0;
                } else {
                    double P = 0.0, Pd = 0.0;
                    for (int i = 0; i < q; ++i) {
                        double x = (Mx - li[i]) / taum;
                        P += pareto2(x);
                        Pd += dpareto2(x);
                    }
                    const double top = (1.0 + Pd / P) / nt;
                    for (int i = 0; i < q; ++i) {
                        double x = (Mx - li[i]) / taum;
                        double dt = -dpareto2(x) / P + (li[i] == Mx ? top : 0.0);
                        g[i] = ws * dt * dlog_fatplus(u[i], tau);
                    }
                }
            }
            for (int i = 0; i < q; ++i) dY[ls * q + i] = g[i];
        }
        __syncthreads();
        for (int p = tid; p < q * D; p += blockDim.x) {
            const int i = p / D, k = p % D;
            if (k >= r + i + 1) continue;  // upper part of br stays zero
            double s = 0.0;
            for (int ls = 0; ls < sc; ++ls) s += dY[ls * q + i] * a.Z[(int64_t)(s0 + ls) * D + k];
            dLq[p] += s;
        }
        for (int i = tid; i < q; i += blockDim.x) {
            double s = 0.0;
            for (int ls = 0; ls < sc; ++ls) s += dY[ls * q + i];
            dmu[i] += s;
        }
        __syncthreads();
    }
    // (8) reverse through br = chol(M): gA = L^-T Phi(L^T dL) L^-1 (symmetric)
    if (tid == 0) {
        // X = tril(L^T dL)   (L = br, dL = d br, both lower)
        for (int i = 0; i < q; ++i)
            for (int j = 0; j < q; ++j) {
                double s = 0.0;
                if (j <= i)
                    for (int k = i; k < q; ++k) s += Lq[k * D + r + i] * dLq[k * D + r + j];
                scr[i * q + j] = s;
            }
        // Phi = 0.5 * (X + tril(X, -1)^T)
        for (int i = 0; i < q; ++i)
            for (int j = 0; j < q; ++j) {
                double v;
                if (i == j) v = 0.5 * scr[i * q + i];
                else if (j < i) v = 0.5 * scr[i * q + j];
                else v = 0.5 * scr[j * q + i];
                gA[i * q + j] = v;
            }
        // gA <- L^-T gA  (solve L^T Y = gA, upper triangular, column by column)
        for (int c = 0; c < q; ++c)
            for (int i = q - 1; i >= 0; --i) {
                double s = gA[i * q + c];
                for (int k = i + 1; k < q; ++k) s -= Lq[k * D + r + i] * gA[k * q + c];
                gA[i * q + c] = s / Lq[i * D + r + i];
            }
        // gA <- gA L^-1  (solve Y L = gA, row by row)
        for (int row = 0; row < q; ++row)
            for (int j = q - 1; j >= 0; --j) {
                double s = gA[row * q + j];
                for (int k = j + 1; k < q; ++k) s -= gA[row * q + k] * Lq[k * D + r + j];
                gA[row * q + j] = s / Lq[j * D + r + j];
            }
    }
    __syncthreads();
    // (9) d bl += -2 gA bl;  dSigma_qb = d bl * Lb^-1;  write seeds in standardised units
    for (int p = tid; p < q * r; p += blockDim.x) {
        const int i = p / r, k = p % r;
        double s = dLq[i * D + k];
        for (int j = 0; j < q; ++j) s -= 2.0 * gA[i * q + j] * Lq[j * D + k];
        scr[p] = s;  // reuse: q*r <= scratch when r <= q; else spill to dLq block below
    }
    __syncthreads();
    for (int p = tid; p < q * r; p += blockDim.x) dLq[(p / r) * D + (p % r)] = scr[p];
    __syncthreads();
    for (int p = tid; p < q * r; p += blockDim.x) {
        const int i = p / r, kp = p % r;
        double s = 0.0;
        for (int k = kp; k < r; ++k) s += dLq[i * D + k] * Lbi[k * r + kp];
        a.gqb[(bidx * q + i) * r + kp] = sy2 * s;
    }
    for (int p = tid; p < q * q; p += blockDim.x) a.gqq[bidx * q * q + p] = sy2 * gA[p];
    for (int i = tid; i < q; i += blockDim.x) a.gmu[bidx * q + i] = sy * dmu[i];
}
#endif  // BGB_QB_STEP

// ---------------------------------------------------------------- batch_step (mixed)
// Per-t-batch step of the mixed path. float64 for the q x q algebra: the
// covariance blocks, bl = Sigma_qb Lb^-T, M = Sigma_qq - bl bl^T, its jittered
// Cholesky and the Cholesky adjoint. float32 for the per-sample work: the
// improvement
//   u = (mu - best_f) + [bl, br] z
// is formed from exact float pairs (hi, lo) of mu and best_f, the leading
// difference mu_hi - bf_hi by an error-free two-sum, so the cancellation near
// the incumbent is exact and only the zero-mean term [bl, br] z carries float32
// rounding. The reverse pass recomputes each sample's forward rather than
// storing it, and accumulates d[bl, br] = sum_s dY_s z_s^T per chunk of samples
// (float32 within a chunk, float64 across chunks).
constexpr int kBsThreads = 64;
constexpr int kBsThreadsFew = 256;
constexpr int kDyLd = kSampleChunk + 1;  // row stride of the reverse-pass dY tile

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// u_i (i < q) of one sample; zs: the sample's D base-sample coordinates; LfT:
// [bl, br] k-major with QMAX entries per k (zero above the diagonal of br and
// for i >= q), so pairs of points take one packed FMA per coordinate
template <int QMAX>
__device__ __forceinline__ void sample_u(const float* __restrict__ LfT, const float* __restrict__ zs,
                                         int q, int D, const float* muh, const float* mul, float bh,
                                         float bl, float* u) {
    float2 y2[QMAX / 2];
#pragma unroll
    for (int j = 0; j < QMAX / 2; ++j) y2[j] = make_float2(0.f, 0.f);
    for (int k = 0; k < D; ++k) {
        const float zk = zs[k];
        const float2 z2 = make_float2(zk, zk);
        const float2* L2 = reinterpret_cast<const float2*>(LfT + k * QMAX);
#pragma unroll
        for (int j = 0; j < QMAX / 2; ++j) y2[j] = __ffma2_rn(L2[j], z2, y2[j]);
    }
#pragma unroll
    for (int i = 0; i < QMAX; ++i) {
        float dh, e;
        two_sum_f(muh[i], -bh, dh, e);
        const float y = (i % 2 == 0) ? y2[i / 2].x : y2[i / 2].y;
        u[i] = (i < q) ? dh + ((e + (mul[i] - bl)) + y) : 0.f;
    }
}

// psd_safe_cholesky of the q x q matrix M (float64, row-major) into scr: plain,
// then jitter j * 10^t (t < max_tries) added to M's diagonal. Returns 0,
// BGB_NOT_PSD or BGB_NAN. Run by the 32 lanes of one warp: each column step
// computes its pivot in every lane (one reciprocal square root per column: the
// pivot is v rsqrt(v)) and lane i updates row i, which spreads the float64 work
// over the warp.
__device__ int psd_chol_warp(double* M, double* scr, int q, int max_tries, double jitter, int lane) {
    bool has_nan = false;
    for (int p = lane; p < q * q; p += 32) has_nan |= isnan(M[p]);
    if (__any_sync(0xffffffffu, has_nan)) return BGB_NAN;
    double jprev = 0.0;
    for (int t = -1; t < max_tries; ++t) {
        if (t >= 0) {
            const double jnew = jitter * pow(10.0, (double)t);
            if (lane < q) M[lane * q + lane] += jnew - jprev;
            jprev = jnew;
            __syncwarp();
        }
        for (int p = lane; p < q * q; p += 32) scr[p] = M[p];
        __syncwarp();
        bool ok = true;
        for (int j = 0; j < q; ++j) {
            double v = scr[j * q + j];
            for (int k = 0; k < j; ++k) v -= scr[j * q + k] * scr[j * q + k];
            if (!(v > 0.0)) { ok = false; break; }
            const double rj = rsqrt(v), djj = v * rj;  // one reciprocal square root
            __syncwarp();
            if (lane == j) scr[j * q + j] = djj;
            if (lane > j && lane < q) {
                double acc = scr[lane * q + j];
                for (int k = 0; k < j; ++k) acc -= scr[lane * q + k] * scr[j * q + k];
                scr[lane * q + j] = acc * rj;
                scr[j * q + lane] = 0.0;
            }
            __syncwarp();
        }
        __syncwarp();
        if (ok) return 0;
    }
    return BGB_NOT_PSD;
}

template <int QMAX, int NT>
__device__ __forceinline__ void batch_step_f32_body(const QBatchArgs& a, int backward,
                                                    int64_t bidx_) {
    extern __shared__ double smd[];
    constexpr int NW = NT / 32;
    const int q = a.q, r = a.r, S = a.S, D = r + q;
    const int64_t bidx = bidx_;
    const int tid = threadIdx.x, lane = tid % 32, warp = tid / 32;
    double* M = smd;                 // q x q
    double* Lq = M + q * q;          // q x D: [bl, br]
    double* dLq = Lq + q * D;        // q x D
    double* gA = dLq + q * D;        // q x q
    double* scr = gA + q * q;        // max(q*q, q*r)
    float* Lf = reinterpret_cast<float*>(scr + (q * q > q * r ? q * q : q * r));  // D x QMAX (k-major)
    float* tS = Lf + D * QMAX;       // S
    float* dY = tS + S;              // q x kDyLd
    __shared__ float s_muh[QMAX], s_mul[QMAX];
    __shared__ double s_dmu[QMAX], s_rd[QMAX];
    __shared__ int s_status;
    __shared__ double s_red[NW];
    __shared__ float s_redf[NW];
    __shared__ double s_lse;
    const double sy = a.y_std, sy2 = sy * sy;
    auto fail = [&](int status) {
        if (tid == 0) {
            a.status[bidx] = status;
            a.value[bidx] = NAN;
        }
        if (backward && status != BGB_DEVICE_TIMEOUT) {
            for (int p = tid; p < q * q; p += NT) a.gqq[bidx * q * q + p] = 0.0;
            for (int p = tid; p < q * r; p += NT) a.gqb[bidx * q * r + p] = 0.0;
            for (int p = tid; p < q; p += NT) a.gmu[bidx * q + p] = 0.0;
        }
    };
    if (tid == 0) s_status = (a.dev_err != nullptr && *a.dev_err != 0) ? BGB_DEVICE_TIMEOUT : 0;
    __syncthreads();
    if (s_status != 0) {
        fail(s_status);
        return;
    }
    // (1) untransformed mean as a float pair, covariance blocks
    for (int i = tid; i < QMAX; i += NT) {
        const double mu = (i < q) ? a.y_mean + sy * a.mu[bidx * q + i] : 0.0;
        const float h = (float)mu;
        s_muh[i] = h;
        s_mul[i] = (float)(mu - (double)h);
    }
    for (int p = tid; p < q * q; p += NT) M[p] = sy2 * a.sig[bidx * q * q + p];
    __syncthreads();
    // (2)-(4) the q new rows [bl, br] of the Cholesky factor of the joint covariance:
    // cached root (joint == 0) or joint sampling level by level, as in the float64 step
    __shared__ int s_lv;
    const double* Lbi = a.Lb_inv;
    const int nlv = a.joint ? a.max_tries + 1 : 1;
    if (tid == 0) s_lv = -1;
    __syncthreads();
    for (int lv = 0; lv < nlv; ++lv) {
        if (a.joint) {
            Lbi = a.Lb_inv_lv + (int64_t)lv * r * r;
            if (r > 0 && isnan(Lbi[0])) continue;  // chol(Sigma_bb + j_t I) failed at this level
            if (lv > 0) {  // M holds the previous level's attempt
                for (int p = tid; p < q * q; p += NT) M[p] = sy2 * a.sig[bidx * q * q + p];
                __syncthreads();
            }
        }
        const double jit = (a.joint && lv > 0) ? a.jitter * pow(10.0, (double)(lv - 1)) : 0.0;
        // (2) bl = Sigma_qb Lb^-T (Lb^-1 lower triangular)
        for (int p = tid; p < q * r; p += NT) {
            const int i = p / r, k = p % r;
            double acc = 0.0;
            for (int kk = 0; kk <= k; ++kk) acc += sy2 * a.sqb[(bidx * q + i) * r + kk] * Lbi[k * r + kk];
            Lq[i * D + k] = acc;
        }
        __syncthreads();
        // (3) M = Sigma_qq (+ j_t I) - bl bl^T
        for (int p = tid; p < q * q; p += NT) {
            const int i = p / q, j = p % q;
            double acc = 0.0;
            for (int k = 0; k < r; ++k) acc += Lq[i * D + k] * Lq[j * D + k];
            M[p] += (i == j ? jit : 0.0) - acc;
        }
        __syncthreads();
        // (4) br = psd_safe_cholesky(M) for this t-batch (warp 0); joint: plain at this level
        if (warp == 0) {
            const int st = psd_chol_warp(M, scr, q, a.joint ? 0 : a.max_tries, a.jitter, lane);
            for (int p = lane; p < q * q; p += 32) {
                const int i = p / q, j = p % q;
                Lq[i * D + r + j] = (j <= i) ? scr[p] : 0.0;
            }
            if (lane == 0) {
                s_status = st;
                if (st == 0) s_lv = lv;
            }
        }
        __syncthreads();
        if (s_status != BGB_NOT_PSD) break;  // factorised, or NaN (no jitter helps)
    }
    if (a.joint && s_lv < 0 && s_status == 0) {  // every level's chol(Sigma_bb + j_t I) failed
        __syncthreads();
        if (tid == 0) s_status = BGB_NOT_PSD;
        __syncthreads();
    }
    if (s_status != 0) {
        fail(s_status);
        return;
    }
    if (a.joint) Lbi = a.Lb_inv_lv + (int64_t)s_lv * r * r;
    for (int p = tid; p < D * QMAX; p += NT) {
        const int k = p / QMAX, i = p % QMAX;
        Lf[p] = (i < q) ? (float)Lq[i * D + k] : 0.f;
    }
    __syncthreads();
    const bool qei = (a.acqf == BGB_ACQF_QEI);
    const float inv_tau = a.inv_tau_relu_f;
    const float log_tau = a.log_tau_relu_f;
    const float taum = (float)a.tau_max, inv_taum = a.inv_tau_max_f;
    const float* __restrict__ z32 = a.z32;
    // best_f per sample as float pairs: per jitter level for cache_root=False
    const float* __restrict__ bf32 = a.joint == 2 ? a.bf32 + 2 * (int64_t)s_lv * S : a.bf32;
    // (5) forward: t_s per sample
    int local_bad = 0;
    for (int s = tid; s < S; s += NT) {
        float u[QMAX];
        sample_u<QMAX>(Lf, z32 + (int64_t)s * D, q, D, s_muh, s_mul, bf32[2 * s], bf32[2 * s + 1], u);
        float Mx = -INFINITY, li[QMAX];
#pragma unroll
        for (int i = 0; i < QMAX; ++i) {
            if (i >= q) { li[i] = -INFINITY; continue; }
            if (!isfinite(u[i])) local_bad = 1;
            if (qei) {
                li[i] = fmaxf(u[i], 0.f);
            } else {
                float dl;
                log_fatplus_f(u[i] * inv_tau, log_tau, inv_tau, li[i], dl);
            }
            Mx = fmaxf(Mx, li[i]);
        }
        float t = Mx;
        if (!qei && !isinf(Mx)) {
            float P = 0.f;
#pragma unroll
            for (int i = 0; i < QMAX; ++i)
                if (i < q) P += pareto2_f((Mx - li[i]) * inv_taum);
            t = Mx + taum * __logf(P);
        }
        tS[s] = t;
    }
    if (__syncthreads_or(local_bad)) {
        fail(BGB_NAN);
        return;
    }
    // (6) reduction over samples: qEI mean, qLogNEI log-mean-exp (inf handling as the reference)
    float mx = -INFINITY;
    for (int s = tid; s < S; s += NT) mx = fmaxf(mx, tS[s]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_redf[warp] = mx;
    __syncthreads();
    mx = s_redf[0];
#pragma unroll
    for (int w = 1; w < NW; ++w) mx = fmaxf(mx, s_redf[w]);
    // per-thread partial sums in float64, so that the value does not depend on
    // how the samples are dealt to the threads beyond float64 rounding
    double acc = 0.0;
    for (int s = tid; s < S; s += NT) {
        if (qei) acc += (double)tS[s];
        else if (!isinf(mx)) acc += (double)__expf(tS[s] - mx);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_red[warp] = acc;
    __syncthreads();
    if (tid == 0) {
        double tot = 0.0;
        for (int w = 0; w < NW; ++w) tot += s_red[w];
        double v, lse;
        if (qei) {
            v = tot / S;
            lse = 0.0;
        } else if (isinf(mx)) {
            v = mx;
            lse = mx;
        } else {
            lse = (double)mx + log(tot);
            v = lse - a.log_S;
        }
        a.value[bidx] = v;
        a.status[bidx] = 0;
        s_lse = lse;
    }
    if (!backward) return;
    for (int p = tid; p < q * D; p += NT) dLq[p] = 0.0;
    for (int i = tid; i < QMAX; i += NT) s_dmu[i] = 0.0;
    __syncthreads();
    const float lse_f = (float)s_lse;
    const bool inf_mx = isinf(mx);
    // (7) reverse through the sample reduction and the sample step, a chunk of samples at a time
    for (int s0 = 0; s0 < S; s0 += kSampleChunk) {
        const int sc = min(kSampleChunk, S - s0);
        for (int ls = tid; ls < sc; ls += NT) {
            const int s = s0 + ls;
            float u[QMAX], li[QMAX], dli[QMAX], g[QMAX];
            sample_u<QMAX>(Lf, z32 + (int64_t)s * D, q, D, s_muh, s_mul, bf32[2 * s], bf32[2 * s + 1], u);
            float Mx = -INFINITY;
#pragma unroll
            for (int i = 0; i < QMAX; ++i) {
                if (i >= q) { li[i] = -INFINITY; dli[i] = 0.f; continue; }
                if (qei) li[i] = fmaxf(u[i], 0.f);
                else log_fatplus_f(u[i] * inv_tau, log_tau, inv_tau, li[i], dli[i]);
                Mx = fmaxf(Mx, li[i]);
            }
            int nt = 0;
#pragma unroll
            for (int i = 0; i < QMAX; ++i) nt += (i < q && li[i] == Mx);
            if (qei) {
                const float w = 1.f / ((float)S * (float)nt);
#pragma unroll
                for (int i = 0; i < QMAX; ++i) g[i] = (i < q && li[i] == Mx && u[i] >= 0.f) ? w : 0.f;
            } else {
                float t = Mx, P = 0.f, Pd = 0.f;
                if (!isinf(Mx)) {
#pragma unroll
                    for (int i = 0; i < QMAX; ++i) {
                        if (i >= q) continue;
                        const float x = (Mx - li[i]) * inv_taum;
                        P += pareto2_f(x);
                        Pd += dpareto2_f(x);
                    }
                    t = Mx + taum * __logf(P);
                }
                const float ws = inf_mx ? (t == mx ? 1.f : 0.f) : __expf(t - lse_f);
                if (isinf(Mx)) {
#pragma unroll
                    for (int i = 0; i < QMAX; ++i) g[i] = (i < q && li[i] == Mx) ? ws : 0.f;
                } else {
                    const float top = (1.f + Pd / P) / (float)nt;
#pragma unroll
                    for (int i = 0; i < QMAX; ++i) {
                        if (i >= q) { g[i] = 0.f; continue; }
                        const float x = (Mx - li[i]) * inv_taum;
                        const float dt = -dpareto2_f(x) / P + (li[i] == Mx ? top : 0.f);
                        g[i] = ws * dt * dli[i];
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < QMAX; ++i)
                if (i < q) dY[i * kDyLd + ls] = g[i];  // point-major, padded: no bank conflicts
        }
        __syncthreads();
        for (int p = tid; p < q * D; p += NT) {
            const int i = p / D, k = p % D;
            if (k >= r + i + 1) continue;  // the upper part of br stays zero
            float cs = 0.f;
            const float* dyi = dY + i * kDyLd;
            for (int ls = 0; ls < sc; ++ls) cs = fmaf(dyi[ls], z32[(int64_t)(s0 + ls) * D + k], cs);
            dLq[p] += (double)cs;
        }
        for (int i = tid; i < q; i += NT) {
            float cs = 0.f;
            const float* dyi = dY + i * kDyLd;
            for (int ls = 0; ls < sc; ++ls) cs += dyi[ls];
            s_dmu[i] += (double)cs;
        }
        __syncthreads();
    }
    // (8) reverse through br = chol(M): gA = L^-T Phi(L^T dL) L^-1 (symmetric),
    // float64, warp 0: entries of L^T dL over the lanes, then one column (first
    // solve) or one row (second solve) per lane.
    if (warp == 0) {
        if (lane < q) s_rd[lane] = 1.0 / Lq[lane * D + r + lane];
        for (int p = lane; p < q * q; p += 32) {
            const int i = p / q, j = p % q;
            double acc2 = 0.0;
            if (j <= i)
                for (int k = i; k < q; ++k) acc2 += Lq[k * D + r + i] * dLq[k * D + r + j];
            scr[p] = acc2;
        }
        __syncwarp();
        for (int p = lane; p < q * q; p += 32) {
            const int i = p / q, j = p % q;
            gA[p] = 0.5 * (j <= i ? scr[i * q + j] : scr[j * q + i]);
        }
        __syncwarp();
        if (lane < q) {
            const int c = lane;
            for (int i = q - 1; i >= 0; --i) {
                double acc2 = gA[i * q + c];
                for (int k = i + 1; k < q; ++k) acc2 -= Lq[k * D + r + i] * gA[k * q + c];
                gA[i * q + c] = acc2 * s_rd[i];
            }
        }
        __syncwarp();
        if (lane < q) {
            const int row = lane;
            for (int j = q - 1; j >= 0; --j) {
                double acc2 = gA[row * q + j];
                for (int k = j + 1; k < q; ++k) acc2 -= gA[row * q + k] * Lq[k * D + r + j];
                gA[row * q + j] = acc2 * s_rd[j];
            }
        }
    }
    __syncthreads();
    // (9) d bl += -2 gA bl;  dSigma_qb = d bl Lb^-1;  seeds in standardised units
    for (int p = tid; p < q * r; p += NT) {
        const int i = p / r, k = p % r;
        double acc2 = dLq[i * D + k];
        for (int j = 0; j < q; ++j) acc2 -= 2.0 * gA[i * q + j] * Lq[j * D + k];
        scr[p] = acc2;
    }
    __syncthreads();
    for (int p = tid; p < q * r; p += NT) dLq[(p / r) * D + (p % r)] = scr[p];
    __syncthreads();
    for (int p = tid; p < q * r; p += NT) {
        const int i = p / r, kp = p % r;
        double acc2 = 0.0;
        for (int k = kp; k < r; ++k) acc2 += dLq[i * D + k] * Lbi[k * r + kp];
        a.gqb[(bidx * q + i) * r + kp] = sy2 * acc2;
    }
    for (int p = tid; p < q * q; p += NT) a.gqq[bidx * q * q + p] = sy2 * gA[p];
    for (int i = tid; i < q; i += NT) a.gmu[bidx * q + i] = sy * s_dmu[i];
    if (a.hmul == nullptr) return;
    // power-of-two row scales of H = gmu beta^T - 2 Gqq V - Gqb Vb for its float16
    // split, from |H[i,c]| <= |gmu_i| max|beta| + sqrt(outputscale) (sum_j 2|Gqq_ij| +
    // sum_k |Gqb_ik|) (rows of V and Vb have 2-norm <= sqrt(outputscale))
    __syncthreads();
    for (int i = tid; i < q; i += NT) {
        double sv = 0.0;
        for (int j = 0; j < q; ++j) sv += 2.0 * fabs(a.gqq[(bidx * q + i) * q + j]);
        for (int k = 0; k < r; ++k) sv += fabs(a.gqb[(bidx * q + i) * r + k]);
        const double bound = fabs(a.gmu[bidx * q + i]) * a.beta_absmax + a.sqrt_outputscale * sv;
        float sc = 1.f;
        if (bound > 0.0 && !isinf(bound)) {
            int e;
            frexp(bound, &e);
            sc = ldexpf(1.f, 14 - e);
        }
        a.hmul[bidx * q + i] = 1.f / sc;
    }
}

// NT threads per t-batch: kBsThreads when the t-batches fill the GPU, kBsThreadsFew
// when they are few and each has many samples (the sample loops and the
// per-sample reverse sums then spread over more threads; the q x q phases stay
// on one warp).
template <int QMAX, int NT>
__global__ void __launch_bounds__(NT)
    batch_step_f32_kernel(const __grid_constant__ QBatchArgs a, int backward) {
    batch_step_f32_body<QMAX, NT>(a, backward, blockIdx.x);
}

template <int QMAX>
__global__ void __launch_bounds__(kBsThreads) batch_step_f32_group_kernel(const GroupTab t) {
    const int m = group_model(t);
    const BstepG& g = static_cast<const BstepG*>(t.args)[m];
    batch_step_f32_body<QMAX, kBsThreads>(g.a, g.backward, blockIdx.x - t.off[m]);
}

#if defined(BGB_QB_STEP)
// Z in float32, and nbf best_f values (S, or S per jitter level) as float pairs.
__global__ void prep_samples_kernel(const double* __restrict__ Z, int64_t nz,
                                    const double* __restrict__ best_f, int64_t nbf, int qei,
                                    float* __restrict__ z32, float* __restrict__ bf32) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < nz) z32[idx] = (float)Z[idx];
    if (idx < nbf) {
        const double bf = best_f[qei ? 0 : idx];
        const float h = (float)bf;
        bf32[2 * idx] = h;
        bf32[2 * idx + 1] = (float)(bf - (double)h);
    }
}
#endif  // BGB_QB_STEP

// ---------------------------------------------------------------- mix_rows
// H[row i of t-batch] = gmu_i beta - 2 sum_j Gqq[i,j] V[j,:] - sum_k Gqb[i,k] Vb[k,:]
// (d value / d V through mu = V beta, Sigma_qq and Sigma_qb). Each thread owns
// E consecutive columns of one t-batch (one 16-byte vector per row when the
// layout allows, else E = 1), so every seed read from shared memory feeds E
// columns; QM >= q bounds the register arrays.
// H16 set (float32 only): H is written as the float16 split of s_i H[i,:] for
// the tensor-core adjoint GEMM, with 1 / s_i in a.hmul: the power of two that
// the batch step derived from the bound
//   |H[i,c]| <= |gmu_i| max|beta| + sqrt(outputscale) (sum_j 2|Gqq[i,j]| + sum_k |Gqb[i,k]|)
// (every row of V and Vb has 2-norm <= sqrt(outputscale) since V V^T <= K(X,X)).
template <typename T, int QM, int E>
__device__ __forceinline__ void mix_rows_body(const QBatchArgs& a, const T* __restrict__ V,
                                              int64_t ldv, const T* __restrict__ Vb,
                                              const T* __restrict__ beta, T* __restrict__ H,
                                              __half* __restrict__ H16, __half* __restrict__ H16_lo,
                                              int64_t ldh, int64_t bx, int64_t by, int64_t gx) {
    extern __shared__ __align__(16) unsigned char gsraw[];  // q*q + q*r + q seeds (as T), q scales
    T* gq = reinterpret_cast<T*>(gsraw);
    const int q = a.q, r = a.r;
    const int64_t n = a.n, bidx = by, rbase = bidx * q;
    T* gqb = gq + q * q;
    T* gm = gqb + q * r;
    float* hs = reinterpret_cast<float*>(gm + q);
    for (int p = threadIdx.x; p < q * q; p += blockDim.x) gq[p] = (T)(-2.0 * a.gqq[bidx * q * q + p]);
    for (int p = threadIdx.x; p < q * r; p += blockDim.x) gqb[p] = (T)(-a.gqb[bidx * q * r + p]);
    for (int p = threadIdx.x; p < q; p += blockDim.x) gm[p] = (T)a.gmu[bidx * q + p];
    __syncthreads();
    if (H16 != nullptr) {  // row scales written by the batch step (a.hmul = 1 / scale)
        for (int i = threadIdx.x; i < q; i += blockDim.x) hs[i] = 1.f / a.hmul[rbase + i];
        __syncthreads();
    }
    using VT = typename Vec16<T>::type;
    // column groups of blockDim.x * E, strided over grid.x
    for (int64_t cg = bx * blockDim.x * E; cg < n; cg += gx * blockDim.x * E) {
    const int64_t c0 = cg + (int64_t)threadIdx.x * E;
    if (c0 >= n) continue;
    T v[QM][E], bc[E];
#pragma unroll
    for (int j = 0; j < QM; ++j) {
        if constexpr (E > 1) {
            VT w;
            if (j < q) w = *reinterpret_cast<const VT*>(V + (rbase + j) * ldv + c0);
#pragma unroll
            for (int e = 0; e < E; ++e) v[j][e] = (j < q) ? Vec16<T>::at(w, e) : T(0);
        } else {
            v[j][0] = (j < q) ? V[(rbase + j) * ldv + c0] : T(0);
        }
    }
    if constexpr (E > 1) {
        const VT w = *reinterpret_cast<const VT*>(beta + c0);
#pragma unroll
        for (int e = 0; e < E; ++e) bc[e] = Vec16<T>::at(w, e);
    } else {
        bc[0] = beta[c0];
    }
    // one output row at a time (the Vb rows are re-read from L1 per row)
    auto row = [&](int i) {
        T h[E];
        const T gmi = gm[i];
#pragma unroll
        for (int e = 0; e < E; ++e) h[e] = gmi * bc[e];
#pragma unroll
        for (int j = 0; j < QM; ++j) {
            if (j < q) {
                const T gij = gq[i * q + j];
#pragma unroll
                for (int e = 0; e < E; ++e) h[e] = fma(gij, v[j][e], h[e]);
            }
        }
        for (int k = 0; k < r; ++k) {
            const T gik = gqb[i * r + k];
            if constexpr (E > 1) {
                const VT w = *reinterpret_cast<const VT*>(Vb + (int64_t)k * n + c0);
#pragma unroll
                for (int e = 0; e < E; ++e) h[e] = fma(gik, Vec16<T>::at(w, e), h[e]);
            } else {
                h[0] = fma(gik, Vb[(int64_t)k * n + c0], h[0]);
            }
        }
        const int64_t off = (rbase + i) * ldh + c0;
        if (H16 != nullptr) {
            __half hh[E], ll[E];
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const float w = (float)h[e] * hs[i];
                hh[e] = __float2half_rn(w);
                ll[e] = __float2half_rn(w - __half2float(hh[e]));
            }
            if constexpr (E == 4) {
                *reinterpret_cast<uint2*>(H16 + off) = *reinterpret_cast<const uint2*>(hh);
                *reinterpret_cast<uint2*>(H16_lo + off) = *reinterpret_cast<const uint2*>(ll);
            } else {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    H16[off + e] = hh[e];
                    H16_lo[off + e] = ll[e];
                }
            }
            return;
        }
        if constexpr (E > 1) {
            VT o;
            T* po = reinterpret_cast<T*>(&o);
#pragma unroll
            for (int e = 0; e < E; ++e) po[e] = h[e];
            *reinterpret_cast<VT*>(H + off) = o;
        } else {
            H[off] = h[0];
        }
    };
    if constexpr (QM <= 8) {
#pragma unroll
        for (int i = 0; i < QM; ++i) {
            if (i >= q) break;
            row(i);
        }
    } else {
        // rolled: a fully unrolled QM x QM body beyond q = 8 gains nothing and
        // is slow to compile
#pragma unroll 1
        for (int i = 0; i < q; ++i) row(i);
    }
    }
}

template <typename T, int QM, int E>
__global__ void __launch_bounds__(256, 3)
    mix_rows_kernel(const __grid_constant__ QBatchArgs a, const T* __restrict__ V, int64_t ldv,
                    const T* __restrict__ Vb, const T* __restrict__ beta, T* __restrict__ H,
                    __half* __restrict__ H16, __half* __restrict__ H16_lo, int64_t ldh) {
    mix_rows_body<T, QM, E>(a, V, ldv, Vb, beta, H, H16, H16_lo, ldh, blockIdx.x, blockIdx.y,
                            gridDim.x);
}

// grouped: model m's CTAs cover its (column group, t-batch) grid row-major in t-batches
template <typename T, int QM, int E>
__global__ void __launch_bounds__(256, 3) mix_rows_group_kernel(const GroupTab t) {
    const int m = group_model(t);
    const MixG<T>& g = static_cast<const MixG<T>*>(t.args)[m];
    const int64_t lb = (int64_t)blockIdx.x - t.off[m];
    mix_rows_body<T, QM, E>(g.a, g.V, g.ldv, g.Vb, g.beta, g.H, g.H16, g.H16_lo, g.ldh,
                            lb % g.gx, lb / g.gx, g.gx);
}

// ---------------------------------------------------------------- adjoint
// d value / d X through K(X, Xt): one thread per row of X, kAdjRows rows per CTA.
// The training points are split into grid.y slabs, since the rows alone give
// too few threads to hide latency. Per chunk of kAdjChunk points the CTA stages
// the points' scaled coordinates point-major (16-byte broadcast reads); the
// float32 form streams each thread's row of D from global memory, the float64
// form stages the D tile of its rows. Each thread sweeps the chunk with its
// row's coordinates and gradient accumulator in registers:
//   g += D[i,c] kappa'(r2_ic) (z_i - zt_c),   r2_ic = |z_i - zt_c|^2.
// One slab: the CTA finishes its rows (adjoint_finish_row). Several: each slab
// writes its partial g to part[slab][k][row] and adjoint_finalize_kernel adds
// the slabs in float64 and finishes the rows.
constexpr int kAdjRows = 128;
constexpr int kAdjChunk = 64;

// K(X, X) and K(X, Xb) terms of the gradient, then the chain rule through the
// scaled coordinates; writes grad[row, :]. Arithmetic in T: float64 for the
// float64 path; float32 for the mixed one, whose coordinates come scaled from
// a.zt (candidates) like the rest of its float32 kernel algebra.
template <typename T, int DMAX>
__device__ __forceinline__ void adjoint_finish_row(const QBatchArgs& a, int64_t row, T* gx) {
    const int q = a.q, r = a.r, d = a.d, kind = a.kernel;
    const int64_t rows = a.b * q;
    const int64_t bidx = row / q;
    const int i = (int)(row % q);
    if (a.dev_err != nullptr && *a.dev_err != 0 && i == 0) a.status[bidx] = BGB_DEVICE_TIMEOUT;
    const int64_t rbase = bidx * q;
    const bool zs = (sizeof(T) == 4) && a.zt != nullptr;
    T zi[DMAX];
#pragma unroll
    for (int k = 0; k < DMAX; ++k)
        zi[k] = (k < d) ? (zs ? (T)a.zt[(int64_t)k * rows + row] : (T)(a.X[row * d + k] * a.inv_ls[k])) : T(0);
    for (int j = 0; j < q + r; ++j) {
        if (j == i) continue;
        const T w = (T)((j < q) ? 2.0 * a.gqq[(bidx * q + i) * q + j] : a.gqb[(bidx * q + i) * r + (j - q)]);
        T dfx[DMAX];
        T r2 = T(0);
#pragma unroll
        for (int k = 0; k < DMAX; ++k) {
            T zj = T(0);
            if (k < d) {
                if (j < q) zj = zs ? (T)a.zt[(int64_t)k * rows + rbase + j] : (T)(a.X[(rbase + j) * d + k] * a.inv_ls[k]);
                else zj = (T)(a.Xb[(int64_t)(j - q) * d + k] * a.inv_ls[k]);
            }
            dfx[k] = zi[k] - zj;
            r2 = fma(dfx[k], dfx[k], r2);
        }
        const T coef = w * dkappa_dr2<T>(kind, r2);
#pragma unroll
        for (int k = 0; k < DMAX; ++k) gx[k] = fma(coef, dfx[k], gx[k]);
    }
#pragma unroll
    for (int k = 0; k < DMAX; ++k)
        if (k < d) a.grad[row * d + k] = 2.0 * a.outputscale * a.inv_ls[k] * (double)gx[k];
}

// d kappa / d r2 in float32 with the fast intrinsics (rsqrtf, __expf: a few ulp,
// far inside the gradient's error budget), for the adjoint sweep; same branches
// as dkappa_dr2.
__device__ __forceinline__ float dkappa_dr2_fast(int kind, float r2) {
    if (kind == BGB_KERNEL_RBF) return -0.5f * __expf(-0.5f * r2);
    const bool live = r2 > (float)kMinSqDist;
    const float rr = live ? r2 : (float)kMinSqDist;
    const float rho = rr * rsqrtf(rr);
    if (kind == BGB_KERNEL_MATERN52) {
        const float sv = 2.2360679774997896964f * rho;
        const float e = __expf(-sv);
        return live ? (-5.f / 6.f) * (1.f + sv) * e : (5.f / 3.f) * e;
    }
    if (kind == BGB_KERNEL_MATERN32) {
        const float sv = 1.7320508075688772935f * rho;
        return live ? -1.5f * __expf(-sv) : 0.f;
    }
    return live ? -__fdividef(__expf(-rho), 2.f * rho) : 0.f;
}

template <typename T, int DMAX, bool FINISH>
__device__ __forceinline__ void adjoint_body(const QBatchArgs& a, const T* __restrict__ Dm,
                                             int64_t ldd, const T* __restrict__ XsT, int64_t slab,
                                             T* __restrict__ part, int64_t bx, int64_t by) {
    using VT = typename Vec16<T>::type;
    constexpr int E = Vec16<T>::E;
    static_assert(DMAX % E == 0, "DMAX must hold whole 16-byte vectors");
    extern __shared__ __align__(16) unsigned char smraw[];
    T* Xc = reinterpret_cast<T*>(smraw);              // [kAdjChunk][DMAX], point-major
    T* Dc = Xc + (size_t)kAdjChunk * DMAX;            // [kAdjRows][kAdjChunk + 1] (float64 only)
    constexpr int LDD = kAdjChunk + 1;
    const int d = a.d, kind = a.kernel;
    const int64_t n = a.n, rows = a.b * a.q;
    const int tid = threadIdx.x;
    const int64_t row0 = bx * kAdjRows;
    const int64_t row = row0 + tid;
    const bool active = row < rows;
    const int64_t cbeg = by * slab;
    const int64_t cend = (cbeg + slab < n) ? cbeg + slab : n;
    T zx[DMAX], g[DMAX];
    float2 zx2[DMAX / 2], g2[DMAX / 2];  // packed copies for the float32 sweep
    const bool zs = (sizeof(T) == 4) && a.zt != nullptr;
#pragma unroll
    for (int k = 0; k < DMAX; ++k) {
        zx[k] = (active && k < d)
                    ? (zs ? (T)a.zt[(int64_t)k * rows + row] : (T)(a.X[row * d + k] * a.inv_ls[k]))
                    : T(0);
        g[k] = T(0);
    }
#pragma unroll
    for (int v = 0; v < DMAX / 2; ++v) {
        zx2[v] = make_float2((float)zx[2 * v], (float)zx[2 * v + 1]);
        g2[v] = make_float2(0.f, 0.f);
    }
    for (int64_t c0 = cbeg; c0 < cend; c0 += kAdjChunk) {
        const int cc = (int)((cend - c0) < kAdjChunk ? (cend - c0) : kAdjChunk);
        __syncthreads();
        if constexpr (sizeof(T) != 4) {
            for (int p = tid; p < kAdjRows * kAdjChunk; p += kAdjRows) {
                const int rr = p / kAdjChunk, c = p % kAdjChunk;
                Dc[rr * LDD + c] = (row0 + rr < rows && c < cc) ? Dm[(row0 + rr) * ldd + c0 + c] : T(0);
            }
        }
        for (int p = tid; p < DMAX * kAdjChunk; p += kAdjRows) {
            const int k = p / kAdjChunk, c = p % kAdjChunk;
            Xc[c * DMAX + k] = (c < cc && k < d) ? XsT[(int64_t)k * n + c0 + c] : T(0);
        }
        __syncthreads();
        if constexpr (sizeof(T) == 4) {
            // each thread streams its own row of D from global memory (16-byte
            // loads along the row; L1 serves the rest of each line), and the pair
            // arithmetic runs on packed float32 pairs of coordinates
            const float2 m1 = make_float2(-1.f, -1.f);
            const float* drow = reinterpret_cast<const float*>(Dm) + row * ldd + c0;
            auto pair = [&](float dk, int c) {
                const float4* xc = reinterpret_cast<const float4*>(Xc + c * DMAX);
                float2 df2[DMAX / 2];
                // two independent packed chains (k mod 4 in {0, 1} and {2, 3})
                float2 r2a = make_float2(0.f, 0.f), r2b = make_float2(0.f, 0.f);
#pragma unroll
                for (int v = 0; v < DMAX / 4; ++v) {
                    const float4 x4 = xc[v];
                    df2[2 * v] = __ffma2_rn(make_float2(x4.x, x4.y), m1, zx2[2 * v]);
                    df2[2 * v + 1] = __ffma2_rn(make_float2(x4.z, x4.w), m1, zx2[2 * v + 1]);
                    r2a = __ffma2_rn(df2[2 * v], df2[2 * v], r2a);
                    r2b = __ffma2_rn(df2[2 * v + 1], df2[2 * v + 1], r2b);
                }
                const float coef = dk * dkappa_dr2_fast(kind, (r2a.x + r2a.y) + (r2b.x + r2b.y));
                const float2 coef2 = make_float2(coef, coef);
#pragma unroll
                for (int v = 0; v < DMAX / 2; ++v) g2[v] = __ffma2_rn(coef2, df2[v], g2[v]);
            };
            if (active) {
                const bool vec = ((reinterpret_cast<uintptr_t>(drow) & 15) == 0);
                int c = 0;
                if (vec) {
                    for (; c + 4 <= cc; c += 4) {
                        const float4 d4 = *reinterpret_cast<const float4*>(drow + c);
                        pair(d4.x, c);
                        pair(d4.y, c + 1);
                        pair(d4.z, c + 2);
                        pair(d4.w, c + 3);
                    }
                }
                for (; c < cc; ++c) pair(drow[c], c);
            }
        } else {
            for (int c = 0; c < cc; ++c) {
                const T dk = Dc[tid * LDD + c];
                const VT* xc = reinterpret_cast<const VT*>(Xc + c * DMAX);
                T df[DMAX];
                T r2a = T(0), r2b = T(0);
#pragma unroll
                for (int v = 0; v < DMAX / E; ++v) {
                    const VT x4 = xc[v];
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                        const int k = v * E + e;
                        df[k] = zx[k] - Vec16<T>::at(x4, e);
                        if (k % 2 == 0) r2a = fma(df[k], df[k], r2a);
                        else r2b = fma(df[k], df[k], r2b);
                    }
                }
                const T coef = dk * dkappa_dr2<T>(kind, r2a + r2b);
#pragma unroll
                for (int k = 0; k < DMAX; ++k) g[k] = fma(coef, df[k], g[k]);
            }
        }
    }
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int v = 0; v < DMAX / 2; ++v) {
            g[2 * v] = g2[v].x;
            g[2 * v + 1] = g2[v].y;
        }
    }
    if (!active) return;
    if constexpr (FINISH) {
        adjoint_finish_row<T, DMAX>(a, row, g);
        return;
    }
    if constexpr (!FINISH) {
    T* pp = part + by * d * rows;
#pragma unroll
    for (int k = 0; k < DMAX; ++k)
        if (k < d) pp[(int64_t)k * rows + row] = g[k];
    }
}

// Sum of the slab partials, one thread per (k, row) element (coalesced over
// rows), compensated; the total overwrites slab 0.

template <typename T, int DMAX, bool FINISH>
__global__ void __launch_bounds__(kAdjRows, (sizeof(T) == 4 && DMAX <= 24) ? 5 : 1)
    adjoint_kernel(const __grid_constant__ QBatchArgs a, const T* __restrict__ Dm, int64_t ldd,
                   const T* __restrict__ XsT, int64_t slab, T* __restrict__ part) {
    adjoint_body<T, DMAX, FINISH>(a, Dm, ldd, XsT, slab, part, blockIdx.x, blockIdx.y);
}

// grouped: model m's CTAs cover its (row block, slab) grid row-major in slabs
template <typename T, int DMAX, bool FINISH>
__global__ void __launch_bounds__(kAdjRows, (sizeof(T) == 4 && DMAX <= 24) ? 5 : 1)
    adjoint_group_kernel(const GroupTab t) {
    const int m = group_model(t);
    const AdjG<T>& g = static_cast<const AdjG<T>*>(t.args)[m];
    const int64_t lb = (int64_t)blockIdx.x - t.off[m];
    adjoint_body<T, DMAX, FINISH>(g.a, g.D, g.ldd, g.XsT, g.slab, g.part, lb % g.gx, lb / g.gx);
}

template <typename T>
__global__ void adjoint_slab_sum_kernel(T* __restrict__ part, int64_t elems, int nslab) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= elems) return;
    T acc = T(0), c = T(0);
    for (int s = 0; s < nslab; ++s) comp_add<T>(acc, c, part[(int64_t)s * elems + e]);
    part[e] = acc - c;
}

template <typename T, int DMAX>
__device__ __forceinline__ void adjoint_finalize_body(const QBatchArgs& a, const T* __restrict__ part,
                                                      int64_t bx) {
    const int64_t rows = a.b * a.q;
    const int64_t row = bx * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    const int d = a.d;
    T gx[DMAX];
#pragma unroll
    for (int k = 0; k < DMAX; ++k) gx[k] = (k < d) ? part[(int64_t)k * rows + row] : T(0);
    adjoint_finish_row<T, DMAX>(a, row, gx);
}

template <typename T, int DMAX>
__global__ void __launch_bounds__(128)
    adjoint_finalize_kernel(const __grid_constant__ QBatchArgs a, const T* __restrict__ part) {
    adjoint_finalize_body<T, DMAX>(a, part, blockIdx.x);
}

// grouped slab sum and finish (models with a single slab have no CTAs here)
template <typename T>
__global__ void adjoint_slab_sum_group_kernel(const GroupTab t) {
    const int m = group_model(t);
    const AdjG<T>& g = static_cast<const AdjG<T>*>(t.args)[m];
    const int64_t elems = (int64_t)g.a.d * g.a.b * g.a.q;
    const int64_t e = ((int64_t)blockIdx.x - t.off[m]) * blockDim.x + threadIdx.x;
    if (e >= elems) return;
    T acc = T(0), c = T(0);
    for (int s = 0; s < g.nslab; ++s) comp_add<T>(acc, c, g.part[(int64_t)s * elems + e]);
    g.part[e] = acc - c;
}

template <typename T, int DMAX>
__global__ void __launch_bounds__(128) adjoint_finalize_group_kernel(const GroupTab t) {
    const int m = group_model(t);
    const AdjG<T>& g = static_cast<const AdjG<T>*>(t.args)[m];
    adjoint_finalize_body<T, DMAX>(g.a, g.part, (int64_t)blockIdx.x - t.off[m]);
}

#if defined(BGB_QB_STATS)
__global__ void posterior_out_kernel(QBatchArgs a, double* mean, double* covar) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = a.q;
    if (idx >= a.b * q * q) return;
    covar[idx] = a.y_std * a.y_std * a.sig[idx];
    if (idx < a.b * q) mean[idx] = a.y_mean + a.y_std * a.mu[idx];
}
#endif  // BGB_QB_STATS

}  // namespace

#if defined(BGB_QB_STATS)
// SMs of the current device (queried once per device, 152 on a GB300; 1 if the
// query fails)
int sm_count() {
    static int num_sms[64] = {};
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < 64 && num_sms[dev] > 0) return num_sms[dev];
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    if (dev >= 0 && dev < 64) num_sms[dev] = v;
    return v;
}

template <typename T>
int launch_sigma_reduce(const QBatchArgs& a, const T* P, const T* C, int64_t ldc,
                        cudaStream_t stream) {
    if (a.b <= 0) return BGB_OK;
    if (a.q <= 4) sigma_reduce_kernel<T, 4><<<(unsigned)a.b, 256, 0, stream>>>(a, P, C, ldc);
    else if (a.q <= 8) sigma_reduce_kernel<T, 8><<<(unsigned)a.b, 256, 0, stream>>>(a, P, C, ldc);
    else {
        const int64_t warps = a.b * a.q * a.q;
        sigma_reduce_pairs_kernel<T><<<(unsigned)ceil_div(warps, 8), 256, 0, stream>>>(a, P, C, ldc);
    }
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
#endif  // BGB_QB_STATS

#if defined(BGB_QB_STEP)
size_t batch_step_smem_bytes(int q, int r, int S) {
    const int D = r + q;
    return sizeof(double) * (size_t)(2 * q * D + 2 * q * q + 2 * q + S + kSampleChunk * q +
                                     (q * q > q * r ? q * q : q * r));
}

size_t batch_step_f32_smem_bytes(int q, int r, int S) {
    const int D = r + q;
    const int qmax = q <= 4 ? 4 : q <= 8 ? 8 : q <= 16 ? 16 : 32;
    return sizeof(double) * (size_t)(2 * q * q + 2 * q * D + (q * q > q * r ? q * q : q * r)) +
           sizeof(float) * (size_t)(D * qmax + S + kDyLd * q);
}

int launch_batch_step(const QBatchArgs& a, int backward, cudaStream_t stream, bool mixed) {
    if (a.b <= 0) return BGB_OK;
    if (a.q > kMaxQ) return BGB_ERR_UNSUPPORTED;
    if (!mixed) {
        const size_t smem = batch_step_smem_bytes(a.q, a.r, a.S);
        if (smem > 200 * 1024) return BGB_ERR_UNSUPPORTED;
        if (smem > 48 * 1024)
            BGB_CUDA_TRY(cudaFuncSetAttribute(batch_step_kernel,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        batch_step_kernel<<<(unsigned)a.b, 128, smem, stream>>>(a, backward);
        BGB_CHECK_LAUNCH();
        return BGB_OK;
    }
    if (a.z32 == nullptr || a.bf32 == nullptr) return BGB_ERR_ARG;
    const size_t smem = batch_step_f32_smem_bytes(a.q, a.r, a.S);
    if (smem > 200 * 1024) return BGB_ERR_UNSUPPORTED;
    int rc = launch_prep_samples(a, stream);
    if (rc) return rc;
    // few t-batches with many samples each: 256 threads per t-batch (small q x S
    // problems keep 64: their fixed per-CTA costs grow with the CTA)
    const bool few = a.b < 2 * kNumSMs && (int64_t)a.S * a.q >= 4096;
#define BGB_BS1(QM, NTH)                                                                         \
    do {                                                                                        \
        if (smem > 48 * 1024)                                                                   \
            BGB_CUDA_TRY(cudaFuncSetAttribute(batch_step_f32_kernel<QM, NTH>,                   \
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                              (int)smem));                                      \
        batch_step_f32_kernel<QM, NTH><<<(unsigned)a.b, NTH, smem, stream>>>(a, backward);      \
    } while (0)
#define BGB_BS(QM)                          \
    do {                                   \
        if (few)                           \
            BGB_BS1(QM, kBsThreadsFew);    \
        else                               \
            BGB_BS1(QM, kBsThreads);       \
    } while (0)
    if (a.q <= 4) BGB_BS(4);
    else if (a.q <= 8) BGB_BS(8);
    else if (a.q <= 16) BGB_BS(16);
    else BGB_BS(32);
#undef BGB_BS
#undef BGB_BS1
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

// Z as float32 and best_f as float pairs (a.z32, a.bf32), the mixed batch step's inputs.
int launch_prep_samples(const QBatchArgs& a, cudaStream_t stream) {
    if (a.z32 == nullptr || a.bf32 == nullptr) return BGB_ERR_ARG;
    const int64_t nz = (int64_t)a.S * (a.r + a.q);
    const int64_t nbf = a.joint == 2 ? (int64_t)a.S * (a.max_tries + 1) : a.S;
    const int64_t np = nz > nbf ? nz : nbf;
    prep_samples_kernel<<<(unsigned)ceil_div(np, 256), 256, 0, stream>>>(
        a.Z, nz, a.joint == 2 ? a.best_f_lv : a.best_f, nbf, a.acqf == BGB_ACQF_QEI, a.z32, a.bf32);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

size_t batch_step_f32_smem(int q, int r, int S) { return batch_step_f32_smem_bytes(q, r, S); }

int launch_batch_step_group(const GroupTab& t, int qmax, size_t smem, int64_t total,
                            cudaStream_t stream) {
    if (total <= 0) return BGB_OK;
    if (qmax > kMaxQ || smem > 200 * 1024 || total > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
#define BGB_BSG(QM)                                                                              \
    do {                                                                                        \
        if (smem > 48 * 1024)                                                                   \
            BGB_CUDA_TRY(cudaFuncSetAttribute(batch_step_f32_group_kernel<QM>,                  \
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                              (int)smem));                                      \
        batch_step_f32_group_kernel<QM><<<(unsigned)total, kBsThreads, smem, stream>>>(t);      \
    } while (0)
    if (qmax <= 4) BGB_BSG(4);
    else if (qmax <= 8) BGB_BSG(8);
    else if (qmax <= 16) BGB_BSG(16);
    else BGB_BSG(32);
#undef BGB_BSG
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
#endif  // BGB_QB_STEP

#if defined(BGB_QB_STATS)
template <typename T>
int launch_qstats(const QBatchArgs& a, const T* V, int64_t ldv, const T* beta, const T* Vb,
                  cudaStream_t stream) {
    if (a.b <= 0) return BGB_OK;
    if (a.q > 8 || a.r > 4 || (a.r > 0 && Vb == nullptr)) return BGB_ERR_UNSUPPORTED;
    constexpr int E = Vec16<T>::E;
    auto al = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) % 16) == 0; };
    const int vec_ok = (ldv % E == 0) && (a.n % E == 0) && al(V) && al(beta) &&
                       (a.r == 0 || al(Vb));
    const unsigned grid = (unsigned)a.b;
    if (a.q <= 4 && a.r <= 2)
        qstats_kernel<T, 4, 2><<<grid, kQstatsThreads, 0, stream>>>(a, V, ldv, beta, Vb, vec_ok);
    else if (a.q <= 4)
        qstats_kernel<T, 4, 4><<<grid, kQstatsThreads, 0, stream>>>(a, V, ldv, beta, Vb, vec_ok);
    else if (a.r <= 2)
        qstats_kernel<T, 8, 2><<<grid, kQstatsThreads, 0, stream>>>(a, V, ldv, beta, Vb, vec_ok);
    else
        qstats_kernel<T, 8, 4><<<grid, kQstatsThreads, 0, stream>>>(a, V, ldv, beta, Vb, vec_ok);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int launch_qstats_group(const GroupTab& t, int qmax, int rmax, int64_t total, cudaStream_t stream) {
    if (total <= 0) return BGB_OK;
    if (qmax > 8 || rmax > 4 || total > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
    const unsigned grid = (unsigned)total;
    if (qmax <= 4 && rmax <= 2)
        qstats_group_kernel<float, 4, 2><<<grid, kQstatsThreads, 0, stream>>>(t);
    else if (qmax <= 4)
        qstats_group_kernel<float, 4, 4><<<grid, kQstatsThreads, 0, stream>>>(t);
    else if (rmax <= 2)
        qstats_group_kernel<float, 8, 2><<<grid, kQstatsThreads, 0, stream>>>(t);
    else
        qstats_group_kernel<float, 8, 4><<<grid, kQstatsThreads, 0, stream>>>(t);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

template <typename T>
int launch_qstats_tile(const QBatchArgs& a, const T* V, int64_t ldv, const T* beta, const T* Vb,
                       void* scratch, size_t scratch_bytes, cudaStream_t stream) {
    if (a.b <= 0) return BGB_OK;
    const int q = a.q, r = a.r;
    const int nout = q * (q + 1) / 2 + q + q * r;
    const size_t smem = sizeof(T) * (size_t)(q + 1 + r) * kQtCols;
    if (q > 32 || nout > kQtThreads * kQtOut || smem > 96 * 1024 || a.b > 0x7fffffff)
        return BGB_ERR_UNSUPPORTED;
    if (smem > 48 * 1024)
        BGB_CUDA_TRY(cudaFuncSetAttribute(qstats_tile_kernel<T>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // few t-batches: split each one's tiles over CTAs (about two waves of CTAs),
    // as far as the scratch holds the partial sums
    const int64_t tiles = ceil_div(a.n, (int64_t)kQtCols);
    int64_t nsplit = ceil_div((int64_t)sm_count() * 2, a.b);
    if (nsplit > tiles) nsplit = tiles;
    while (nsplit > 1 && (size_t)(a.b * nsplit * nout) * sizeof(double) > scratch_bytes) --nsplit;
    if (nsplit < 1 || a.b * nsplit > 0x7fffffff) nsplit = 1;
    double* part = nsplit > 1 ? static_cast<double*>(scratch) : nullptr;
    qstats_tile_kernel<T><<<(unsigned)(a.b * nsplit), kQtThreads, smem, stream>>>(
        a, V, ldv, beta, Vb, (int)nsplit, part);
    BGB_CHECK_LAUNCH();
    if (nsplit > 1) {
        qstats_tile_finish_kernel<T><<<(unsigned)a.b, kQtThreads, 0, stream>>>(a, (int)nsplit, part);
        BGB_CHECK_LAUNCH();
    }
    return BGB_OK;
}

template <typename T>
int launch_row_dots(const QBatchArgs& a, const T* V, int64_t ldv, const T* beta, const T* Vb, T* P,
                    cudaStream_t stream) {
    const int64_t rows = a.b * a.q;
    if (rows <= 0) return BGB_OK;
    row_dots_kernel<T><<<(unsigned)ceil_div(rows, 8), 256, 0, stream>>>(a, V, ldv, beta, Vb, P);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

#endif  // BGB_QB_STATS

#if defined(BGB_QB_MIX)
template <typename T>
int launch_mix_rows(const QBatchArgs& a, const T* V, int64_t ldv, const T* Vb, const T* beta, T* H,
                    cudaStream_t stream, __half* H16, __half* H16_lo, int64_t ldh) {
    if (a.b <= 0) return BGB_OK;
    if (a.q > kMaxQ) return BGB_ERR_UNSUPPORTED;
    if (H16 != nullptr && (sizeof(T) != 4 || H16_lo == nullptr || a.hmul == nullptr)) return BGB_ERR_ARG;
    const size_t smem = sizeof(T) * (size_t)(a.q * a.q + a.q * a.r + a.q) + sizeof(float) * a.q;
    if (smem > 48 * 1024) return BGB_ERR_UNSUPPORTED;
    const int64_t ld = ldh > 0 ? ldh : a.n;
    constexpr int E = Vec16<T>::E;
    auto al = [](const void* p, int b) { return (reinterpret_cast<uintptr_t>(p) % b) == 0; };
    const bool vec = (a.n % E == 0) && (ldv % E == 0) && (ld % E == 0) && al(V, 16) &&
                     al(beta, 16) && (a.r == 0 || al(Vb, 16)) &&
                     (H16 != nullptr ? (al(H16, 8) && al(H16_lo, 8)) : al(H, 16));
    auto groups = [&](int64_t per) { return (unsigned)mix_rows_groups(a, (int)(per / 256), 0); };
#define BGB_MIX(QM)                                                                              \
    do {                                                                                        \
        if (vec) {                                                                              \
            dim3 grid(groups(256 * E), (unsigned)a.b);                                          \
            mix_rows_kernel<T, QM, E><<<grid, 256, smem, stream>>>(a, V, ldv, Vb, beta, H, H16,   \
                                                                   H16_lo, ld);                 \
        } else {                                                                                \
            dim3 grid(groups(256), (unsigned)a.b);                                              \
            mix_rows_kernel<T, QM, 1><<<grid, 256, smem, stream>>>(a, V, ldv, Vb, beta, H, H16,   \
                                                                   H16_lo, ld);                 \
        }                                                                                       \
    } while (0)
    if (a.q <= 4) BGB_MIX(4);
    else if (a.q <= 8) BGB_MIX(8);
    else if (a.q <= 16) BGB_MIX(16);
    else BGB_MIX(32);
#undef BGB_MIX
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
// column groups per t-batch for vector width E: enough CTAs for ~6 per SM, each
// CTA loads its t-batch's seeds once and strides over the rest
// (total_b: the t-batches of every launch sharing the GPU, 0 for a.b alone)
int64_t mix_rows_groups(const QBatchArgs& a, int E, int64_t total_b) {
    const int64_t all = ceil_div(a.n, (int64_t)256 * E);
    const int64_t tb = total_b > 0 ? total_b : (a.b > 0 ? a.b : 1);
    const int64_t want = ceil_div((int64_t)sm_count() * 6, tb);
    return want < 1 ? 1 : (want > all ? all : want);
}

size_t mix_rows_smem_bytes(const QBatchArgs& a) {
    return sizeof(float) * (size_t)(a.q * a.q + a.q * a.r + a.q) + sizeof(float) * a.q;
}

// float32, scalar columns (E = 1: the models' n and strides need not be multiples of 4)
int launch_mix_rows_group(const GroupTab& t, int qmax, size_t smem, int64_t total,
                          cudaStream_t stream) {
    if (total <= 0) return BGB_OK;
    if (qmax > kMaxQ || smem > 48 * 1024 || total > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
    const unsigned grid = (unsigned)total;
    if (qmax <= 4) mix_rows_group_kernel<float, 4, 1><<<grid, 256, smem, stream>>>(t);
    else if (qmax <= 8) mix_rows_group_kernel<float, 8, 1><<<grid, 256, smem, stream>>>(t);
    else if (qmax <= 16) mix_rows_group_kernel<float, 16, 1><<<grid, 256, smem, stream>>>(t);
    else mix_rows_group_kernel<float, 32, 1><<<grid, 256, smem, stream>>>(t);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
#endif  // BGB_QB_MIX

#if defined(BGB_QB_ADJ_F64) || defined(BGB_QB_ADJ_F32)
template <typename T, int DMAX>
size_t adjoint_smem_bytes() {
    // float32 rows stream D from global memory; float64 stages its D tile
    return sizeof(T) * ((size_t)kAdjChunk * DMAX +
                        (sizeof(T) == 4 ? 0 : (size_t)kAdjRows * (kAdjChunk + 1)));
}

// part_cap: elements of scratch available for the slab partials (0: one slab).
template <typename T>
int launch_adjoint(const QBatchArgs& a, const T* D, int64_t ldd, const T* XsT, T* part,
                   int64_t part_cap, cudaStream_t stream) {
    const int64_t rows = a.b * a.q;
    if (rows <= 0) return BGB_OK;
    int64_t row_blocks, nslab, slab;
    adjoint_split(a, part != nullptr ? part_cap : 0, &row_blocks, &nslab, &slab);
    T* pp = nslab > 1 ? part : nullptr;
    dim3 grid((unsigned)row_blocks, (unsigned)nslab);
#define BGB_ADJ(DM)                                                                              \
    do {                                                                                        \
        const size_t smem = adjoint_smem_bytes<T, DM>();                                        \
        if (pp == nullptr) {                                                                    \
            if (smem > 48 * 1024)                                                               \
                BGB_CUDA_TRY(cudaFuncSetAttribute(adjoint_kernel<T, DM, true>,                  \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                                  (int)smem));                                  \
            adjoint_kernel<T, DM, true><<<grid, kAdjRows, smem, stream>>>(a, D, ldd, XsT, slab, pp); \
            BGB_CHECK_LAUNCH();                                                                 \
        } else {                                                                                \
            if (smem > 48 * 1024)                                                               \
                BGB_CUDA_TRY(cudaFuncSetAttribute(adjoint_kernel<T, DM, false>,                 \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                                  (int)smem));                                  \
            adjoint_kernel<T, DM, false><<<grid, kAdjRows, smem, stream>>>(a, D, ldd, XsT, slab, pp); \
            BGB_CHECK_LAUNCH();                                                                 \
            const int64_t elems = (int64_t)a.d * rows;                                          \
            adjoint_slab_sum_kernel<T><<<(unsigned)ceil_div(elems, 256), 256, 0, stream>>>(      \
                pp, elems, (int)nslab);                                                         \
            BGB_CHECK_LAUNCH();                                                                 \
            adjoint_finalize_kernel<T, DM><<<(unsigned)ceil_div(rows, 128), 128, 0, stream>>>(  \
                a, pp);                                                                         \
            BGB_CHECK_LAUNCH();                                                                 \
        }                                                                                       \
    } while (0)
    if (a.d <= 8) BGB_ADJ(8);
    else if (a.d <= 12) BGB_ADJ(12);
    else if (a.d <= 16) BGB_ADJ(16);
    else if (a.d <= 20) BGB_ADJ(20);
    else if (a.d <= 24) BGB_ADJ(24);
    else if (a.d <= 32) BGB_ADJ(32);
    else if (a.d <= 64) BGB_ADJ(64);
    else return BGB_ERR_UNSUPPORTED;
#undef BGB_ADJ
    return BGB_OK;
}

#endif  // BGB_QB_ADJ_*

#if defined(BGB_QB_ADJ_F32)
// slabs: a.adj_ctas_per_sm CTAs per SM (default 16: about four waves of four
// resident CTAs), slabs of whole chunks, partials within part_cap elements
void adjoint_split(const QBatchArgs& a, int64_t part_cap, int64_t* row_blocks_out,
                   int64_t* nslab_out, int64_t* slab_out) {
    const int64_t rows = a.b * a.q;
    const int64_t row_blocks = ceil_div(rows > 0 ? rows : 1, kAdjRows);
    const int num_sms = sm_count();
    const int64_t chunks = ceil_div(a.n, kAdjChunk);
    const int64_t per_sm = a.adj_ctas_per_sm > 0 ? a.adj_ctas_per_sm : 16;
    int64_t nslab = ceil_div((int64_t)num_sms * per_sm, row_blocks);
    if (nslab > chunks) nslab = chunks;
    if (nslab > 65535) nslab = 65535;
    if (part_cap <= 0) nslab = 1;
    while (nslab > 1 && nslab * a.d * rows > part_cap) --nslab;
    if (nslab < 1) nslab = 1;
    const int64_t slab = ceil_div(chunks, nslab) * kAdjChunk;
    *row_blocks_out = row_blocks;
    *nslab_out = ceil_div(a.n, slab);
    *slab_out = slab;
}

int launch_adjoint_group(const GroupTab& t, int dmax, bool partials, int64_t total,
                         cudaStream_t stream) {
    if (total <= 0) return BGB_OK;
    if (total > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
    const unsigned grid = (unsigned)total;
#define BGB_ADJG(DM)                                                                             \
    do {                                                                                        \
        const size_t smem = adjoint_smem_bytes<float, DM>();                                    \
        if (partials) {                                                                         \
            if (smem > 48 * 1024)                                                               \
                BGB_CUDA_TRY(cudaFuncSetAttribute(adjoint_group_kernel<float, DM, false>,       \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                                  (int)smem));                                  \
            adjoint_group_kernel<float, DM, false><<<grid, kAdjRows, smem, stream>>>(t);        \
        } else {                                                                                \
            if (smem > 48 * 1024)                                                               \
                BGB_CUDA_TRY(cudaFuncSetAttribute(adjoint_group_kernel<float, DM, true>,        \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                                  (int)smem));                                  \
            adjoint_group_kernel<float, DM, true><<<grid, kAdjRows, smem, stream>>>(t);         \
        }                                                                                       \
    } while (0)
    if (dmax <= 8) BGB_ADJG(8);
    else if (dmax <= 12) BGB_ADJG(12);
    else if (dmax <= 16) BGB_ADJG(16);
    else if (dmax <= 20) BGB_ADJG(20);
    else if (dmax <= 24) BGB_ADJG(24);
    else if (dmax <= 32) BGB_ADJG(32);
    else if (dmax <= 64) BGB_ADJG(64);
    else return BGB_ERR_UNSUPPORTED;
#undef BGB_ADJG
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int launch_adjoint_finish_group(const GroupTab& t_sum, int64_t total_sum, const GroupTab& t_fin,
                                int dmax, int64_t total_fin, cudaStream_t stream) {
    if (total_sum > 0x7fffffff || total_fin > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
    if (total_sum > 0) {
        adjoint_slab_sum_group_kernel<float><<<(unsigned)total_sum, 256, 0, stream>>>(t_sum);
        BGB_CHECK_LAUNCH();
    }
    if (total_fin <= 0) return BGB_OK;
    const unsigned grid = (unsigned)total_fin;
    if (dmax <= 8) adjoint_finalize_group_kernel<float, 8><<<grid, 128, 0, stream>>>(t_fin);
    else if (dmax <= 12) adjoint_finalize_group_kernel<float, 12><<<grid, 128, 0, stream>>>(t_fin);
    else if (dmax <= 16) adjoint_finalize_group_kernel<float, 16><<<grid, 128, 0, stream>>>(t_fin);
    else if (dmax <= 20) adjoint_finalize_group_kernel<float, 20><<<grid, 128, 0, stream>>>(t_fin);
    else if (dmax <= 24) adjoint_finalize_group_kernel<float, 24><<<grid, 128, 0, stream>>>(t_fin);
    else if (dmax <= 32) adjoint_finalize_group_kernel<float, 32><<<grid, 128, 0, stream>>>(t_fin);
    else if (dmax <= 64) adjoint_finalize_group_kernel<float, 64><<<grid, 128, 0, stream>>>(t_fin);
    else return BGB_ERR_UNSUPPORTED;
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
#endif  // BGB_QB_ADJ_F32

#if defined(BGB_QB_STATS)
int launch_posterior_out(const QBatchArgs& a, double* mean, double* covar, cudaStream_t stream) {
    const int64_t tot = a.b * a.q * a.q;
    if (tot <= 0) return BGB_OK;
    posterior_out_kernel<<<(unsigned)ceil_div(tot, 256), 256, 0, stream>>>(a, mean, covar);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

template int launch_sigma_reduce<double>(const QBatchArgs&, const double*, const double*, int64_t,
                                         cudaStream_t);
template int launch_sigma_reduce<float>(const QBatchArgs&, const float*, const float*, int64_t,
                                        cudaStream_t);
template int launch_qstats<double>(const QBatchArgs&, const double*, int64_t, const double*,
                                   const double*, cudaStream_t);
template int launch_qstats<float>(const QBatchArgs&, const float*, int64_t, const float*,
                                  const float*, cudaStream_t);
template int launch_qstats_tile<double>(const QBatchArgs&, const double*, int64_t, const double*,
                                        const double*, void*, size_t, cudaStream_t);
template int launch_qstats_tile<float>(const QBatchArgs&, const float*, int64_t, const float*,
                                       const float*, void*, size_t, cudaStream_t);
template int launch_row_dots<double>(const QBatchArgs&, const double*, int64_t, const double*,
                                     const double*, double*, cudaStream_t);
template int launch_row_dots<float>(const QBatchArgs&, const float*, int64_t, const float*,
                                    const float*, float*, cudaStream_t);
#endif  // BGB_QB_STATS
#if defined(BGB_QB_MIX)
template int launch_mix_rows<double>(const QBatchArgs&, const double*, int64_t, const double*,
                                     const double*, double*, cudaStream_t, __half*, __half*,
                                     int64_t);
template int launch_mix_rows<float>(const QBatchArgs&, const float*, int64_t, const float*,
                                    const float*, float*, cudaStream_t, __half*, __half*, int64_t);
#endif  // BGB_QB_MIX
#if defined(BGB_QB_ADJ_F64)
template int launch_adjoint<double>(const QBatchArgs&, const double*, int64_t, const double*,
                                    double*, int64_t, cudaStream_t);
#endif
#if defined(BGB_QB_ADJ_F32)
template int launch_adjoint<float>(const QBatchArgs&, const float*, int64_t, const float*,
                                   float*, int64_t, cudaStream_t);
#endif

}  // namespace bgb
