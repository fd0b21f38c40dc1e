// Fused log-areas of qLogEHVI / qLogNEHVI: forward and backward over
// obj_subsets (B, n_sub, i, m) and box-decomposition cells (B_cells, nc, m),
// B_cells in {1, B}.
//
// Replaces the reference's CPU kernel botorch/csrc/logei_fused.cpp:184-374
// (called from botorch/acquisition/multi_objective/logei.py:107-165,386-392),
// which fuses steps 1-4 of _compute_log_qehvi:
//   li[j][k]  = log_fatplus(obj[b][s][j][k] - lower[c][k], tau_relu)
//   lim[k]    = fatmin_j li[j][k]                          (Pareto kernel, tau_max)
//   area      = sum_k fatmin(lim[k], log(min(upper[c][k], clamp) - lower[c][k]))
//   out[b][c][s] = area
// and its gradient with respect to obj (the only differentiable input),
// summed over cells. The smooth functions keep the reference's branches:
// softplus linear above y = 20 and exp below y = -20, log_fatplus -> -1e30
// where tau * fatplus underflows to 0, fatmin returning the minimum (one-hot
// gradient) when it is below -1e29, and the upper-bound clamp (1e10 in
// double, 1e8 in float).
//
// GPU layout: forward runs one thread per output element (b, c, s), s
// fastest, so that the stores are coalesced; the thread keeps the i values
// of one objective at a time in registers. Backward runs G adjacent threads
// per (b, s, k) (the gradient factorises over the objectives k): each takes
// every G-th cell, keeps li, d li / d x and its i partial sums in registers,
// and the G partial sums are added with warp shuffles. G grows with the
// number of cells until the launch fills the GPU.
#include <math.h>

#include "bgb_common.cuh"

namespace bgb {

namespace {

constexpr int kLaMaxI = 32;  // subset size limit (the reference's MAX_I)
constexpr int kLaMaxM = 8;   // objective limit (the reference's MAX_M)
constexpr int kLaThreads = 256;

template <typename T> struct LaMath;
template <> struct LaMath<double> {
    static __device__ __forceinline__ double exp_(double x) { return exp(x); }
    static __device__ __forceinline__ double log_(double x) { return log(x); }
    static __device__ __forceinline__ double log1p_(double x) { return log1p(x); }
    static constexpr double kClamp = 1e10;
    static constexpr double kExpZero = -750.0;  // exp(y) rounds to +0 below this
    static constexpr double kSigOne = 38.0;     // 1 + exp(-y) rounds to 1 above this
};
template <> struct LaMath<float> {
    static __device__ __forceinline__ float exp_(float x) { return expf(x); }
    static __device__ __forceinline__ float log_(float x) { return logf(x); }
    static __device__ __forceinline__ float log1p_(float x) { return log1pf(x); }
    static constexpr float kClamp = 1e8f;
    static constexpr float kExpZero = -105.f;
    static constexpr float kSigOne = 18.f;
};

// The exp calls are skipped where their result is exactly what the rounded
// arithmetic gives anyway (exp underflowing to +0, 1 + exp(-y) rounding to
// 1): the values are unchanged and most elements, far from the cell corners
// (|y| = |x| / tau_relu >> 20), need no exp at all.
template <typename T>
__device__ __forceinline__ T la_softplus(T y) {
    if (y > T(20)) return y;
    if (y < T(-20)) return y < LaMath<T>::kExpZero ? T(0) : LaMath<T>::exp_(y);
    return LaMath<T>::log1p_(LaMath<T>::exp_(y));
}

template <typename T>
__device__ __forceinline__ T la_sigmoid(T y) {
    if (y >= T(0)) return y > LaMath<T>::kSigOne ? T(1) : T(1) / (T(1) + LaMath<T>::exp_(-y));
    if (y < LaMath<T>::kExpZero) return T(0);
    const T e = LaMath<T>::exp_(y);
    return e / (T(1) + e);
}

template <typename T>
__device__ __forceinline__ T la_log_fatplus(T x, T tau, T inv_tau) {
    const T y = x * inv_tau;
    const T f = la_softplus(y) + T(0.1) * (T(1) / (T(1) + y * y));
    const T v = tau * f;
    return v > T(0) ? LaMath<T>::log_(v) : T(-1e30);
}

// value and d/dx of log_fatplus
template <typename T>
__device__ __forceinline__ void la_log_fatplus_grad(T x, T tau, T inv_tau, T& val, T& grad) {
    const T y = x * inv_tau;
    const T cy = T(1) / (T(1) + y * y);
    const T f = la_softplus(y) + T(0.1) * cy;
    const T tf = tau * f;
    if (tf <= T(0)) {
        val = T(-1e30);
        grad = T(0);
        return;
    }
    val = LaMath<T>::log_(tf);
    grad = (la_sigmoid(y) - T(2) * T(0.1) * y * cy * cy) / tf;
}

// min(upper, clamp), returning `upper` unless clamp < upper
template <typename T>
__device__ __forceinline__ T la_min_clamp(T u) {
    return LaMath<T>::kClamp < u ? LaMath<T>::kClamp : u;
}

// Pareto kernel 2 / (2 + 2z + z^2) and its derivative
template <typename T>
__device__ __forceinline__ T la_pareto(T z) {
    return T(2) / (T(2) + T(2) * z + z * z);
}
// value and derivative from one reciprocal: 2 RN(1/d) is RN(2/d) exactly, so
// the value is unchanged; the derivative moves by a few ulps
template <typename T>
__device__ __forceinline__ void la_pareto_vd(T z, T& val, T& deriv) {
    const T d = T(2) + T(2) * z + z * z;
    const T r = T(1) / d;
    val = T(2) * r;
    deriv = T(-2) * (T(2) + T(2) * z) * r * r;
}

// fatmin of two values and d/d(first)
template <typename T>
__device__ __forceinline__ T la_fatmin2(T a, T b, T tau, T inv_tau, T* ga) {
    const bool a_min = !(b < a);
    const T mn = a_min ? a : b;
    if (mn < T(-1e29)) {
        if (ga) *ga = a_min ? T(1) : T(0);
        return mn;
    }
    const T other = a_min ? b : a;
    const T z = (other - mn) * inv_tau;
    if (!ga) return mn - tau * LaMath<T>::log_(T(1) + la_pareto(z));  // pareto(0) = 1
    T pv, pd;
    la_pareto_vd(z, pv, pd);
    const T S = T(1) + pv;
    // sum of the derivatives (pareto'(0) = -1 for the minimum);
    // d/d(min) = 1 + (S_pd - pareto'(0)) / S, d/d(other) = -pd / S
    const T S_pd = T(-1) + pd;
    *ga = a_min ? T(1) + (S_pd + T(1)) / S : -pd / S;
    return mn - tau * LaMath<T>::log_(S);
}

// ---------------------------------------------------------------------------
// forward: out[b][c][s]
template <typename T, int IM>
__global__ void __launch_bounds__(kLaThreads) log_areas_forward_kernel(
    const T* __restrict__ obj, int64_t B, int64_t n_sub, int isz, int m,
    const T* __restrict__ lower, const T* __restrict__ upper, int64_t B_cells, int64_t nc,
    T tau_relu, T tau_max, T* __restrict__ out) {
    const int64_t total = B * nc * n_sub;
    const T inv_relu = T(1) / tau_relu, inv_max = T(1) / tau_max;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = idx % n_sub;
        const int64_t bc = idx / n_sub;
        const int64_t c = bc % nc, b = bc / nc;
        const int64_t cb = B_cells == 1 ? 0 : b;
        const T* o = obj + (b * n_sub + s) * isz * m;
        const T* lo = lower + (cb * nc + c) * m;
        const T* up = upper + (cb * nc + c) * m;
        T area = T(0);
        for (int k = 0; k < m; ++k) {
            const T lk = lo[k];
            const T lcl = LaMath<T>::log_(la_min_clamp(up[k]) - lk);
            T li[IM];
            T mn = T(0);
#pragma unroll
            for (int j = 0; j < IM; ++j) {
                if (j < isz) {
                    li[j] = la_log_fatplus(o[j * m + k] - lk, tau_relu, inv_relu);
                    if (j == 0 || li[j] < mn) mn = li[j];
                }
            }
            T lim;
            if (isz == 1 || mn < T(-1e29)) {
                lim = isz == 1 ? li[0] : mn;
            } else {
                T S = T(0);
#pragma unroll
                for (int j = 0; j < IM; ++j)
                    if (j < isz) S += la_pareto((li[j] - mn) * inv_max);
                lim = mn - tau_max * LaMath<T>::log_(S);
            }
            area += la_fatmin2(lim, lcl, tau_max, inv_max, (T*)nullptr);
        }
        out[idx] = area;
    }
}

// ---------------------------------------------------------------------------
// forward that also keeps the Jacobian of each area with respect to its
// subset's objective values: jac[b][c][s][j][k] = d out[b][c][s] / d obj[b][s][j][k]
// (the pair fatmin's weight x the subset fatmin's weight x d log_fatplus / dx).
// Same thread layout as the forward; each thread writes its i m entries
// contiguously, so a warp writes one contiguous run.
template <typename T, int IM>
__global__ void __launch_bounds__(kLaThreads) log_areas_forward_jac_kernel(
    const T* __restrict__ obj, int64_t B, int64_t n_sub, int isz, int m,
    const T* __restrict__ lower, const T* __restrict__ upper, int64_t B_cells, int64_t nc,
    T tau_relu, T tau_max, T* __restrict__ out, T* __restrict__ jac) {
    const int64_t total = B * nc * n_sub;
    const T inv_relu = T(1) / tau_relu, inv_max = T(1) / tau_max;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = idx % n_sub;
        const int64_t bc = idx / n_sub;
        const int64_t c = bc % nc, b = bc / nc;
        const int64_t cb = B_cells == 1 ? 0 : b;
        const T* o = obj + (b * n_sub + s) * isz * m;
        const T* lo = lower + (cb * nc + c) * m;
        const T* up = upper + (cb * nc + c) * m;
        T* J = jac + idx * isz * m;
        T area = T(0);
        for (int k = 0; k < m; ++k) {
            const T lk = lo[k];
            const T lcl = LaMath<T>::log_(la_min_clamp(up[k]) - lk);
            T li[IM], lg[IM];
            T mn = T(0);
            int ami = 0;
#pragma unroll
            for (int j = 0; j < IM; ++j) {
                if (j < isz) {
                    la_log_fatplus_grad(o[j * m + k] - lk, tau_relu, inv_relu, li[j], lg[j]);
                    if (j == 0 || li[j] < mn) {
                        mn = li[j];
                        ami = j;
                    }
                }
            }
            if (isz == 1 || mn < T(-1e29)) {
                const T lim = isz == 1 ? li[0] : mn;
                T g2;
                area += la_fatmin2(lim, lcl, tau_max, inv_max, &g2);
#pragma unroll
                for (int j = 0; j < IM; ++j)
                    if (j < isz) J[j * m + k] = j == ami ? g2 * lg[j] : T(0);
            } else {
                T S = T(0), S_pd = T(0);
#pragma unroll
                for (int j = 0; j < IM; ++j) {
                    if (j < isz) {
                        T pv;
                        la_pareto_vd((li[j] - mn) * inv_max, pv, li[j]);  // li[j] <- pareto'(z_j)
                        S += pv;
                        S_pd += li[j];
                    }
                }
                const T lim = mn - tau_max * LaMath<T>::log_(S);
                T g2;
                area += la_fatmin2(lim, lcl, tau_max, inv_max, &g2);
                const T inv_S = T(1) / S;
#pragma unroll
                for (int j = 0; j < IM; ++j) {
                    if (j < isz) {
                        const T w = j == ami ? T(1) + (S_pd + T(1)) * inv_S : -li[j] * inv_S;
                        J[j * m + k] = g2 * w * lg[j];
                    }
                }
            }
        }
        out[idx] = area;
    }
}

// g_obj[b][s][e] = sum_c g_out[b][c][s] jac[b][c][s][e], e = (j, k): one thread
// per (b, s, e), e fastest, so consecutive threads read consecutive Jacobian
// entries of one cell; cells in order.
template <typename T>
__global__ void __launch_bounds__(kLaThreads) log_areas_backward_jac_kernel(
    const T* __restrict__ g_out, const T* __restrict__ jac, int64_t B, int64_t n_sub, int im,
    int64_t nc, T* __restrict__ g_obj) {
    const int64_t total = B * n_sub * im;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t % im;
        const int64_t bs = t / im;
        const int64_t s = bs % n_sub, b = bs / n_sub;
        const T* J = jac + (b * nc * n_sub + s) * im + e;  // cell 0
        const T* go = g_out + b * nc * n_sub + s;
        const int64_t cstride = n_sub * im;
        T acc = T(0);
#pragma unroll 8
        for (int64_t c = 0; c < nc; ++c) acc = fma(go[c * n_sub], J[c * cstride], acc);
        g_obj[t] = acc;
    }
}

// ---------------------------------------------------------------------------
// backward: g_obj[b][s][j][k] = sum_c g_out[b][c][s] d out[b][c][s] / d obj[b][s][j][k]
template <typename T, int IM>
__global__ void __launch_bounds__(kLaThreads) log_areas_backward_kernel(
    const T* __restrict__ g_out, const T* __restrict__ obj, int64_t B, int64_t n_sub, int isz,
    int m, const T* __restrict__ lower, const T* __restrict__ upper, int64_t B_cells, int64_t nc,
    T tau_relu, T tau_max, int G, T* __restrict__ g_obj) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane_g = (int)(t % G);
    const int64_t rest = t / G;
    const int k = (int)(rest % m);
    const int64_t bs = rest / m;
    const bool valid = bs < B * n_sub;
    const int64_t b = valid ? bs / n_sub : 0, s = valid ? bs % n_sub : 0;
    const int64_t cb = B_cells == 1 ? 0 : b;
    const T inv_relu = T(1) / tau_relu, inv_max = T(1) / tau_max;
    const T* o = obj + (valid ? bs : 0) * isz * m + k;
    T g[IM];
#pragma unroll
    for (int j = 0; j < IM; ++j) g[j] = T(0);
    if (valid) {
        for (int64_t c = lane_g; c < nc; c += G) {
            const T lk = lower[(cb * nc + c) * m + k];
            const T lcl = LaMath<T>::log_(la_min_clamp(upper[(cb * nc + c) * m + k]) - lk);
            const T go = g_out[(b * nc + c) * n_sub + s];
            T li[IM], lg[IM];
            T mn = T(0);
            int ami = 0;
#pragma unroll
            for (int j = 0; j < IM; ++j) {
                if (j < isz) {
                    la_log_fatplus_grad(o[j * m] - lk, tau_relu, inv_relu, li[j], lg[j]);
                    if (j == 0 || li[j] < mn) {
                        mn = li[j];
                        ami = j;
                    }
                }
            }
            if (isz == 1 || mn < T(-1e29)) {
                // fatmin over the subset is the minimum itself: one-hot weights
                const T lim = isz == 1 ? li[0] : mn;
                T g2;
                la_fatmin2(lim, lcl, tau_max, inv_max, &g2);
                const T gl = go * g2;
#pragma unroll
                for (int j = 0; j < IM; ++j)
                    if (j == ami && j < isz) g[j] += gl * lg[j];
            } else {
                T S = T(0), S_pd = T(0);
#pragma unroll
                for (int j = 0; j < IM; ++j) {
                    if (j < isz) {
                        T pv;
                        la_pareto_vd((li[j] - mn) * inv_max, pv, li[j]);  // li[j] <- pareto'(z_j)
                        S += pv;
                        S_pd += li[j];
                    }
                }
                const T lim = mn - tau_max * LaMath<T>::log_(S);
                T g2;
                la_fatmin2(lim, lcl, tau_max, inv_max, &g2);
                const T gl = go * g2;
                const T inv_S = T(1) / S;
#pragma unroll
                for (int j = 0; j < IM; ++j) {
                    if (j < isz) {
                        // pareto'(0) = -1
                        const T w = j == ami ? T(1) + (S_pd + T(1)) * inv_S : -li[j] * inv_S;
                        g[j] += gl * w * lg[j];
                    }
                }
            }
        }
    }
    // add the G partial sums (G adjacent lanes of one warp; every lane takes part)
    for (int off = G >> 1; off > 0; off >>= 1) {
#pragma unroll
        for (int j = 0; j < IM; ++j) g[j] += __shfl_xor_sync(0xffffffffu, g[j], off);
    }
    if (valid && lane_g == 0) {
        T* go_ = g_obj + bs * isz * m + k;
#pragma unroll
        for (int j = 0; j < IM; ++j)
            if (j < isz) go_[j * m] = g[j];
    }
}

int la_bucket(int64_t isz) { return isz <= 4 ? 4 : isz <= 8 ? 8 : isz <= 16 ? 16 : 32; }

int la_check(int64_t B, int64_t n_sub, int64_t isz, int64_t m, int64_t B_cells, int64_t nc,
             double tau_relu, double tau_max) {
    if (B < 0 || n_sub < 0 || nc < 0 || isz < 1 || m < 1) return BGB_ERR_ARG;
    if (B_cells != 1 && B_cells != B) return BGB_ERR_ARG;
    if (!(tau_relu > 0.0) || !(tau_max > 0.0)) return BGB_ERR_ARG;
    if (isz > kLaMaxI || m > kLaMaxM) return BGB_ERR_UNSUPPORTED;
    return BGB_OK;
}

int sm_count_la() {
    static int n[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return kNumSMs;
    if (dev < 0 || dev >= 64) return kNumSMs;
    if (n[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = kNumSMs;
        n[dev] = v;
    }
    return n[dev];
}

template <typename T>
int log_areas_forward(const T* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                      const T* lower, const T* upper, int64_t B_cells, int64_t nc,
                      double tau_relu, double tau_max, T* out, cudaStream_t st) {
    int rc = la_check(B, n_sub, isz, m, B_cells, nc, tau_relu, tau_max);
    if (rc) return rc;
    const int64_t total = B * nc * n_sub;
    if (total == 0) return BGB_OK;
    if (!obj || !lower || !upper || !out) return BGB_ERR_ARG;
    const int64_t want = (total + kLaThreads - 1) / kLaThreads;
    const int64_t cap = (int64_t)sm_count_la() * 32;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
#define BGB_LA_FWD(IM)                                                                          \
    log_areas_forward_kernel<T, IM><<<grid, kLaThreads, 0, st>>>(                               \
        obj, B, n_sub, (int)isz, (int)m, lower, upper, B_cells, nc, (T)tau_relu, (T)tau_max, out)
    switch (la_bucket(isz)) {
        case 4: BGB_LA_FWD(4); break;
        case 8: BGB_LA_FWD(8); break;
        case 16: BGB_LA_FWD(16); break;
        default: BGB_LA_FWD(32); break;
    }
#undef BGB_LA_FWD
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

template <typename T>
int log_areas_backward(const T* g_out, const T* obj, int64_t B, int64_t n_sub, int64_t isz,
                       int64_t m, const T* lower, const T* upper, int64_t B_cells, int64_t nc,
                       double tau_relu, double tau_max, T* g_obj, cudaStream_t st) {
    int rc = la_check(B, n_sub, isz, m, B_cells, nc, tau_relu, tau_max);
    if (rc) return rc;
    const int64_t rows = B * n_sub * m;  // (b, s, k) triples
    if (rows == 0) return BGB_OK;
    if (!obj || !g_obj) return BGB_ERR_ARG;
    if (nc == 0) {
        BGB_CUDA_TRY(cudaMemsetAsync(g_obj, 0, sizeof(T) * (size_t)(rows * isz), st));
        return BGB_OK;
    }
    if (!g_out || !lower || !upper) return BGB_ERR_ARG;
    // lanes per (b, s, k): grow while cells remain to split and the launch is
    // below ~4 waves of full occupancy
    const int64_t fill = (int64_t)sm_count_la() * 2048 * 4;
    int G = 1;
    while (G < 32 && G < nc && rows * G < fill) G <<= 1;
    const int64_t threads = rows * G;
    const int64_t blocks = (threads + kLaThreads - 1) / kLaThreads;
    if (blocks > 0x7fffffffLL) return BGB_ERR_UNSUPPORTED;
#define BGB_LA_BWD(IM)                                                                       \
    log_areas_backward_kernel<T, IM><<<(unsigned)blocks, kLaThreads, 0, st>>>(                 \
        g_out, obj, B, n_sub, (int)isz, (int)m, lower, upper, B_cells, nc, (T)tau_relu,       \
        (T)tau_max, G, g_obj)
    switch (la_bucket(isz)) {
        case 4: BGB_LA_BWD(4); break;
        case 8: BGB_LA_BWD(8); break;
        case 16: BGB_LA_BWD(16); break;
        default: BGB_LA_BWD(32); break;
    }
#undef BGB_LA_BWD
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

template <typename T>
int log_areas_forward_jac(const T* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                          const T* lower, const T* upper, int64_t B_cells, int64_t nc,
                          double tau_relu, double tau_max, T* out, T* jac, cudaStream_t st) {
    int rc = la_check(B, n_sub, isz, m, B_cells, nc, tau_relu, tau_max);
    if (rc) return rc;
    const int64_t total = B * nc * n_sub;
    if (total == 0) return BGB_OK;
    if (!obj || !lower || !upper || !out || !jac) return BGB_ERR_ARG;
    const int64_t want = (total + kLaThreads - 1) / kLaThreads;
    const int64_t cap = (int64_t)sm_count_la() * 32;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
#define BGB_LA_FJ(IM)                                                                           \
    log_areas_forward_jac_kernel<T, IM><<<grid, kLaThreads, 0, st>>>(                           \
        obj, B, n_sub, (int)isz, (int)m, lower, upper, B_cells, nc, (T)tau_relu, (T)tau_max,    \
        out, jac)
    switch (la_bucket(isz)) {
        case 4: BGB_LA_FJ(4); break;
        case 8: BGB_LA_FJ(8); break;
        case 16: BGB_LA_FJ(16); break;
        default: BGB_LA_FJ(32); break;
    }
#undef BGB_LA_FJ
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

template <typename T>
int log_areas_backward_jac(const T* g_out, const T* jac, int64_t B, int64_t n_sub, int64_t isz,
                           int64_t m, int64_t nc, T* g_obj, cudaStream_t st) {
    if (B < 0 || n_sub < 0 || nc < 0 || isz < 1 || m < 1) return BGB_ERR_ARG;
    if (isz > kLaMaxI || m > kLaMaxM) return BGB_ERR_UNSUPPORTED;
    const int64_t total = B * n_sub * isz * m;
    if (total == 0) return BGB_OK;
    if (!g_obj) return BGB_ERR_ARG;
    if (nc == 0) {
        BGB_CUDA_TRY(cudaMemsetAsync(g_obj, 0, sizeof(T) * (size_t)total, st));
        return BGB_OK;
    }
    if (!g_out || !jac) return BGB_ERR_ARG;
    const int64_t want = (total + kLaThreads - 1) / kLaThreads;
    const int64_t cap = (int64_t)sm_count_la() * 32;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    log_areas_backward_jac_kernel<T><<<grid, kLaThreads, 0, st>>>(g_out, jac, B, n_sub,
                                                                   (int)(isz * m), nc, g_obj);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

}  // namespace

}  // namespace bgb

extern "C" {

int bgb_log_areas_forward(const double* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                          const double* cell_lower, const double* cell_upper, int64_t B_cells,
                          int64_t nc, double tau_relu, double tau_max, double* out, void* stream) {
    return bgb::log_areas_forward<double>(obj, B, n_sub, isz, m, cell_lower, cell_upper, B_cells,
                                          nc, tau_relu, tau_max, out,
                                          static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_forward_f32(const float* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                              const float* cell_lower, const float* cell_upper, int64_t B_cells,
                              int64_t nc, double tau_relu, double tau_max, float* out,
                              void* stream) {
    return bgb::log_areas_forward<float>(obj, B, n_sub, isz, m, cell_lower, cell_upper, B_cells,
                                         nc, tau_relu, tau_max, out,
                                         static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_backward(const double* grad_out, const double* obj, int64_t B, int64_t n_sub,
                           int64_t isz, int64_t m, const double* cell_lower,
                           const double* cell_upper, int64_t B_cells, int64_t nc, double tau_relu,
                           double tau_max, double* grad_obj, void* stream) {
    return bgb::log_areas_backward<double>(grad_out, obj, B, n_sub, isz, m, cell_lower,
                                           cell_upper, B_cells, nc, tau_relu, tau_max, grad_obj,
                                           static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_backward_f32(const float* grad_out, const float* obj, int64_t B, int64_t n_sub,
                               int64_t isz, int64_t m, const float* cell_lower,
                               const float* cell_upper, int64_t B_cells, int64_t nc,
                               double tau_relu, double tau_max, float* grad_obj, void* stream) {
    return bgb::log_areas_backward<float>(grad_out, obj, B, n_sub, isz, m, cell_lower, cell_upper,
                                          B_cells, nc, tau_relu, tau_max, grad_obj,
                                          static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_forward_jac(const double* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                              const double* cell_lower, const double* cell_upper, int64_t B_cells,
                              int64_t nc, double tau_relu, double tau_max, double* out,
                              double* jac, void* stream) {
    return bgb::log_areas_forward_jac<double>(obj, B, n_sub, isz, m, cell_lower, cell_upper,
                                              B_cells, nc, tau_relu, tau_max, out, jac,
                                              static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_forward_jac_f32(const float* obj, int64_t B, int64_t n_sub, int64_t isz,
                                  int64_t m, const float* cell_lower, const float* cell_upper,
                                  int64_t B_cells, int64_t nc, double tau_relu, double tau_max,
                                  float* out, float* jac, void* stream) {
    return bgb::log_areas_forward_jac<float>(obj, B, n_sub, isz, m, cell_lower, cell_upper,
                                             B_cells, nc, tau_relu, tau_max, out, jac,
                                             static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_backward_jac(const double* grad_out, const double* jac, int64_t B,
                               int64_t n_sub, int64_t isz, int64_t m, int64_t nc,
                               double* grad_obj, void* stream) {
    return bgb::log_areas_backward_jac<double>(grad_out, jac, B, n_sub, isz, m, nc, grad_obj,
                                               static_cast<cudaStream_t>(stream));
}

int bgb_log_areas_backward_jac_f32(const float* grad_out, const float* jac, int64_t B,
                                   int64_t n_sub, int64_t isz, int64_t m, int64_t nc,
                                   float* grad_obj, void* stream) {
    return bgb::log_areas_backward_jac<float>(grad_out, jac, B, n_sub, isz, m, nc, grad_obj,
                                              static_cast<cudaStream_t>(stream));
}

}  // extern "C"
