// Initialisation-time entry points of qLogNEI (float64): the joint posterior
// over a point set, baseline pruning counts and the cached baseline root.
#include <math.h>
#include <string.h>

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

using namespace bgb;

namespace {

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

__global__ void affine_kernel(const double* x, double* y, int64_t n, double a, double b) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a + b * x[i];
}
__global__ void scale_kernel(double* x, int64_t n, double s) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= s;
}

// One CTA per sample row: value and first index of the row maximum of
// (mean + samples[row]); counts[argmax] += 1. NaN rows count nothing.
__global__ void argmax_count_kernel(const double* samples, const double* mean, int64_t m,
                                    int32_t* counts) {
    const int64_t row = blockIdx.x;
    double best = -INFINITY;
    int64_t bi = -1;
    for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
        double v = samples[row * m + j] + mean[j];
        if (v == v && (bi < 0 || v > best)) {  // j increases: the first maximum wins
            best = v;
            bi = j;
        }
    }
    __shared__ double sv[256];
    __shared__ int64_t si[256];
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            double ov = sv[threadIdx.x + s];
            int64_t oi = si[threadIdx.x + s];
            if (oi >= 0 && (si[threadIdx.x] < 0 || ov > sv[threadIdx.x] ||
                            (ov == sv[threadIdx.x] && oi < si[threadIdx.x]))) {
                sv[threadIdx.x] = ov;
                si[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && si[0] >= 0) atomicAdd(&counts[si[0]], 1);
}

// best_f[s] = max_j (mean[j] + samples[s, j])
__global__ void row_max_kernel(const double* samples, const double* mean, int64_t S, int64_t m,
                               double* out) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    double best = -INFINITY;
    for (int64_t j = 0; j < m; ++j) best = fmax(best, samples[s * m + j] + mean[j]);
    out[s] = best;
}

size_t joint_ws(int64_t n, int64_t m) { return 2 * align_up(sizeof(double) * m * n); }

int posterior_joint(const bgb_gp_t* gp, const double* Linv, const double* alpha, const double* X,
                    int64_t m, double* mean, double* covar, Arena* ar, cudaStream_t st) {
    const int64_t n = gp->n;
    double* Kc = ar->take<double>(m * n);
    double* V = ar->take<double>(m * n);
    if (Kc == nullptr || V == nullptr) return BGB_ERR_WORKSPACE;
    int rc = launch_kernel_matrix<double, double, double>(X, m, gp->train_X, n, gp->d,
                                                          gp->inv_lengthscale, gp->outputscale,
                                                          gp->kernel, 0.0, 0, Kc, n, st);
    if (rc) return rc;
    // V = Kc L^-T (root-inverse form of the predictive covariance)
    rc = gemm_f64(m, n, n, 1.0, Kc, n, 0, Linv, n, 1, 0.0, V, n, KB_UPPER, 0, nullptr, st, n);
    if (rc) return rc;
    rc = launch_kernel_matrix<double, double, double>(X, m, X, m, gp->d, gp->inv_lengthscale,
                                                      gp->outputscale, gp->kernel, 0.0, 1, covar,
                                                      m, st);
    if (rc) return rc;
    rc = gemm_f64(m, m, n, -1.0, V, n, 0, V, n, 1, 1.0, covar, m, KFULL, 0, nullptr, st);
    if (rc) return rc;
    scale_kernel<<<(unsigned)ceil_div(m * m, 256), 256, 0, st>>>(covar, m * m,
                                                                gp->y_std * gp->y_std);
    BGB_CHECK_LAUNCH();
    rc = gemv_f64(m, n, 1.0, Kc, n, alpha, 0.0, mean, st);
    if (rc) return rc;
    affine_kernel<<<(unsigned)ceil_div(m, 256), 256, 0, st>>>(
        mean, mean, m, gp->y_mean + gp->y_std * gp->mean_constant, gp->y_std);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int valid_gp(const bgb_gp_t* gp) {
    return gp != nullptr && gp->n > 0 && gp->d > 0 && gp->train_X != nullptr &&
           gp->inv_lengthscale != nullptr && gp->kernel >= BGB_KERNEL_MATERN52 &&
           gp->kernel <= BGB_KERNEL_RBF;
}

}  // namespace

extern "C" {

size_t bgb_posterior_joint_workspace_bytes(int64_t n, int64_t m) { return joint_ws(n, m); }

int bgb_posterior_joint(const bgb_gp_t* gp, const double* Linv, const double* alpha,
                        const double* X, int64_t m, double* mean, double* covar, void* workspace,
                        size_t workspace_bytes, void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || alpha == nullptr || X == nullptr || mean == nullptr ||
        covar == nullptr || m <= 0)
        return BGB_ERR_ARG;
    if (workspace == nullptr || workspace_bytes < joint_ws(gp->n, m)) return BGB_ERR_WORKSPACE;
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    return posterior_joint(gp, Linv, alpha, X, m, mean, covar, &ar, as_stream(stream));
}

size_t bgb_prune_counts_workspace_bytes(int64_t n, int64_t m, int32_t S) {
    return joint_ws(n, m) + align_up(sizeof(double) * m) + 2 * align_up(sizeof(double) * m * m) +
           bgb_cholesky_workspace_bytes(m) + align_up(sizeof(double) * (int64_t)S * m);
}

int bgb_prune_counts(const bgb_gp_t* gp, const double* Linv, const double* alpha, const double* X,
                     int64_t m, const double* Z, int32_t S, int32_t max_tries, int32_t* counts,
                     void* workspace, size_t workspace_bytes, void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || alpha == nullptr || X == nullptr || Z == nullptr ||
        counts == nullptr || m <= 0 || S <= 0)
        return BGB_ERR_ARG;
    if (workspace == nullptr || workspace_bytes < bgb_prune_counts_workspace_bytes(gp->n, m, S))
        return BGB_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    double* mean = ar.take<double>(m);
    double* covar = ar.take<double>(m * m);
    double* L = ar.take<double>(m * m);
    void* cws = ar.take<char>(bgb_cholesky_workspace_bytes(m));
    double* samples = ar.take<double>((int64_t)S * m);
    int rc = posterior_joint(gp, Linv, alpha, X, m, mean, covar, &ar, st);
    if (rc) return rc;
    rc = bgb_psd_safe_cholesky(covar, m, m, L, m, max_tries, 1e-8, nullptr, cws,
                               bgb_cholesky_workspace_bytes(m), stream);
    if (rc) return rc;
    rc = gemm_f64(S, m, m, 1.0, Z, m, 0, L, m, 1, 0.0, samples, m, KFULL, 0, nullptr, st);
    if (rc) return rc;
    BGB_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int32_t) * m, st));
    argmax_count_kernel<<<(unsigned)S, 256, 0, st>>>(samples, mean, m, counts);
    BGB_CHECK_LAUNCH();
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    return BGB_OK;
}

size_t bgb_qlognei_baseline_workspace_bytes(int64_t n, int32_t r, int32_t S) {
    return joint_ws(n, r) + align_up(sizeof(double) * r) + align_up(sizeof(double) * r * r) +
           bgb_cholesky_workspace_bytes(r) + bgb_tri_inverse_workspace_bytes(r) +
           align_up(sizeof(double) * (int64_t)S * r);
}

int bgb_qlognei_baseline(const bgb_gp_t* gp, const double* Linv, const double* alpha,
                         const double* X_baseline, int32_t r, const double* Zb, int32_t S,
                         int32_t max_tries, double* Lb, double* Lb_inv, double* best_f,
                         double* jitter_host, void* workspace, size_t workspace_bytes,
                         void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || alpha == nullptr || X_baseline == nullptr ||
        Zb == nullptr || Lb == nullptr || Lb_inv == nullptr || best_f == nullptr || r <= 0 ||
        S <= 0)
        return BGB_ERR_ARG;
    if (workspace == nullptr ||
        workspace_bytes < bgb_qlognei_baseline_workspace_bytes(gp->n, r, S))
        return BGB_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    double* mean = ar.take<double>(r);
    double* covar = ar.take<double>((int64_t)r * r);
    void* cws = ar.take<char>(bgb_cholesky_workspace_bytes(r));
    double* tws = ar.take<double>(bgb_tri_inverse_workspace_bytes(r) / sizeof(double));
    double* samples = ar.take<double>((int64_t)S * r);
    int rc = posterior_joint(gp, Linv, alpha, X_baseline, r, mean, covar, &ar, st);
    if (rc) return rc;
    rc = bgb_psd_safe_cholesky(covar, r, r, Lb, r, max_tries, 1e-8, jitter_host, cws,
                               bgb_cholesky_workspace_bytes(r), stream);
    if (rc) return rc;
    rc = copy_matrix_f64(Lb, r, Lb_inv, r, r, r, 0.0, st);
    if (rc) return rc;
    rc = tri_inverse_f64(Lb_inv, r, r, tws, st);
    if (rc) return rc;
    rc = gemm_f64(S, r, r, 1.0, Zb, r, 0, Lb, r, 1, 0.0, samples, r, KFULL, 0, nullptr, st);
    if (rc) return rc;
    row_max_kernel<<<(unsigned)ceil_div(S, 128), 128, 0, st>>>(samples, mean, S, r, best_f);
    BGB_CHECK_LAUNCH();
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    return BGB_OK;
}

size_t bgb_qlognei_joint_levels_workspace_bytes(int64_t n, int32_t r, int32_t S) {
    return joint_ws(n, r) + align_up(sizeof(double) * r) + 2 * align_up(sizeof(double) * r * r) +
           bgb_cholesky_workspace_bytes(r) + bgb_tri_inverse_workspace_bytes(r) +
           align_up(sizeof(double) * (int64_t)S * r);
}

int bgb_qlognei_joint_levels(const bgb_gp_t* gp, const double* Linv, const double* alpha,
                             const double* X_baseline, int32_t r, const double* Zb, int32_t S,
                             double* Lb_inv_lv, double* best_f_lv, void* workspace,
                             size_t workspace_bytes, void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || alpha == nullptr || X_baseline == nullptr ||
        Zb == nullptr || Lb_inv_lv == nullptr || best_f_lv == nullptr || r <= 0 || S <= 0)
        return BGB_ERR_ARG;
    if (workspace == nullptr ||
        workspace_bytes < bgb_qlognei_joint_levels_workspace_bytes(gp->n, r, S))
        return BGB_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    double* mean = ar.take<double>(r);
    double* covar = ar.take<double>((int64_t)r * r);
    double* L = ar.take<double>((int64_t)r * r);
    void* cws = ar.take<char>(bgb_cholesky_workspace_bytes(r));
    double* tws = ar.take<double>(bgb_tri_inverse_workspace_bytes(r) / sizeof(double));
    double* samples = ar.take<double>((int64_t)S * r);
    int rc = posterior_joint(gp, Linv, alpha, X_baseline, r, mean, covar, &ar, st);
    if (rc) return rc;
    constexpr int kLevels = 7;  // plain, then jitter 1e-8 x 10^t for t < 6 (botorch/__init__.py:54)
    for (int t = 0; t < kLevels; ++t) {
        const double jit = t == 0 ? 0.0 : 1e-8 * pow(10.0, (double)(t - 1));
        double* Li = Lb_inv_lv + (int64_t)t * r * r;
        double* bf = best_f_lv + (int64_t)t * S;
        rc = copy_matrix_f64(covar, r, L, r, r, r, jit, st);
        if (rc) return rc;
        int32_t info = 0;
        rc = bgb_cholesky(L, r, r, &info, cws, bgb_cholesky_workspace_bytes(r), stream);
        if (rc == BGB_NOT_PSD) {
            // all-ones bytes are a NaN pattern: marks the level as failed
            BGB_CUDA_TRY(cudaMemsetAsync(Li, 0xFF, sizeof(double) * r * r, st));
            BGB_CUDA_TRY(cudaMemsetAsync(bf, 0xFF, sizeof(double) * S, st));
            continue;
        }
        if (rc) return rc;
        rc = copy_matrix_f64(L, r, Li, r, r, r, 0.0, st);
        if (rc) return rc;
        rc = tri_inverse_f64(Li, r, r, tws, st);
        if (rc) return rc;
        rc = gemm_f64(S, r, r, 1.0, Zb, r, 0, L, r, 1, 0.0, samples, r, KFULL, 0, nullptr, st);
        if (rc) return rc;
        row_max_kernel<<<(unsigned)ceil_div(S, 128), 128, 0, st>>>(samples, mean, S, r, bf);
        BGB_CHECK_LAUNCH();
    }
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    return BGB_OK;
}

}  // extern "C"
