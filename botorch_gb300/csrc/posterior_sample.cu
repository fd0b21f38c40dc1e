// Reparameterised samples of a batched multivariate normal posterior (float64):
// the sample step of GPyTorchPosterior.rsample_from_base_samples
// (botorch/posteriors/gpytorch.py:86-127 -> gpytorch MultivariateNormal.rsample).
//
// One CTA per batch member: L = psd_safe_cholesky(covar) (plain, then jitter
// 1e-8 x 10^t added to the diagonal for t < max_tries, for this member only, as
// linear_operator does for the failing members of a batch), then
//   samples[s][b][i] = mean[b][i] + sum_{j <= i} L[i][j] Z[s][j]
// with the base samples Z (S x q) shared by every member (the reference's
// collapsed batch dimensions of the base sample shape).
#include <math.h>

#include "bgb_common.cuh"

namespace {

constexpr int kSampleThreads = 256;

// In-place Cholesky of a q x q row-major matrix (lower) by one thread;
// 0 on success, else the 1-based failing pivot.
__device__ int chol_serial(double* A, int q) {
    for (int j = 0; j < q; ++j) {
        double v = A[j * q + j];
        for (int k = 0; k < j; ++k) v -= A[j * q + k] * A[j * q + k];
        if (!(v > 0.0)) return j + 1;
        const double djj = sqrt(v);
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

__global__ void __launch_bounds__(kSampleThreads) mvn_sample_kernel(
    const double* __restrict__ mean, const double* __restrict__ covar, int64_t b, int q,
    const double* __restrict__ Z, int S, int max_tries, double jitter,
    double* __restrict__ samples, int32_t* __restrict__ status) {
    extern __shared__ double sm[];
    double* A = sm;           // q x q: the covariance
    double* Lf = A + q * q;   // q x q: its (jittered) factor
    __shared__ int s_status;
    const int64_t bi = blockIdx.x;
    const double* C = covar + bi * q * q;
    for (int p = threadIdx.x; p < q * q; p += blockDim.x) A[p] = C[p];
    __syncthreads();
    if (threadIdx.x == 0) {
        bool has_nan = false;
        for (int p = 0; p < q * q; ++p) has_nan |= isnan(A[p]);
        int st = BGB_NAN;
        if (!has_nan) {
            st = BGB_NOT_PSD;
            for (int t = -1; t < max_tries; ++t) {
                const double jit = t < 0 ? 0.0 : jitter * pow(10.0, (double)t);
                for (int p = 0; p < q * q; ++p) Lf[p] = A[p] + ((p % (q + 1)) == 0 ? jit : 0.0);
                if (chol_serial(Lf, q) == 0) {
                    st = BGB_OK;
                    break;
                }
            }
        }
        s_status = st;
        status[bi] = st;
    }
    __syncthreads();
    if (s_status != BGB_OK) {
        for (int64_t p = threadIdx.x; p < (int64_t)S * q; p += blockDim.x) {
            const int64_t s = p / q, i = p % q;
            samples[(s * b + bi) * q + i] = NAN;
        }
        return;
    }
    const double* mu = mean + bi * q;
    for (int64_t p = threadIdx.x; p < (int64_t)S * q; p += blockDim.x) {
        const int64_t s = p / q;
        const int i = (int)(p % q);
        const double* z = Z + s * q;
        double y = mu[i];
        for (int j = 0; j <= i; ++j) y += Lf[i * q + j] * z[j];
        samples[(s * b + bi) * q + i] = y;
    }
}

}  // namespace

extern "C" int bgb_mvn_rsample(const double* mean, const double* covar, int64_t b, int32_t q,
                               const double* Z, int32_t S, int32_t max_tries, double* samples,
                               int32_t* status, void* stream) {
    if (mean == nullptr || covar == nullptr || Z == nullptr || samples == nullptr ||
        status == nullptr || b < 0 || q <= 0 || S <= 0 || max_tries < 0)
        return BGB_ERR_ARG;
    if (q > 64) return BGB_ERR_UNSUPPORTED;  // two q x q float64 blocks in shared memory
    if (b == 0) return BGB_OK;
    const size_t smem = 2 * sizeof(double) * (size_t)q * q;
    mvn_sample_kernel<<<(unsigned)b, kSampleThreads, smem, reinterpret_cast<cudaStream_t>(stream)>>>(
        mean, covar, b, q, Z, S, max_tries, 1e-8, samples, status);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
