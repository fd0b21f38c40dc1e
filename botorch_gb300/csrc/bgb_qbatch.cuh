// Arguments of the per-t-batch kernels (device pointers, float64 unless noted).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace bgb {

constexpr int kMaxQ = 32;  // largest q of the fused per-batch kernel

struct QBatchArgs {
    int64_t b;          // t-batches
    int64_t n;          // training points
    int q, r, S, d;
    int kernel;
    int acqf;
    int max_tries;
    double jitter;      // first jitter of psd_safe_cholesky (float64: 1e-8)
    double outputscale, mean_constant, y_mean, y_std;
    double tau_relu, tau_max;
    // per-call constants computed once on the host (float64 is slow per CTA):
    // 1 / tau_relu, log(tau_relu) and 1 / tau_max as floats, log(S), sqrt(outputscale)
    float inv_tau_relu_f, log_tau_relu_f, inv_tau_max_f;
    double log_S, sqrt_outputscale;
    const double* X;        // b*q x d candidates
    const double* Xt;       // n x d training inputs
    const double* Xb;       // r x d baseline
    const double* inv_ls;   // d
    const double* Lb_inv;   // r x r
    const double* Z;        // S x (r+q)
    const double* best_f;   // S (qLogNEI) or 1 (qEI)
    // intermediates (standardised space)
    double* sig;            // b x q x q
    double* sqb;            // b x q x r
    double* mu;             // b x q
    double* gqq;            // b x q x q   d value / d Sigma_qq (standardised)
    double* gqb;            // b x q x r
    double* gmu;            // b x q
    // outputs
    double* value;          // b
    double* grad;           // b x q x d
    int32_t* status;        // b
    const int* dev_err;     // non-zero: a bounded wait in a tensor-core GEMM expired
    float* zt;              // mixed: candidates scaled by 1 / lengthscale, d x (b*q), k-major
    float* z32;             // mixed: Z in float32 (S x (r+q))
    float* bf32;            // mixed: best_f per sample as float (hi, lo) pairs (S x 2)
    double beta_absmax;     // max |beta| (row-scale bound of the float16 adjoint operand)
    int adj_ctas_per_sm;    // adjoint slab split target (0: default)
    float* hmul;            // tensor cores: b*q inverse row scales of the float16 H
    // joint sampling (the reference's fallback to full joint sampling, and
    // cache_root=False): psd_safe_cholesky of the whole (r+q) x (r+q) covariance
    // per t-batch, level t adding j_t (0, then jitter 10^(t-1)) to its diagonal
    int joint;              // 0: cached root; 1: joint, cached best_f; 2: joint, best_f per level
    const double* Lb_inv_lv;  // (max_tries+1) x r x r: chol(Sigma_bb + j_t I)^-1, NaN at [0] if it failed
    const double* best_f_lv;  // (max_tries+1) x S: max over the baseline of the level's samples
};

// ---------------------------------------------------------------- grouped launches
// One stage of many models in one launch: CTA blockIdx.x belongs to model m with
// off[m] <= blockIdx.x < off[m + 1] (off: nm + 1 prefix sums in device memory);
// args: the models' argument structs (one of the *G structs below) in device memory.
struct GroupTab {
    int nm;
    const int* off;
    const void* args;
};

template <typename T>
struct QstatsG {
    QBatchArgs a;
    const T* V;
    int64_t ldv;
    const T* beta;
    const T* Vb;
    int vec_ok;
};
struct BstepG {
    QBatchArgs a;
    int backward;
};
template <typename T>
struct MixG {
    QBatchArgs a;
    const T* V;
    int64_t ldv;
    const T* Vb;
    const T* beta;
    T* H;
    __half* H16;
    __half* H16_lo;
    int64_t ldh;
    int64_t gx;  // column groups per t-batch
};
template <typename T>
struct AdjG {
    QBatchArgs a;
    const T* D;
    int64_t ldd;
    const T* XsT;
    int64_t slab;
    T* part;     // nullptr: a single slab
    int64_t gx;  // row blocks
    int nslab;
};

// kernel build of one model: zt = (X / lengthscale)^T (d x rows, float32), then
// K(X, Xt) as the float16 split (K16, K16_lo, ldk) of k16_scale * K
struct KmG {
    const double* X;
    const double* inv_ls;
    float* zt;
    int64_t rows;
    int d;
    int kind;
    const float* Xs32;  // training inputs / lengthscale, d x n
    int64_t n;
    double outputscale;
    __half* K16;
    __half* K16_lo;
    float k16_scale;
    int64_t ldk;
    int64_t gx;  // column tiles
};
int64_t kernel_matrix_col_tiles(int64_t n);
int64_t kernel_matrix_row_tiles(int64_t m);
// scale (rows * d elements per model, 256 per CTA) then the kernel build
int launch_kernel_matrix_group(const GroupTab& t_scale, int64_t total_scale, const GroupTab& t_km,
                               int64_t total_km, cudaStream_t stream);

// Sizes the standalone launchers use, shared with the grouped ones.
int64_t mix_rows_groups(const QBatchArgs& a, int E, int64_t total_b);
size_t mix_rows_smem_bytes(const QBatchArgs& a);
// adjoint split: row blocks, slabs and slab length for part_cap partial elements
void adjoint_split(const QBatchArgs& a, int64_t part_cap, int64_t* row_blocks, int64_t* nslab,
                   int64_t* slab);
size_t batch_step_f32_smem(int q, int r, int S);
int launch_prep_samples(const QBatchArgs& a, cudaStream_t stream);

// Grouped launchers (float32 path, total = off[nm] CTAs); qmax / rmax / dmax: the
// largest q / r / d of the group's models.
int launch_qstats_group(const GroupTab& t, int qmax, int rmax, int64_t total, cudaStream_t stream);
int launch_batch_step_group(const GroupTab& t, int qmax, size_t smem, int64_t total,
                            cudaStream_t stream);
int launch_mix_rows_group(const GroupTab& t, int qmax, size_t smem, int64_t total,
                          cudaStream_t stream);
int launch_adjoint_group(const GroupTab& t, int dmax, bool partials, int64_t total,
                         cudaStream_t stream);
// per model: sum the slabs of part (d x b*q elements), then finish the rows
int launch_adjoint_finish_group(const GroupTab& t_sum, int64_t total_sum, const GroupTab& t_fin,
                                int dmax, int64_t total_fin, cudaStream_t stream);

// mu, Sigma_qq and Sigma_qb in one pass over V (q <= 8, r <= 4); returns
// BGB_ERR_UNSUPPORTED (nothing launched) outside those sizes.
template <typename T>
int launch_qstats(const QBatchArgs& a, const T* V, int64_t ldv, const T* beta, const T* Vb,
                  cudaStream_t stream);
// the same outputs for q <= 32 from shared-memory tiles of V (BGB_ERR_UNSUPPORTED,
// nothing launched, beyond its output count or shared memory); scratch holds the
// float64 partial sums when few t-batches split their columns over CTAs
template <typename T>
int launch_qstats_tile(const QBatchArgs& a, const T* V, int64_t ldv, const T* beta, const T* Vb,
                       void* scratch, size_t scratch_bytes, cudaStream_t stream);
// mu (into a.mu) = m + V beta and P (b*q x r) = V Vb^T
template <typename T>
int launch_row_dots(const QBatchArgs& a, const T* V, int64_t ldv, const T* beta, const T* Vb, T* P,
                    cudaStream_t stream);
// P: b*q x r (V Vb^T) or null when r = 0; C: b*q x ldc holding V.
template <typename T>
int launch_sigma_reduce(const QBatchArgs& a, const T* P, const T* C, int64_t ldc,
                        cudaStream_t stream);
// mixed: float32 evaluation of the per-sample smooth reductions (see qbatch_impl.cuh)
int launch_batch_step(const QBatchArgs& a, int backward, cudaStream_t stream, bool mixed = false);
size_t batch_step_smem_bytes(int q, int r, int S);
// H (b*q x n) = gmu beta^T - 2 Gqq V - Gqb Vb per t-batch
// H16 non-null (float32 only): write H as the row-scaled float16 hi/lo split
// (H16, H16_lo, leading dimension ldh) with the inverse row scales in a.hmul.
template <typename T>
int launch_mix_rows(const QBatchArgs& a, const T* V, int64_t ldv, const T* Vb, const T* beta, T* H,
                    cudaStream_t stream, __half* H16 = nullptr, __half* H16_lo = nullptr,
                    int64_t ldh = 0);
// d value / d X from D (b*q x n) = H L^-1; XsT: training inputs scaled by 1 / lengthscale,
// d x n (k-major). part: scratch of part_cap elements for per-slab partial
// gradients (nullptr / 0: a single slab, no finalize pass).
template <typename T>
int launch_adjoint(const QBatchArgs& a, const T* D, int64_t ldd, const T* XsT, T* part,
                   int64_t part_cap, cudaStream_t stream);
int launch_posterior_out(const QBatchArgs& a, double* mean, double* covar, cudaStream_t stream);

}  // namespace bgb
