/*
 * botorch_gb300 — C ABI of the GB300 (sm_103a) GP-posterior + Monte-Carlo
 * acquisition path.
 *
 * The reference (BoTorch 0.18.1) has no C/C++ interface for this path: it is
 * reached through Python classes. Each entry point below replaces one step of
 * that Python path and says which reference code it stands in for. All
 * pointers are DEVICE pointers unless marked "host". Matrices are row-major
 * with the stated leading dimension. Every call is asynchronous on `stream`
 * (a cudaStream_t passed as void*) unless it says it synchronises; scratch
 * memory is the caller's `workspace` (size from the matching *_bytes query);
 * nothing here allocates device memory.
 *
 * Return codes: BGB_OK (0); positive values are numerical conditions
 * (BGB_NOT_PSD, BGB_NAN) that the Python layer maps to the reference's
 * NotPSDError / NanError; negative values are argument or launch errors.
 */
#ifndef BOTORCH_GB300_H
#define BOTORCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BGB_OK 0
#define BGB_NOT_PSD 1          /* psd_safe_cholesky gave up (linear_operator NotPSDError) */
#define BGB_NAN 2              /* NaN input / non-finite samples (linear_operator NanError) */
#define BGB_DEVICE_TIMEOUT 3   /* a bounded wait inside a tensor-core GEMM expired */
#define BGB_ERR_ARG (-1)       /* invalid size, pointer or option */
#define BGB_ERR_WORKSPACE (-2) /* workspace smaller than the *_bytes query */
#define BGB_ERR_CUDA (-3)      /* a CUDA launch or runtime call failed */
#define BGB_ERR_UNSUPPORTED (-4)
#define BGB_ERR_SCRATCH_LIMIT (-5) /* call needs more than BGB_NOALLOC_SCRATCH_BYTES of scratch */

/* Stationary kernels (gpytorch ScaleKernel over MaternKernel(nu) / RBFKernel, ARD). */
#define BGB_KERNEL_MATERN52 0
#define BGB_KERNEL_MATERN32 1
#define BGB_KERNEL_MATERN12 2
#define BGB_KERNEL_RBF 3

/* Arithmetic of the per-call path. FP64: every step in float64 (the plain
 * FP64 GPU path). MIXED: kernel build, row mix and adjoint in float32, the
 * cross-covariance GEMMs on float16 hi/lo splits with float32 accumulation
 * (tensor cores) or in float32 (BGB_FLAG_SIMT); the q x q algebra (Sigma
 * assembly, psd_safe_cholesky, its adjoint) and every sum across tiles, lanes,
 * samples and slabs in float64 or compensated float32; per-sample improvements
 * in float32 from exact float pairs of mu and best_f. */
#define BGB_PREC_FP64 0
#define BGB_PREC_MIXED 1

#define BGB_ACQF_QEI 0
#define BGB_ACQF_QLOGNEI 1

/* bgb_acq_t.flags */
#define BGB_FLAG_SIMT 1        /* MIXED: use the FFMA GEMM even when tensor-core operands are set */
/* bits 8-15: CTAs per SM the adjoint contraction aims for when it splits the
 * training points into slabs (0: 16); a schedule knob for autotuners */
#define BGB_FLAG_ADJ_CTAS_SHIFT 8
#define BGB_FLAG_ADJ_CTAS_MASK 0xFF00
/* qLogNEI sampling without the cached root (needs Lb_inv_lv, from
 * bgb_qlognei_joint_levels): the q new rows of the Cholesky factor of the whole
 * (r+q) x (r+q) joint covariance, psd_safe_cholesky jitter applied to the whole
 * diagonal per t-batch.
 * JOINT_SAMPLING: best_f stays the cached baseline incumbent -- the reference's
 *   fallback to standard sampling when the low-rank update fails
 *   (botorch/acquisition/cached_cholesky.py:143-158);
 * UNCACHED_ROOT (with JOINT_SAMPLING): best_f from the joint draw's own baseline
 *   samples (needs best_f_lv) -- qLogNoisyExpectedImprovement(cache_root=False)
 *   (botorch/acquisition/logei.py:543-553, acquisition/utils.py:97-141). */
#define BGB_FLAG_JOINT_SAMPLING 2
#define BGB_FLAG_UNCACHED_ROOT 4

/* An exact GP with fixed hyperparameters (SingleTaskGP, gp_regression.py:108-214).
 * Hyperparameters live in the standardised outcome space; y_mean / y_std
 * undo the Standardize outcome transform (transforms/outcome.py:431-511). */
typedef struct bgb_gp {
    int64_t n;                     /* training points */
    int32_t d;                     /* input dimension */
    int32_t kernel;                /* BGB_KERNEL_* */
    double outputscale;            /* sigma_f^2 */
    double mean_constant;          /* constant prior mean */
    double y_mean;                 /* Standardize offset */
    double y_std;                  /* Standardize scale */
    const double* train_X;         /* n x d */
    const double* inv_lengthscale; /* d: 1 / lengthscale */
} bgb_gp_t;

/* Everything one acquisition call needs besides the candidates.
 * With L the Cholesky factor of K = K(Xt,Xt) + noise I:
 *   B (n x ldb)  L^-T: right operand of the cross-covariance GEMM
 *                V = K(X,Xt) L^-T (the reference's root-inverse form of the
 *                predictive covariance: Sigma = K(X,X) - V V^T);
 *   Linv (n x n) L^-1, right operand of the adjoint GEMM dK = (d value / d V) L^-1;
 *   beta (n)     L^-1 (y - m), so that the mean is m + V beta;
 *   Vb (r x n)   K(X_baseline, Xt) L^-T and VbT (n x r) its transpose.
 * (built by bgb_gp_operands and bgb_baseline_operands). The *32 copies are
 * used by BGB_PREC_MIXED, the *64 ones by BGB_PREC_FP64. */
typedef struct bgb_acq {
    bgb_gp_t gp;
    int32_t acqf;            /* BGB_ACQF_* */
    int32_t precision;       /* BGB_PREC_* */
    int32_t q;               /* points per t-batch */
    int32_t r;               /* baseline points (0 for qEI) */
    int32_t n_samples;       /* MC samples S */
    int32_t flags;           /* BGB_FLAG_* */
    int64_t ldb;             /* leading dimension of B, >= n */
    const double* B64;
    const float* B32;
    const double* Linv64;
    const float* Linv32;
    const double* Vb64;
    const float* Vb32;
    const double* VbT64;
    const float* VbT32;
    const double* beta64;
    const float* beta32;
    const double* Xs64;      /* d x n (k-major): training inputs / lengthscale (adjoint) */
    const float* Xs32;
    /* tensor-core operands of MIXED (IEEE binary16 bit patterns, n x ldl,
     * ldl >= n, ldl % 8 == 0; from bgb_gp_tc_operands): the scaled float16
     * hi/lo split of L^-1 for the forward GEMM and of L^-T for the adjoint
     * GEMM, with the inverse row scales; NULL: FFMA GEMM */
    const uint16_t* Lhi;
    const uint16_t* Llo;
    const uint16_t* LThi;
    const uint16_t* LTlo;
    const float* Lmul;       /* n: 1 / scale of row j of L^-1 */
    const float* LTmul;      /* n: 1 / scale of row j of L^-T */
    int64_t ldl;
    double beta_absmax;      /* max_j |beta_j| (bounds the adjoint GEMM's rows) */
    const double* X_baseline;/* r x d */
    const double* Lb_inv;    /* r x r: inverse of the Cholesky factor of the
                                untransformed baseline posterior covariance */
    const double* Z;         /* S x (r+q) base samples */
    const double* best_f;    /* S values (qLogNEI) or 1 value (qEI) */
    double tau_relu;         /* logei.py:67 */
    double tau_max;          /* logei.py:68 */
    const double* Lb_inv_lv; /* 7 x r x r (BGB_FLAG_JOINT_SAMPLING): per jitter level, from
                                bgb_qlognei_joint_levels */
    const double* best_f_lv; /* 7 x S (BGB_FLAG_UNCACHED_ROOT) */
} bgb_acq_t;

/* Library version (major * 10000 + minor * 100 + patch). */
int bgb_version(void);

/* (a) Kernel matrix K[i,j] = outputscale * kappa(|(X1_i - X2_j) / l|^2)
 *     (+ diag_add on i == j when X1 and X2 are the same pointer).
 * Replaces the evaluation of the covariance module in SingleTaskGP.forward
 * (botorch/models/gp_regression.py:209-214; gpytorch MaternKernel/RBFKernel). */
int bgb_kernel_matrix(const bgb_gp_t* gp, const double* X1, int64_t m, const double* X2,
                      int64_t n2, double diag_add, double* K, int64_t ldk, void* stream);

/* (b) Blocked Cholesky of one SPD matrix in place (lower factor; the strict
 * upper triangle is zeroed). On failure *info_host = first failing pivot
 * (1-based) and BGB_NOT_PSD is returned. Synchronises `stream`.
 * Replaces torch.linalg.cholesky_ex inside linear_operator's psd_safe_cholesky. */
int bgb_cholesky(double* A, int64_t n, int64_t lda, int32_t* info_host, void* workspace,
                 size_t workspace_bytes, void* stream);
size_t bgb_cholesky_workspace_bytes(int64_t n);

/* (b) psd_safe_cholesky for one matrix: plain factorisation, then jitter
 * j * 10^i added to the diagonal for i < max_tries (j = 1e-8 when jitter <= 0).
 * `A` is preserved; the factor goes to `L` (ldl). *jitter_host = total jitter.
 * Synchronises `stream`. Replaces linear_operator psd_safe_cholesky as called
 * by the exact prediction strategy, cached_cholesky.py:98-124 and
 * low_rank.py:137-140. */
int bgb_psd_safe_cholesky(const double* A, int64_t n, int64_t lda, double* L, int64_t ldl,
                          int32_t max_tries, double jitter, double* jitter_host,
                          void* workspace, size_t workspace_bytes, void* stream);

/* (b) Lower-triangular inverse in place (recursive: 64 x 64 diagonal blocks,
 * then pairs of adjacent blocks joined level by level with batched float64
 * GEMMs). The upper triangle of L is set to zero. */
int bgb_tri_inverse(double* L, int64_t n, int64_t lda, void* workspace, size_t workspace_bytes,
                    void* stream);
size_t bgb_tri_inverse_workspace_bytes(int64_t n);

/* (b) Exact-GP training cache: L = psd_safe_cholesky(K + noise I), Linv = L^-1
 * (recursive triangular inverse), alpha = K^-1 (y - mean_constant) = L^-T L^-1
 * (y - m) with one step of iterative refinement, and beta = L^T alpha. y is the
 * standardised training target (n). Synchronises `stream`. Replaces the
 * training-side caches of gpytorch's exact prediction strategy (mean cache and
 * root-inverse cache) under the settings of botorch/__init__.py:51-56. */
int bgb_gp_fit(const bgb_gp_t* gp, const double* y, double noise, int32_t max_tries,
               double* L, double* Linv, double* alpha, double* beta, double* jitter_host,
               void* workspace, size_t workspace_bytes, void* stream);
size_t bgb_gp_fit_workspace_bytes(int64_t n);

/* (a3) Exact marginal log-likelihood of the standardised training targets y (n)
 * and its gradient w.r.t. the hyperparameters, float64, from the training cache
 * of bgb_gp_fit (L, Linv, alpha): out_host (host, d + 4 doubles) = [mll / n,
 * d/d lengthscale_k (d values), d/d outputscale, d/d noise, d/d mean_constant],
 * per data point like gpytorch's ExactMarginalLogLikelihood. Replaces the loss
 * that fit_gpytorch_mll minimises (botorch/fit.py:76 with
 * botorch/optim/closures/model_closures.py:117-143; no priors). d <= 64.
 * Synchronises `stream`. */
int bgb_gp_mll(const bgb_gp_t* gp, const double* y, const double* L, const double* Linv,
               const double* alpha, double* out_host, void* workspace, size_t workspace_bytes,
               void* stream);
size_t bgb_gp_mll_workspace_bytes(int64_t n, int32_t d);

/* (c) Model-level operands: B = Linv^T (n x ldb, ldb >= n) in float64 and
 * float32 (B32 may be NULL), float32 copies of Linv and beta (may be NULL), and
 * the training inputs scaled by 1 / lengthscale, Xs (d x n, k-major) in
 * float64 and float32 (Xs32 may be NULL). */
int bgb_gp_operands(const bgb_gp_t* gp, const double* Linv, const double* beta, double* B64,
                    float* B32, int64_t ldb, float* Linv32, float* beta32, double* Xs64,
                    float* Xs32, void* stream);

/* (c) Tensor-core operands of the mixed path: each row j of L^-1 (and of
 * L^-T) scaled by a power of two s_j that brings its largest magnitude to at
 * most 2^14, split into float16 hi = f16(s_j x), lo = f16(s_j x - hi):
 * (Lhi, Llo) and (LThi, LTlo), n x ldl each (ldl >= n, ldl % 8 == 0, columns
 * >= n zero); Lmul / LTmul (n floats) receive 1 / s_j. */
int bgb_gp_tc_operands(const bgb_gp_t* gp, const double* Linv, int64_t ldl, uint16_t* Lhi,
                       uint16_t* Llo, uint16_t* LThi, uint16_t* LTlo, float* Lmul, float* LTmul,
                       void* stream);

/* (c) The tensor-core GEMM of the mixed path on caller operands:
 *   C (M x N, ldc) = diag(row_mul) A op(B) diag(col_mul),
 * with A given as its float16 hi/lo split (M x K, lda) and B by its K-major
 * storage Bs (N x K, float16 hi/lo, ldbs): op(B)[k][j] = Bs[j][k]; the product
 * is ah*bh + ah*bl + al*bh accumulated in float32 (TMEM, drained into float32
 * registers every 64 k). row_mul (M floats) may be NULL, then every row uses
 * row_mul_const; col_mul (N floats) is required. kmode 3: op(B) upper
 * triangular (k <= j); kmode 1: op(B) lower triangular (k >= j); kmode 0:
 * full. *err_dev (device int, may be NULL) is set non-zero if a bounded wait
 * expired. lda and ldbs must be multiples of 8, ldc of 4, the pointers 16-byte
 * aligned. Exposed for tests and for callers with their own operands. */
int bgb_crosscov_gemm_f16x3(int64_t M, int64_t N, int64_t K, const uint16_t* A_hi,
                            const uint16_t* A_lo, int64_t lda, const uint16_t* B_hi,
                            const uint16_t* B_lo, int64_t ldbs, float* C, int64_t ldc,
                            const float* row_mul, float row_mul_const, const float* col_mul,
                            int32_t kmode, int32_t* err_dev, void* stream);

/* (c) Baseline operands of qLogNEI: Vb = K(X_baseline, Xt) L^-T (r x n) and
 * VbT (n x r), float64 and float32 (the float32 pointers may be NULL). */
int bgb_baseline_operands(const bgb_gp_t* gp, const double* Linv, const double* X_baseline,
                          int32_t r, double* Vb64, float* Vb32, double* VbT64, float* VbT32,
                          void* workspace, size_t workspace_bytes, void* stream);
size_t bgb_baseline_operands_workspace_bytes(int64_t n, int32_t r);

/* (c)+(d) Posterior mean (b x q) and covariance (b x q x q), untransformed
 * (acq->r must be 0). Replaces
 * BatchedMultiOutputGPyTorchModel.posterior (botorch/models/gpytorch.py:544-611)
 * followed by Standardize.untransform_posterior. */
int bgb_posterior(const bgb_acq_t* acq, const double* X, int64_t b, double* mean, double* covar,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Joint posterior over m points (mean m, covariance m x m, untransformed):
 * Kc = K(X, Xt), V = Kc L^-T, covar = K(X, X) - V V^T, mean = m + Kc alpha,
 * float64. Used at initialisation for the baseline posterior and for pruning
 * (botorch/acquisition/logei.py:393-459, acquisition/utils.py:276-437). */
int bgb_posterior_joint(const bgb_gp_t* gp, const double* Linv, const double* alpha,
                        const double* X, int64_t m, double* mean, double* covar, void* workspace,
                        size_t workspace_bytes, void* stream);
size_t bgb_posterior_joint_workspace_bytes(int64_t n, int64_t m);

/* prune_inferior_points (botorch/acquisition/utils.py:347-437): joint posterior
 * at X (m x d), L = psd_safe_cholesky(covar), samples = mean + Z L^T for the S
 * base samples Z (S x m), and counts[j] = number of samples whose argmax (first
 * maximal index, as torch.argmax) is j. counts is int32 (m). Synchronises. */
int bgb_prune_counts(const bgb_gp_t* gp, const double* Linv, const double* alpha, const double* X,
                     int64_t m, const double* Z, int32_t S, int32_t max_tries, int32_t* counts,
                     void* workspace, size_t workspace_bytes, void* stream);
size_t bgb_prune_counts_workspace_bytes(int64_t n, int64_t m, int32_t S);

/* qLogNEI baseline with cached root (logei.py:393-459, cached_cholesky.py:98-124):
 * joint posterior at X_baseline (r x d), Lb = psd_safe_cholesky(covar) (r x r),
 * Lb_inv = Lb^-1, baseline samples mean + Zb Lb^T and best_f[s] = max over r
 * (acquisition/utils.py:137-141). Synchronises. */
int bgb_qlognei_baseline(const bgb_gp_t* gp, const double* Linv, const double* alpha,
                         const double* X_baseline, int32_t r, const double* Zb, int32_t S,
                         int32_t max_tries, double* Lb, double* Lb_inv, double* best_f,
                         double* jitter_host, void* workspace, size_t workspace_bytes,
                         void* stream);
size_t bgb_qlognei_baseline_workspace_bytes(int64_t n, int32_t r, int32_t S);

/* Joint-sampling operands of qLogNEI (BGB_FLAG_JOINT_SAMPLING, BGB_FLAG_UNCACHED_ROOT):
 * the untransformed baseline posterior (mean_b, Sigma_bb) at X_baseline (r x d)
 * and, for each of the 7 jitter levels t of psd_safe_cholesky (total jitter 0,
 * then 1e-8 x 10^(t-1)), L_t = chol(Sigma_bb + j_t I), Lb_inv_lv[t] = L_t^-1
 * (r x r) and best_f_lv[t][s] = max_j (mean_b + Zb L_t^T)[s][j] (S values). A
 * level whose factorisation fails has NaN in Lb_inv_lv[t][0] and in best_f_lv[t].
 * The levels are those the reference's psd_safe_cholesky tries on the joint
 * covariance inside MultivariateNormal.rsample, reached from
 * get_posterior_samples (botorch/acquisition/acquisition.py:128-138) on the
 * fallback path of cached_cholesky.py:143-158 and for cache_root=False
 * (logei.py:543-553). Synchronises. */
int bgb_qlognei_joint_levels(const bgb_gp_t* gp, const double* Linv, const double* alpha,
                             const double* X_baseline, int32_t r, const double* Zb, int32_t S,
                             double* Lb_inv_lv, double* best_f_lv, void* workspace,
                             size_t workspace_bytes, void* stream);
size_t bgb_qlognei_joint_levels_workspace_bytes(int64_t n, int32_t r, int32_t S);

/* Reparameterised samples of the batched posterior MVN (float64): per batch member
 * L = psd_safe_cholesky(covar[b]) (jitter 1e-8 x 10^t for t < max_tries, this
 * member only) and samples[s][b][i] = mean[b][i] + sum_j L[i][j] Z[s][j], for
 * mean (b x q), covar (b x q x q), base samples Z (S x q, shared by every member)
 * and samples (S x b x q). status (b): 0, BGB_NOT_PSD or BGB_NAN (samples NaN
 * there). q <= 64 (BGB_ERR_UNSUPPORTED above). Replaces
 * GPyTorchPosterior.rsample_from_base_samples (botorch/posteriors/gpytorch.py:86-127;
 * gpytorch MultivariateNormal.rsample) as called by MCSampler.forward
 * (botorch/sampling/normal.py:34-50). */
int bgb_mvn_rsample(const double* mean, const double* covar, int64_t b, int32_t q,
                    const double* Z, int32_t S, int32_t max_tries, double* samples,
                    int32_t* status, void* stream);

/* Workspace for bgb_acq_forward / bgb_acq_forward_backward / bgb_posterior at b t-batches. */
size_t bgb_acq_workspace_bytes(const bgb_acq_t* acq, int64_t b);

/* (c)-(e) Acquisition value (b) at X (b x q x d). status (b, int32): 0 ok,
 * BGB_NOT_PSD / BGB_NAN per t-batch (value NaN there).
 * Replaces qExpectedImprovement.forward / qLogNoisyExpectedImprovement.forward
 * (botorch/acquisition/monte_carlo.py:268-305; logei.py:376-391, 527-565;
 * cached_cholesky.py:126-170; utils/low_rank.py:84-172). Asynchronous: the
 * return code covers the launches, the per-batch outcome is in `status`. */
int bgb_acq_forward(const bgb_acq_t* acq, const double* X, int64_t b, double* value,
                    int32_t* status, void* workspace, size_t workspace_bytes, void* stream);

/* Value (b) and gradient d value / d X (b x q x d) by the hand-written adjoint:
 * reverse through the sample reduction, the sample step, the q x q Cholesky and
 * the cross-covariance solve, recomputing K(X, Xt). Replaces
 * torch.autograd.grad(acqf(X).sum(), X) in botorch/generation/gen.py:466-469. */
int bgb_acq_forward_backward(const bgb_acq_t* acq, const double* X, int64_t b, double* value,
                             double* grad, int32_t* status, void* workspace,
                             size_t workspace_bytes, void* stream);

/* Same as bgb_acq_forward_backward, with CUDA events recorded on `stream`
 * between its seven stages (kernel build, forward cross-covariance GEMMs,
 * covariance reduction, per-batch step, row mix, adjoint GEMM, adjoint
 * contraction); stage_ms_host (7 floats, host) gets the stage durations.
 * Synchronises. Measurement aid; no reference counterpart. */
int bgb_acq_forward_backward_timed(const bgb_acq_t* acq, const double* X, int64_t b,
                                   double* value, double* grad, int32_t* status, void* workspace,
                                   size_t workspace_bytes, float* stage_ms_host, void* stream);

/* ---- No-allocation variant. No counterpart in the reference: there, PyTorch's
 * caching allocator always supplies the scratch memory.
 *
 * Computes what bgb_acq_forward_backward computes, but takes no workspace. Its
 * scratch is one fixed array of BGB_NOALLOC_SCRATCH_BYTES (32 MiB) that the
 * library keeps in device memory. The call itself allocates and frees nothing,
 * on the device or the host. It is for callers that cannot allocate at the
 * point of the call:
 *   - C, C++ or FFI hosts without a device allocator of their own (no PyTorch);
 *   - services that fix their device memory at start-up and must not grow it
 *     inside an optimisation loop;
 *   - latency-bound loops, where cudaMalloc / cudaFree may synchronise the
 *     device and stall work queued on other streams.
 * Limits:
 *   - The array holds about 48 KB per candidate point at n = 4096 in the mixed
 *     tensor-core form (b * q up to ~680 at n = 4096, ~2700 at n = 1024). A call
 *     that needs more (bgb_acq_workspace_bytes(acq, b) > BGB_NOALLOC_SCRATCH_BYTES)
 *     returns BGB_ERR_SCRATCH_LIMIT and launches nothing. Split the t-batches
 *     over several calls instead.
 *   - The first call on each device looks up the array's address on that device
 *     (with that device current), which may load the library's device code
 *     there. Make that first call before any stream capture on the device.
 *   - `stream` must belong to the current device (the array's address is per
 *     device); a stream of another device returns BGB_ERR_ARG.
 *   - All calls on a device share the one array. Calls that overlap on the GPU
 *     (two streams, or two host threads with their own streams) race and
 *     corrupt each other's results: issue them on one stream, or serialise them.
 *   - Each call clears, on its own stream, the one part of the array that must
 *     start at zero (the device error word); nothing else is read before it is
 *     written. */
#define BGB_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
int bgb_acq_forward_backward_noalloc(const bgb_acq_t* acq, const double* X, int64_t b,
                                     double* value, double* grad, int32_t* status, void* stream);

/* ---- Grouped evaluation of many independent problems. The reference
 * evaluates each model's acquisition function in its own optimize_acqf call
 * (botorch/generation/gen.py:423-487 per model; MCAcquisitionFunction.forward,
 * botorch/acquisition/logei.py:247-289); a group runs the value and gradient of
 * `count` problems (one model each, uneven n and d) in about ten launches:
 * each stage (kernel build, forward tensor-core GEMM, covariance reduction,
 * batch step, row mix, adjoint GEMM, adjoint) is one launch over all problems,
 * its CTAs mapped to (problem, block) through per-stage prefix tables, and the
 * two GEMMs walk one tile list over all problems, dealt out largest first to
 * the least-loaded two-SM cluster. The results equal `count` calls of
 * bgb_acq_forward_backward on the same structs.
 * Every member must be the mixed tensor-core form with a cached root (no
 * BGB_FLAG_JOINT_SAMPLING), q <= 8, r <= 4; otherwise the size query returns 0
 * and create returns BGB_ERR_UNSUPPORTED.
 * The plan keeps the pointers it is given: X[i] (b[i] x q x d), value[i],
 * grad[i], status[i] are read and written by every bgb_group_run, and the
 * structs' operands must stay alive and unchanged. create synchronises
 * `stream` and launches work on it; run only launches (capturable in a CUDA
 * graph); the workspace belongs to the plan until destroy. */
typedef struct bgb_group bgb_group_t;
size_t bgb_group_workspace_bytes(const bgb_acq_t* acqs, const int64_t* b, int32_t count);
int bgb_group_create(const bgb_acq_t* acqs, const int64_t* b, int32_t count,
                     const double* const* X, double* const* value, double* const* grad,
                     int32_t* const* status, void* workspace, size_t workspace_bytes, void* stream,
                     bgb_group_t** out);
int bgb_group_run(const bgb_group_t* group, void* stream);
/* kernels one run launches (8, or 10 when an adjoint is split into slabs) */
int32_t bgb_group_launches(const bgb_group_t* group);
void bgb_group_destroy(bgb_group_t* group);

/* ---- Fused log-areas of qLogEHVI / qLogNEHVI (the inner loop of
 * _compute_log_qehvi, botorch/acquisition/multi_objective/logei.py:272-392).
 * Replace the reference's CPU extension botorch/csrc/logei_fused.cpp:
 * bgb_log_areas_forward  <- fused_log_areas_forward  (logei_fused.cpp:184-264),
 * bgb_log_areas_backward <- fused_log_areas_backward (logei_fused.cpp:266-374).
 * All pointers are device pointers to contiguous row-major arrays:
 *   obj       (B, n_sub, isz, m)  objective values of the q-subsets of size isz
 *   cell_lower, cell_upper (B_cells, nc, m), B_cells == 1 (shared cells) or B
 *   out       (B, nc, n_sub)      log area of each cell and subset
 *   grad_out  (B, nc, n_sub), grad_obj (B, n_sub, isz, m)
 * Limits as the reference's: 1 <= isz <= 32, 1 <= m <= 8 (larger returns
 * BGB_ERR_UNSUPPORTED); tau_relu, tau_max > 0. Empty B, n_sub or nc is a no-op
 * (grad_obj is zero-filled when nc == 0). The *_f32 forms compute in float
 * with the reference's float clamp of the upper bounds (1e8; 1e10 in double). */
int bgb_log_areas_forward(const double* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                          const double* cell_lower, const double* cell_upper, int64_t B_cells,
                          int64_t nc, double tau_relu, double tau_max, double* out, void* stream);
int bgb_log_areas_forward_f32(const float* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                              const float* cell_lower, const float* cell_upper, int64_t B_cells,
                              int64_t nc, double tau_relu, double tau_max, float* out,
                              void* stream);
int bgb_log_areas_backward(const double* grad_out, const double* obj, int64_t B, int64_t n_sub,
                           int64_t isz, int64_t m, const double* cell_lower,
                           const double* cell_upper, int64_t B_cells, int64_t nc, double tau_relu,
                           double tau_max, double* grad_obj, void* stream);
int bgb_log_areas_backward_f32(const float* grad_out, const float* obj, int64_t B, int64_t n_sub,
                               int64_t isz, int64_t m, const float* cell_lower,
                               const float* cell_upper, int64_t B_cells, int64_t nc,
                               double tau_relu, double tau_max, float* grad_obj, void* stream);

/* Forward that also keeps the Jacobian of every area with respect to its
 * subset's objective values, and the backward as a contraction with it (no
 * counterpart in the reference, which recomputes in its backward; here the
 * recomputation is FP64-bound and the contraction HBM-bound):
 *   jac      (B, nc, n_sub, isz, m): d out[b][c][s] / d obj[b][s][j][k]
 *   grad_obj[b][s][j][k] = sum_c grad_out[b][c][s] jac[b][c][s][j][k]
 * out equals bgb_log_areas_forward's; grad_obj equals bgb_log_areas_backward's
 * up to rounding. */
int bgb_log_areas_forward_jac(const double* obj, int64_t B, int64_t n_sub, int64_t isz, int64_t m,
                              const double* cell_lower, const double* cell_upper, int64_t B_cells,
                              int64_t nc, double tau_relu, double tau_max, double* out,
                              double* jac, void* stream);
int bgb_log_areas_forward_jac_f32(const float* obj, int64_t B, int64_t n_sub, int64_t isz,
                                  int64_t m, const float* cell_lower, const float* cell_upper,
                                  int64_t B_cells, int64_t nc, double tau_relu, double tau_max,
                                  float* out, float* jac, void* stream);
int bgb_log_areas_backward_jac(const double* grad_out, const double* jac, int64_t B,
                               int64_t n_sub, int64_t isz, int64_t m, int64_t nc,
                               double* grad_obj, void* stream);
int bgb_log_areas_backward_jac_f32(const float* grad_out, const float* jac, int64_t B,
                                   int64_t n_sub, int64_t isz, int64_t m, int64_t nc,
                                   float* grad_obj, void* stream);

/* ---- Batched L-BFGS-B on the device: the per-restart optimiser of the
 * reference's fast path (botorch/generation/gen.py:226-247, which drives
 * fmin_l_bfgs_b_batched, botorch/optim/batched_lbfgs_b.py:169-636, stepping
 * scipy's L-BFGS-B routine once per restart and round). `restarts`
 * independent problems of n variables share the bounds; each keeps its own
 * L-BFGS-B 3.0 state (history m, line search of More and Thuente) in the
 * workspace. Reverse communication, as scipy's routine: init projects every
 * row of X (restarts x n) onto the box and leaves each restart waiting for f
 * and g at its row; every step consumes the objective f = sign * value[r] and
 * g = sign * grad[r] of the restarts that wait, advances each to the next
 * point it needs (written into its row of X) or stops it, and (summary !=
 * NULL) writes four int32 counts: restarts still waiting for f and g, restarts
 * held back because some row's status was nonzero (ignore_status = 0; the
 * caller evaluates X again another way and repeats the step with ignore_status
 * = 1), restarts stopped on a non-finite value or gradient, restarts stopped.
 * Stopped restarts keep their row of X. The stopping rules and options mean
 * what they mean for scipy.optimize.minimize(method="L-BFGS-B"): factr =
 * ftol / machine epsilon, pgtol = gtol, maxls, maxiter (iterations), maxfun
 * (evaluations). 1 <= n <= 8192 and 1 <= m <= 20 (else BGB_ERR_UNSUPPORTED);
 * lower / upper are device arrays of n bounds (+-inf: none). Every call only
 * launches (capturable in a CUDA graph). */
typedef struct bgb_lbfgsb_opts {
    int64_t restarts;
    int64_t n;
    int32_t m;
    int32_t maxls;
    int64_t maxiter;
    int64_t maxfun;
    double factr;
    double pgtol;
} bgb_lbfgsb_opts;
#define BGB_LBFGSB_RUNNING 0
#define BGB_LBFGSB_CONV_PGTOL 1    /* projected gradient <= pgtol */
#define BGB_LBFGSB_CONV_FTOL 2     /* relative reduction of f <= factr * eps */
#define BGB_LBFGSB_ABNORMAL 3      /* line search failed with no history left */
#define BGB_LBFGSB_MAXITER 4
#define BGB_LBFGSB_MAXFUN 5
#define BGB_LBFGSB_NONFINITE 6     /* f or g not finite at the restart's point */
size_t bgb_lbfgsb_workspace_bytes(const bgb_lbfgsb_opts* opts);
int bgb_lbfgsb_init(const bgb_lbfgsb_opts* opts, double* X, const double* lower, const double* upper,
                    void* workspace, size_t workspace_bytes, void* stream);
int bgb_lbfgsb_step(const bgb_lbfgsb_opts* opts, double* X, const double* value, double sign,
                    const double* grad, const int32_t* status, int32_t ignore_status,
                    void* workspace, size_t workspace_bytes, int32_t* summary, void* stream);
/* Per restart: f at its row of X, iterations, evaluations, BGB_LBFGSB_* code
 * (any pointer may be NULL). */
int bgb_lbfgsb_results(const bgb_lbfgsb_opts* opts, const void* workspace, size_t workspace_bytes,
                       double* f, int64_t* nit, int64_t* nfev, int32_t* code, void* stream);

/* ---- Scrambled Sobol points mapped to a box (the raw samples of the
 * acquisition optimisation: botorch/utils/sampling.py:74-111, draw_sobol_samples,
 * which draws torch.quasirandom.SobolEngine(q * d, scramble=True, seed) on the
 * host). The engine's state comes from the host: `state` (dim x maxbit int64,
 * its scrambled direction numbers), `shift` (dim int64, its digital shift) and
 * `first_point` (dim doubles: point 0 as the engine returns it). Writes points
 * first .. first + n - 1 of the sequence, mapped to lower + (upper - lower) * u
 * with the bounds repeating every `period` dimensions (dim % period == 0), as
 * out (n x dim, row-major), bit for bit what the engine's draw followed by the
 * elementwise map gives in float64. first + n <= 2^maxbit. */
int bgb_sobol_box(const int64_t* state, const int64_t* shift, const double* first_point, int32_t dim,
                  int32_t maxbit, int64_t first, int64_t n, const double* lower, const double* upper,
                  int32_t period, double* out, void* stream);

/* Number of kernel launches this library has issued in the process so far.
 * Measurement aid; no reference counterpart. */
unsigned long long bgb_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* BOTORCH_GB300_H */
