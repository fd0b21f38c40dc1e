// extern "C" entry points of libbotorch_gb300.so (declared in include/botorch_gb300.h).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <new>
#include <vector>
#include <cmath>
#include <mutex>

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"
#include "bgb_qbatch.cuh"

using namespace bgb;

namespace bgb {
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace bgb

// Scratch of bgb_acq_forward_backward_noalloc: one fixed array per device,
// shared by every call of that entry point on the device. Part of the module's
// static device memory, so using it allocates nothing at call time.
static __device__ __align__(256) unsigned char g_noalloc_scratch[BGB_NOALLOC_SCRATCH_BYTES];

namespace {

__global__ void sub_const_kernel(const double* x, double c, double* y, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] - c;
}

// ZT[k][i] = X[i][k] / l_k in float32 (k-major): the candidates' scaled
// coordinates for the float32 kernel build, scaled once per call.
__global__ void scale_rows_t_kernel(const double* X, int64_t rows, int d, const double* il,
                                    float* ZT) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * d) return;
    const int64_t i = idx / d;
    const int k = (int)(idx % d);
    ZT[(int64_t)k * rows + i] = (float)(X[idx] * il[k]);
}

// XsT[k][c] = Xt[c][k] / l_k (k-major, for the adjoint's coalesced staging)
__global__ void scale_inputs_kernel(const double* X, const double* il, int64_t n, int d,
                                    double* Xs64, float* Xs32) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * d) return;
    const int64_t c = idx / d;
    const int k = (int)(idx % d);
    const double v = X[idx] * il[k];
    Xs64[(int64_t)k * n + c] = v;
    if (Xs32 != nullptr) Xs32[(int64_t)k * n + c] = (float)v;
}

// B = [Linv^T | 0]: B[k][j] = Linv[j][k] for j < n
__global__ void fill_b_kernel(const double* Linv, int64_t n, double* B, int64_t ldb) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * ldb) return;
    int64_t k = idx / ldb, j = idx % ldb;
    B[idx] = (j < n) ? Linv[j * n + k] : 0.0;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int valid_gp(const bgb_gp_t* gp) {
    if (gp == nullptr || gp->n <= 0 || gp->d <= 0 || gp->train_X == nullptr ||
        gp->inv_lengthscale == nullptr)
        return 0;
    if (gp->kernel < BGB_KERNEL_MATERN52 || gp->kernel > BGB_KERNEL_RBF) return 0;
    return 1;
}

// The mixed path runs its GEMMs on the tensor cores when the float16 operands are set.
bool use_tc(const bgb_acq_t* a) {
    return a->precision == BGB_PREC_MIXED && !(a->flags & BGB_FLAG_SIMT) && a->Lhi != nullptr &&
           a->Llo != nullptr && a->LThi != nullptr && a->LTlo != nullptr && a->Lmul != nullptr &&
           a->LTmul != nullptr && a->ldl >= a->gp.n && (a->ldl % 8) == 0 && (a->ldb % 4) == 0 &&
           tc_gemm_available();
}

// Elements (of the path's float type) of the Kc / H region: rows x n, or on the
// tensor cores the float16 hi and lo halves, rows x ldl each (= rows x ldl floats).
int64_t kc_region_elems(const bgb_acq_t* a, int64_t rows) {
    return use_tc(a) ? rows * a->ldl : rows * a->gp.n;
}

int joint_mode(const bgb_acq_t* a);
// best_f sets the mixed path converts to float pairs: one, or one per jitter level
int64_t bf_levels(const bgb_acq_t* a) { return joint_mode(a) == 2 ? 7 : 1; }

// Workspace of one call: the Kc (later H, later the adjoint's slab partials)
// region, C = V (later D) rows x ldb, P rows x r, the float64 per-batch blocks,
// the device error word, and for the mixed path the scaled candidates, the
// float32 base samples and best_f pairs, and (tensor cores) H's row multipliers.
size_t acq_ws_layout(const bgb_acq_t* a, int64_t b, Arena* ar, QBatchArgs* qa, void** Kc,
                     void** C, void** P, int** err = nullptr) {
    const int64_t n = a->gp.n;
    const int64_t rows = b * a->q;
    const int64_t rr = a->r > 0 ? a->r : 1;
    const size_t es = (a->precision == BGB_PREC_MIXED) ? sizeof(float) : sizeof(double);
    const bool tc = use_tc(a);
    const int64_t kc_elems = kc_region_elems(a, rows);
    size_t total = 0;
    total += align_up(kc_elems * es);
    total += align_up(rows * a->ldb * es);
    total += align_up(rows * rr * es);
    total += align_up(sizeof(double) * b * a->q * a->q) * 2;
    total += align_up(sizeof(double) * b * a->q * rr) * 2;
    total += align_up(sizeof(double) * b * a->q) * 2;
    total += align_up(sizeof(int));
    if (es == sizeof(float)) {
        total += align_up(sizeof(float) * rows * a->gp.d);
        total += align_up(sizeof(float) * (size_t)a->n_samples * (a->r + a->q));
        total += align_up(sizeof(float) * 2 * (size_t)a->n_samples * bf_levels(a));
        if (tc) total += align_up(sizeof(float) * rows);
    }
    if (ar == nullptr) return total;
    if (ar->cap < total) return 0;
    if (es == sizeof(float)) {
        *Kc = ar->take<float>(kc_elems);
        *C = ar->take<float>(rows * a->ldb);
        *P = ar->take<float>(rows * rr);
    } else {
        *Kc = ar->take<double>(kc_elems);
        *C = ar->take<double>(rows * a->ldb);
        *P = ar->take<double>(rows * rr);
    }
    qa->sig = ar->take<double>(b * a->q * a->q);
    qa->gqq = ar->take<double>(b * a->q * a->q);
    qa->sqb = ar->take<double>(b * a->q * rr);
    qa->gqb = ar->take<double>(b * a->q * rr);
    qa->mu = ar->take<double>(b * a->q);
    qa->gmu = ar->take<double>(b * a->q);
    int* e = ar->take<int>(1);
    if (err != nullptr) *err = e;
    if (es == sizeof(float)) {
        qa->zt = ar->take<float>(rows * a->gp.d);
        qa->z32 = ar->take<float>((int64_t)a->n_samples * (a->r + a->q));
        qa->bf32 = ar->take<float>(2 * (int64_t)a->n_samples * bf_levels(a));
        if (tc) qa->hmul = ar->take<float>(rows);
    }
    return total;
}

// Sampling of the q new points: 0 cached root, 1 joint sampling with the cached
// incumbent (the reference's fallback), 2 joint sampling without the cached root.
int joint_mode(const bgb_acq_t* a) {
    if (a->r <= 0 || !(a->flags & BGB_FLAG_JOINT_SAMPLING)) return 0;
    return (a->flags & BGB_FLAG_UNCACHED_ROOT) ? 2 : 1;
}

void fill_qargs(const bgb_acq_t* a, const double* X, int64_t b, QBatchArgs* qa) {
    qa->b = b;
    qa->n = a->gp.n;
    qa->q = a->q;
    qa->r = a->r;
    qa->S = a->n_samples;
    qa->d = a->gp.d;
    qa->kernel = a->gp.kernel;
    qa->acqf = a->acqf;
    qa->max_tries = 6;     // botorch/__init__.py:54, utils/low_rank.py:90
    qa->jitter = 1e-8;     // float64 jitter of psd_safe_cholesky
    qa->outputscale = a->gp.outputscale;
    qa->mean_constant = a->gp.mean_constant;
    qa->y_mean = a->gp.y_mean;
    qa->y_std = a->gp.y_std;
    qa->tau_relu = a->tau_relu;
    qa->tau_max = a->tau_max;
    qa->inv_tau_relu_f = (float)(1.0 / a->tau_relu);
    qa->log_tau_relu_f = (float)log(a->tau_relu);
    qa->inv_tau_max_f = (float)(1.0 / a->tau_max);
    qa->log_S = log((double)a->n_samples);
    qa->sqrt_outputscale = sqrt(a->gp.outputscale);
    qa->X = X;
    qa->Xt = a->gp.train_X;
    qa->Xb = a->X_baseline;
    qa->inv_ls = a->gp.inv_lengthscale;
    qa->Lb_inv = a->Lb_inv;
    qa->Z = a->Z;
    qa->best_f = a->best_f;
    qa->beta_absmax = a->beta_absmax;
    qa->adj_ctas_per_sm = (a->flags & BGB_FLAG_ADJ_CTAS_MASK) >> BGB_FLAG_ADJ_CTAS_SHIFT;
    qa->joint = joint_mode(a);
    qa->Lb_inv_lv = a->Lb_inv_lv;
    qa->best_f_lv = a->best_f_lv;
}

int valid_acq(const bgb_acq_t* a) {
    if (a == nullptr || !valid_gp(&a->gp)) return 0;
    if (a->q <= 0 || a->r < 0 || a->ldb < a->gp.n) return 0;
    if (a->precision == BGB_PREC_FP64) {
        if (a->B64 == nullptr || a->Linv64 == nullptr || a->beta64 == nullptr ||
            a->Xs64 == nullptr)
            return 0;
        if (a->r > 0 && (a->Vb64 == nullptr || a->VbT64 == nullptr)) return 0;
    } else if (a->precision == BGB_PREC_MIXED) {
        if (a->B32 == nullptr || a->Linv32 == nullptr || a->beta32 == nullptr ||
            a->Xs32 == nullptr)
            return 0;
        if (a->r > 0 && (a->Vb32 == nullptr || a->VbT32 == nullptr)) return 0;
    } else {
        return 0;
    }
    if (a->r > 0 && (a->X_baseline == nullptr || a->Lb_inv == nullptr)) return 0;
    if (joint_mode(a) >= 1 && a->Lb_inv_lv == nullptr) return 0;
    if (joint_mode(a) == 2 && a->best_f_lv == nullptr) return 0;
    return 1;
}

// Typed pieces of the per-call pipeline.
template <typename T> struct Ops;
template <> struct Ops<float> {
    static const float* B(const bgb_acq_t* a) { return a->B32; }
    static const float* Linv(const bgb_acq_t* a) { return a->Linv32; }
    static const float* Vb(const bgb_acq_t* a) { return a->Vb32; }
    static const float* VbT(const bgb_acq_t* a) { return a->VbT32; }
    static const float* beta(const bgb_acq_t* a) { return a->beta32; }
    static const float* Xs(const bgb_acq_t* a) { return a->Xs32; }
    static int gemm(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                    int64_t ldb, float* C, int64_t ldc, int kmode, int64_t n_tri, cudaStream_t st) {
        return gemm_f32(M, N, K, A, lda, B, ldb, C, ldc, kmode, n_tri, st);
    }
    // K(X, Xt) in float32 from the scaled coordinates (zt: d x rows, Xs32: d x n);
    // K16 non-null: the float16 hi / lo split of k16_scale * K with leading dimension ldk
    static int kmat(const bgb_acq_t* a, const double* X, int64_t rows, float* zt, float* K,
                    int64_t ldk, __half* K16, __half* K16_lo, float k16_scale, cudaStream_t st) {
        const int64_t tot = rows * a->gp.d;
        scale_rows_t_kernel<<<(unsigned)ceil_div(tot, 256), 256, 0, st>>>(
            X, rows, a->gp.d, a->gp.inv_lengthscale, zt);
        BGB_CHECK_LAUNCH();
        return launch_kernel_matrix_zt(zt, rows, rows, a->Xs32, a->gp.n, a->gp.n, a->gp.d,
                                       a->gp.outputscale, a->gp.kernel, K, K16, K16_lo, k16_scale,
                                       ldk, st);
    }
};
template <> struct Ops<double> {
    static const double* B(const bgb_acq_t* a) { return a->B64; }
    static const double* Linv(const bgb_acq_t* a) { return a->Linv64; }
    static const double* Vb(const bgb_acq_t* a) { return a->Vb64; }
    static const double* VbT(const bgb_acq_t* a) { return a->VbT64; }
    static const double* beta(const bgb_acq_t* a) { return a->beta64; }
    static const double* Xs(const bgb_acq_t* a) { return a->Xs64; }
    static int gemm(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                    const double* B, int64_t ldb, double* C, int64_t ldc, int kmode, int64_t n_tri,
                    cudaStream_t st) {
        return gemm_f64(M, N, K, 1.0, A, lda, 0, B, ldb, 0, 0.0, C, ldc, kmode, 0, nullptr, st,
                        n_tri);
    }
    static int kmat(const bgb_acq_t* a, const double* X, int64_t rows, float* /*zt*/, double* K,
                    int64_t ldk, __half* /*K16*/, __half* /*K16_lo*/, float /*k16_scale*/,
                    cudaStream_t st) {
        return launch_kernel_matrix<double, double, double>(
            X, rows, a->gp.train_X, a->gp.n, a->gp.d, a->gp.inv_lengthscale, a->gp.outputscale,
            a->gp.kernel, 0.0, 0, K, ldk, st);
    }
};

// Power of two s with outputscale * s <= 2^14: the float16 scale of K(X, Xt),
// whose entries are at most outputscale.
float kc_scale(double outputscale) {
    if (!(outputscale > 0.0) || std::isinf(outputscale)) return 1.f;
    int e;
    frexp(outputscale, &e);
    return ldexpf(1.f, 14 - e);
}

// Kernel build, V = K(X,Xt) L^-T, mu = m + V beta and P = V Vb^T, covariance reduction.
template <typename T>
int run_front(const bgb_acq_t* a, const double* X, int64_t b, QBatchArgs* qa, T* Kc, T* C, T* P,
              cudaStream_t st, cudaEvent_t* ev) {
    const int64_t n = a->gp.n, rows = b * a->q;
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[0], st));
    int rc;
    if constexpr (sizeof(T) == 4) {
        if (use_tc(a)) {
            // tensor cores: K(X, Xt) as its scaled float16 split, then V = K L^-T
            __half* Khi = reinterpret_cast<__half*>(Kc);
            __half* Klo = Khi + rows * a->ldl;
            const float ks = kc_scale(a->gp.outputscale);
            rc = Ops<float>::kmat(a, X, rows, qa->zt, nullptr, a->ldl, Khi, Klo, ks, st);
            if (rc) return rc;
            if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[1], st));
            rc = tc_gemm_f16x3(rows, n, n, Khi, Klo, a->ldl, reinterpret_cast<const __half*>(a->Lhi),
                               reinterpret_cast<const __half*>(a->Llo), a->ldl, C, a->ldb, KB_UPPER,
                               nullptr, 1.f / ks, a->Lmul, const_cast<int*>(qa->dev_err), st);
            if (rc) return rc;
            goto after_gemm;
        }
    }
    rc = Ops<T>::kmat(a, X, rows, qa->zt, Kc, n, nullptr, nullptr, 0.f, st);
    if (rc) return rc;
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[1], st));
    rc = Ops<T>::gemm(rows, n, n, Kc, n, Ops<T>::B(a), a->ldb, C, a->ldb, KB_UPPER, n, st);
    if (rc) return rc;
after_gemm:
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[2], st));
    rc = launch_qstats<T>(*qa, C, a->ldb, Ops<T>::beta(a), Ops<T>::Vb(a), st);
    if (rc == BGB_ERR_UNSUPPORTED)  // q > 8 or r > 4: shared-memory tiles; the Kc region is
        // free here (the forward GEMM has read it) and holds split partial sums
        rc = launch_qstats_tile<T>(*qa, C, a->ldb, Ops<T>::beta(a), Ops<T>::Vb(a), Kc,
                                   sizeof(T) * (size_t)kc_region_elems(a, b * a->q), st);
    if (rc == BGB_ERR_UNSUPPORTED) {  // beyond those: separate row and pair passes
        rc = launch_row_dots<T>(*qa, C, a->ldb, Ops<T>::beta(a), Ops<T>::Vb(a), P, st);
        if (rc) return rc;
        rc = launch_sigma_reduce<T>(*qa, P, C, a->ldb, st);
    }
    if (rc) return rc;
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[3], st));
    return BGB_OK;
}

// Stage boundaries of the per-stage timing variant: kernel build, forward
// cross-covariance GEMMs, covariance reduction, per-batch step, row mix,
// adjoint GEMM, adjoint contraction.
constexpr int kStages = 7;

template <typename T>
int run_call(const bgb_acq_t* a, const double* X, int64_t b, QBatchArgs& qa, T* Kc, T* C, T* P,
             int backward, cudaStream_t st, cudaEvent_t* ev) {
    const int64_t n = a->gp.n, rows = b * a->q;
    int rc = run_front<T>(a, X, b, &qa, Kc, C, P, st, ev);
    if (rc) return rc;
    rc = launch_batch_step(qa, backward, st, sizeof(T) == 4);
    if (rc) return rc;
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[4], st));
    if (!backward) return BGB_OK;
    // H = gmu beta^T - 2 Gqq V - Gqb Vb into the Kc buffer; D = H L^-1 into the V buffer
    T* H = Kc;
    bool tc = false;
    if constexpr (sizeof(T) == 4) tc = use_tc(a);
    if (tc) {
        __half* Hhi = reinterpret_cast<__half*>(Kc);
        __half* Hlo = Hhi + rows * a->ldl;
        rc = launch_mix_rows<T>(qa, C, a->ldb, Ops<T>::Vb(a), Ops<T>::beta(a), nullptr, st, Hhi,
                                Hlo, a->ldl);
        if (rc) return rc;
        if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[5], st));
        if constexpr (sizeof(T) == 4) {
            rc = tc_gemm_f16x3(rows, n, n, Hhi, Hlo, a->ldl,
                               reinterpret_cast<const __half*>(a->LThi),
                               reinterpret_cast<const __half*>(a->LTlo), a->ldl, C, a->ldb, KB_LOWER,
                               qa.hmul, 1.f, a->LTmul, const_cast<int*>(qa.dev_err), st);
            if (rc) return rc;
        }
    } else {
        rc = launch_mix_rows<T>(qa, C, a->ldb, Ops<T>::Vb(a), Ops<T>::beta(a), H, st);
        if (rc) return rc;
        if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[5], st));
        rc = Ops<T>::gemm(rows, n, n, H, n, Ops<T>::Linv(a), n, C, a->ldb, KB_LOWER, 0, st);
        if (rc) return rc;
    }
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[6], st));
    // the Kc / H region is free once the adjoint GEMM has read H: slab partials go there
    const int64_t kc_elems = kc_region_elems(a, rows);
    rc = launch_adjoint<T>(qa, C, a->ldb, Ops<T>::Xs(a), Kc, kc_elems, st);
    if (rc) return rc;
    if (ev) BGB_CUDA_TRY(cudaEventRecord(ev[7], st));
    return BGB_OK;
}

int acq_call(const bgb_acq_t* a, const double* X, int64_t b, double* value, double* grad,
             int32_t* status, void* ws, size_t ws_bytes, cudaStream_t st,
             cudaEvent_t* ev = nullptr) {
    if (!valid_acq(a) || X == nullptr || value == nullptr || status == nullptr || b < 0)
        return BGB_ERR_ARG;
    if (a->n_samples <= 0 || a->Z == nullptr || a->best_f == nullptr) return BGB_ERR_ARG;
    if (b == 0) return BGB_OK;
    Arena ar{static_cast<char*>(ws), ws_bytes, 0};
    QBatchArgs qa;
    memset(&qa, 0, sizeof(qa));
    void *Kc = nullptr, *C = nullptr, *P = nullptr;
    int* err = nullptr;
    if (ws == nullptr || acq_ws_layout(a, b, &ar, &qa, &Kc, &C, &P, &err) == 0)
        return BGB_ERR_WORKSPACE;
    fill_qargs(a, X, b, &qa);
    BGB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    qa.dev_err = err;
    qa.value = value;
    qa.grad = grad;
    qa.status = status;
    if (a->precision == BGB_PREC_MIXED)
        return run_call<float>(a, X, b, qa, static_cast<float*>(Kc), static_cast<float*>(C),
                               static_cast<float*>(P), grad != nullptr, st, ev);
    return run_call<double>(a, X, b, qa, static_cast<double*>(Kc), static_cast<double*>(C),
                            static_cast<double*>(P), grad != nullptr, st, ev);
}

// Device address of g_noalloc_scratch on the current device, looked up once per
// device (cudaGetSymbolAddress with that device current) and cached. `stream`
// must belong to the current device.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

int noalloc_scratch(cudaStream_t stream, void** out) {
    int dev = -1;
    BGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return BGB_ERR_UNSUPPORTED;
    // the array's address is per device: a stream of another device would get
    // this device's address, so such a call is rejected
    if (stream != nullptr) {
        int sdev = -1;
        BGB_CUDA_TRY(cudaStreamGetDevice(stream, &sdev));
        if (sdev != dev) return BGB_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr)
            return BGB_ERR_CUDA;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return BGB_OK;
}

// ---------------------------------------------------------------- grouped plans
// Stages of a grouped run, in launch order (each one launch over all models).
enum GroupStage : int { GS_SCALE, GS_KM, GS_QSTATS, GS_BSTEP, GS_MIX, GS_ADJ, GS_SUM, GS_FIN, GS_N };

// The adjoint's register arrays are sized by a compile-time bound on d: models
// are launched in buckets of equal bound (as their own calls would run them).
constexpr int kDBuckets = 7;
constexpr int kDBound[kDBuckets] = {8, 12, 16, 20, 24, 32, 64};
inline int d_bucket(int d) {
    for (int i = 0; i < kDBuckets; ++i)
        if (d <= kDBound[i]) return i;
    return -1;
}


// Requirements of a grouped problem: the mixed tensor-core path with a cached
// root, q <= 8 and r <= 4 (the one-pass covariance reduction).
int group_member_ok(const bgb_acq_t* a, int64_t b) {
    if (!valid_acq(a) || b <= 0) return BGB_ERR_ARG;
    if (a->n_samples <= 0 || a->Z == nullptr || a->best_f == nullptr) return BGB_ERR_ARG;
    if (a->precision != BGB_PREC_MIXED || !use_tc(a) || joint_mode(a) != 0 || a->q > 8 ||
        a->gp.d > 64 ||
        a->r > 4 || a->Xs32 == nullptr || a->beta32 == nullptr || (a->r > 0 && a->Vb32 == nullptr))
        return BGB_ERR_UNSUPPORTED;
    return BGB_OK;
}

struct GroupSizes {
    size_t arenas = 0, tables = 0, total = 0;
    int64_t tiles_fwd = 0, tiles_adj = 0;
};

GroupSizes group_sizes(const bgb_acq_t* acqs, const int64_t* b, int count) {
    GroupSizes z;
    for (int i = 0; i < count; ++i) {
        z.arenas += align_up(acq_ws_layout(&acqs[i], b[i], nullptr, nullptr, nullptr, nullptr, nullptr));
        const int64_t rows = b[i] * acqs[i].q, n = acqs[i].gp.n;
        const int64_t t = tc_group_tiles(rows, n);
        z.tiles_fwd += t;
        z.tiles_adj += t;
    }
    const size_t cnt = (size_t)count;
    z.tables = align_up(sizeof(int)) + align_up(cnt * sizeof(KmG)) +
               align_up(cnt * sizeof(QstatsG<float>)) + align_up(cnt * sizeof(BstepG)) +
               align_up(cnt * sizeof(MixG<float>)) + align_up(cnt * sizeof(AdjG<float>)) +
               GS_N * align_up((cnt + 1) * sizeof(int)) +
               kDBuckets * align_up((cnt + 1) * sizeof(int)) +
               2 * (align_up(cnt * tc_group_entry_bytes()) + align_up(sizeof(int) * 256)) +
               align_up(sizeof(uint64_t) * (size_t)z.tiles_fwd) +
               align_up(sizeof(uint64_t) * (size_t)z.tiles_adj);
    z.total = z.arenas + z.tables;
    return z;
}

}  // namespace

// The plan of a grouped run (opaque to C callers).
struct bgb_group {
    int count = 0;
    int launches = 0;
    int* err = nullptr;
    GroupTab tab[GS_N];
    int64_t ctas[GS_N] = {};
    // the adjoint per d bucket (models in bucket order in the AdjG table)
    GroupTab adj_tab[kDBuckets];
    int64_t adj_ctas[kDBuckets] = {};
    int qmax = 0, rmax = 0, dmax = 0;
    size_t bs_smem = 0, mix_smem = 0;
    bool partials = false;
    const void* tc_entries[2] = {nullptr, nullptr};
    const int* tc_off[2] = {nullptr, nullptr};
    const uint64_t* tc_tiles[2] = {nullptr, nullptr};
    int tc_clusters[2] = {0, 0};
};

namespace {

// Host tables of a plan, copied to the workspace in one pass.
struct GroupBuild {
    std::vector<KmG> km;
    std::vector<QstatsG<float>> qs;
    std::vector<BstepG> bs;
    std::vector<MixG<float>> mix;
    std::vector<AdjG<float>> adj;
    std::vector<int> off[GS_N];
    std::vector<TcGroupGemm> gemm[2];
};

int group_create(const bgb_acq_t* acqs, const int64_t* b, int count, const double* const* X,
                 double* const* value, double* const* grad, int32_t* const* status,
                 void* workspace, size_t workspace_bytes, cudaStream_t st, bgb_group** out) {
    if (acqs == nullptr || b == nullptr || count <= 0 || X == nullptr || value == nullptr ||
        grad == nullptr || status == nullptr || out == nullptr)
        return BGB_ERR_ARG;
    for (int i = 0; i < count; ++i) {
        int rc = group_member_ok(&acqs[i], b[i]);
        if (rc) return rc;
        if (X[i] == nullptr || value[i] == nullptr || grad[i] == nullptr || status[i] == nullptr)
            return BGB_ERR_ARG;
    }
    const GroupSizes z = group_sizes(acqs, b, count);
    if (workspace == nullptr || workspace_bytes < z.total) return BGB_ERR_WORKSPACE;
    char* base = static_cast<char*>(workspace);
    auto g = std::make_unique<bgb_group>();
    g->count = count;
    GroupBuild hb;
    for (int s = 0; s < GS_N; ++s) hb.off[s].assign((size_t)count + 1, 0);
    // tables after the arenas
    Arena tar{base + z.arenas, z.total - z.arenas, 0};
    g->err = tar.take<int>(1);
    KmG* d_km = tar.take<KmG>(count);
    QstatsG<float>* d_qs = tar.take<QstatsG<float>>(count);
    BstepG* d_bs = tar.take<BstepG>(count);
    MixG<float>* d_mix = tar.take<MixG<float>>(count);
    AdjG<float>* d_adj = tar.take<AdjG<float>>(count);
    int* d_off[GS_N];
    for (int s = 0; s < GS_N; ++s) d_off[s] = tar.take<int>(count + 1);
    void* d_tc_ent[2];
    int* d_tc_off[2];
    for (int k = 0; k < 2; ++k) {
        d_tc_ent[k] = tar.take<unsigned char>(count * tc_group_entry_bytes());
        d_tc_off[k] = tar.take<int>(256);
    }
    uint64_t* d_tc_tiles[2] = {tar.take<uint64_t>(z.tiles_fwd), tar.take<uint64_t>(z.tiles_adj)};
    int* d_boff[kDBuckets];
    for (int k = 0; k < kDBuckets; ++k) d_boff[k] = tar.take<int>(count + 1);
    if (d_boff[kDBuckets - 1] == nullptr) return BGB_ERR_WORKSPACE;
    // per model: arena, arguments, CTA counts
    int64_t total_b = 0;
    for (int i = 0; i < count; ++i) total_b += b[i];
    size_t aoff = 0;
    int64_t c[GS_N] = {};
    for (int i = 0; i < count; ++i) {
        const bgb_acq_t* a = &acqs[i];
        const size_t asz = align_up(acq_ws_layout(a, b[i], nullptr, nullptr, nullptr, nullptr, nullptr));
        Arena ar{base + aoff, asz, 0};
        aoff += asz;
        QBatchArgs qa;
        memset(&qa, 0, sizeof(qa));
        void *Kc = nullptr, *C = nullptr, *P = nullptr;
        if (acq_ws_layout(a, b[i], &ar, &qa, &Kc, &C, &P, nullptr) == 0) return BGB_ERR_WORKSPACE;
        fill_qargs(a, X[i], b[i], &qa);
        qa.dev_err = g->err;
        qa.value = value[i];
        qa.grad = grad[i];
        qa.status = status[i];
        const int64_t n = a->gp.n, rows = b[i] * a->q;
        const int d = a->gp.d;
        __half* Khi = static_cast<__half*>(Kc);
        __half* Klo = Khi + rows * a->ldl;
        const float ks = kc_scale(a->gp.outputscale);
        // base samples and incumbents in float32 once: they are fixed for the plan
        int rc = launch_prep_samples(qa, st);
        if (rc) return rc;
        hb.km.push_back(KmG{X[i], a->gp.inv_lengthscale, qa.zt, rows, d, a->gp.kernel, a->Xs32, n,
                            a->gp.outputscale, Khi, Klo, ks, a->ldl, kernel_matrix_col_tiles(n)});
        const int64_t km_ctas = kernel_matrix_col_tiles(n) * kernel_matrix_row_tiles(rows);
        hb.gemm[0].push_back(TcGroupGemm{rows, n, n, Khi, Klo, a->ldl,
                                         reinterpret_cast<const __half*>(a->Lhi),
                                         reinterpret_cast<const __half*>(a->Llo), a->ldl,
                                         static_cast<float*>(C), a->ldb, KB_UPPER, nullptr, 1.f / ks,
                                         a->Lmul});
        auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) % 16) == 0; };
        const int vec_ok = (a->ldb % 4 == 0) && (n % 4 == 0) && al16(C) && al16(a->beta32) &&
                           (a->r == 0 || al16(a->Vb32));
        hb.qs.push_back(QstatsG<float>{qa, static_cast<const float*>(C), a->ldb, a->beta32,
                                       a->Vb32, vec_ok});
        hb.bs.push_back(BstepG{qa, 1});
        const int64_t mgx = mix_rows_groups(qa, 1, total_b);
        hb.mix.push_back(MixG<float>{qa, static_cast<const float*>(C), a->ldb, a->Vb32, a->beta32,
                                     nullptr, Khi, Klo, a->ldl, mgx});
        hb.gemm[1].push_back(TcGroupGemm{rows, n, n, Khi, Klo, a->ldl,
                                         reinterpret_cast<const __half*>(a->LThi),
                                         reinterpret_cast<const __half*>(a->LTlo), a->ldl,
                                         static_cast<float*>(C), a->ldb, KB_LOWER, qa.hmul, 1.f,
                                         a->LTmul});
        int64_t rb, nslab, slab;
        adjoint_split(qa, kc_region_elems(a, rows), &rb, &nslab, &slab);
        // slab partials (d x rows per slab) go to the Kc region, which holds rows x ldl
        if ((int64_t)d * rows > kc_region_elems(a, rows)) return BGB_ERR_UNSUPPORTED;
        hb.adj.push_back(AdjG<float>{qa, static_cast<const float*>(C), a->ldb, a->Xs32, slab,
                                     static_cast<float*>(Kc), rb, (int)nslab});
        if (nslab > 1) g->partials = true;
        const int64_t per[GS_N] = {ceil_div(rows * d, (int64_t)256), km_ctas, b[i], b[i], mgx * b[i],
                                   rb * nslab, ceil_div((int64_t)d * rows, (int64_t)256),
                                   ceil_div(rows, (int64_t)128)};
        for (int s = 0; s < GS_N; ++s) {
            c[s] += per[s];
            hb.off[s][i + 1] = (int)c[s];
            if (c[s] > 0x7fffffff) return BGB_ERR_UNSUPPORTED;
        }
        g->qmax = std::max(g->qmax, a->q);
        g->rmax = std::max(g->rmax, a->r);
        g->dmax = std::max(g->dmax, d);
        g->bs_smem = std::max(g->bs_smem, batch_step_f32_smem(a->q, a->r, a->n_samples));
        g->mix_smem = std::max(g->mix_smem, mix_rows_smem_bytes(qa));
    }
    if (!g->partials) {  // one slab everywhere: the adjoint finishes its rows itself
        c[GS_SUM] = c[GS_FIN] = 0;
        for (auto& e : hb.adj) e.part = nullptr;
    }
    // adjoint tables in d-bucket order: one launch per bucket
    std::vector<int> order((size_t)count);
    for (int i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return d_bucket(acqs[x].gp.d) < d_bucket(acqs[y].gp.d);
    });
    std::vector<AdjG<float>> adj_sorted;
    std::vector<int> sum_off(1, 0);
    std::vector<int> boff[kDBuckets];
    int bstart[kDBuckets + 1] = {};
    for (int k = 0, pos = 0; k < kDBuckets; ++k) {
        bstart[k] = pos;
        boff[k].assign(1, 0);
        for (; pos < count && d_bucket(acqs[order[pos]].gp.d) == k; ++pos) {
            const AdjG<float>& e = hb.adj[order[pos]];
            const int64_t rows = e.a.b * e.a.q;
            adj_sorted.push_back(e);
            boff[k].push_back(boff[k].back() + (int)(e.gx * e.nslab));
            sum_off.push_back(sum_off.back() + (int)ceil_div((int64_t)e.a.d * rows, (int64_t)256));
        }
        bstart[k + 1] = pos;
    }
    hb.adj.swap(adj_sorted);
    hb.off[GS_SUM] = sum_off;
    // one finish launch over every model (latency-bound: per-bucket launches cost
    // more than the larger register arrays), in the bucket order of the table
    hb.off[GS_FIN].assign(1, 0);
    for (const auto& e : hb.adj)
        hb.off[GS_FIN].push_back(hb.off[GS_FIN].back() + (int)ceil_div(e.a.b * e.a.q, (int64_t)128));
    // tensor-core tile schedules
    std::vector<unsigned char> ent[2];
    std::vector<int> toff[2];
    std::vector<uint64_t> tiles[2];
    for (int k = 0; k < 2; ++k) {
        int rc = tc_group_build(hb.gemm[k].data(), count, reinterpret_cast<uintptr_t>(d_tc_ent[k]),
                                ent[k], toff[k], tiles[k], g->tc_clusters[k]);
        if (rc) return rc;
        if ((int64_t)tiles[k].size() > (k == 0 ? z.tiles_fwd : z.tiles_adj) || toff[k].size() > 256)
            return BGB_ERR_UNSUPPORTED;
    }
    // upload (pageable host memory: the copies complete before the synchronise below)
    auto up = [&](void* dst, const void* src, size_t bytes) -> int {
        if (bytes == 0) return BGB_OK;
        BGB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
        return BGB_OK;
    };
    int rc = up(d_km, hb.km.data(), sizeof(KmG) * count);
    if (!rc) rc = up(d_qs, hb.qs.data(), sizeof(QstatsG<float>) * count);
    if (!rc) rc = up(d_bs, hb.bs.data(), sizeof(BstepG) * count);
    if (!rc) rc = up(d_mix, hb.mix.data(), sizeof(MixG<float>) * count);
    if (!rc) rc = up(d_adj, hb.adj.data(), sizeof(AdjG<float>) * count);
    for (int s = 0; !rc && s < GS_N; ++s) rc = up(d_off[s], hb.off[s].data(), sizeof(int) * (count + 1));
    for (int k = 0; !rc && k < 2; ++k) {
        rc = up(d_tc_ent[k], ent[k].data(), ent[k].size());
        if (!rc) rc = up(d_tc_off[k], toff[k].data(), sizeof(int) * toff[k].size());
        if (!rc) rc = up(d_tc_tiles[k], tiles[k].data(), sizeof(uint64_t) * tiles[k].size());
    }
    for (int k = 0; !rc && k < kDBuckets; ++k)
        rc = up(d_boff[k], boff[k].data(), sizeof(int) * boff[k].size());
    if (rc) return rc;
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    const void* args[GS_N] = {d_km, d_km, d_qs, d_bs, d_mix, d_adj, d_adj, d_adj};
    for (int s = 0; s < GS_N; ++s) {
        g->tab[s] = GroupTab{count, d_off[s], args[s]};
        g->ctas[s] = c[s];
    }
    for (int k = 0; k < 2; ++k) {
        g->tc_entries[k] = d_tc_ent[k];
        g->tc_off[k] = d_tc_off[k];
        g->tc_tiles[k] = d_tc_tiles[k];
    }
    int nb = 0;
    for (int k = 0; k < kDBuckets; ++k) {
        const int nm = bstart[k + 1] - bstart[k];
        g->adj_tab[k] = GroupTab{nm, d_boff[k], d_adj + bstart[k]};
        g->adj_ctas[k] = nm > 0 ? boff[k].back() : 0;
        nb += nm > 0 ? 1 : 0;
    }
    g->ctas[GS_SUM] = g->partials ? sum_off.back() : 0;
    g->ctas[GS_FIN] = g->partials ? hb.off[GS_FIN].back() : 0;
    g->launches = 7 + nb + (g->partials ? 2 : 0);
    *out = g.release();
    return BGB_OK;
}

int group_run(const bgb_group* g, cudaStream_t st) {
    BGB_CUDA_TRY(cudaMemsetAsync(g->err, 0, sizeof(int), st));
    int rc = launch_kernel_matrix_group(g->tab[GS_SCALE], g->ctas[GS_SCALE], g->tab[GS_KM],
                                        g->ctas[GS_KM], st);
    if (!rc) rc = tc_group_launch(g->tc_entries[0], g->tc_off[0], g->tc_tiles[0], g->tc_clusters[0],
                                  g->err, st);
    if (!rc) rc = launch_qstats_group(g->tab[GS_QSTATS], g->qmax, g->rmax, g->ctas[GS_QSTATS], st);
    if (!rc) rc = launch_batch_step_group(g->tab[GS_BSTEP], g->qmax, g->bs_smem, g->ctas[GS_BSTEP], st);
    if (!rc) rc = launch_mix_rows_group(g->tab[GS_MIX], g->qmax, g->mix_smem, g->ctas[GS_MIX], st);
    if (!rc) rc = tc_group_launch(g->tc_entries[1], g->tc_off[1], g->tc_tiles[1], g->tc_clusters[1],
                                  g->err, st);
    for (int k = 0; !rc && k < kDBuckets; ++k)
        rc = launch_adjoint_group(g->adj_tab[k], kDBound[k], g->partials, g->adj_ctas[k], st);
    if (!rc && g->partials)
        rc = launch_adjoint_finish_group(g->tab[GS_SUM], g->ctas[GS_SUM], g->tab[GS_FIN],
                                         kDBound[d_bucket(g->dmax)], g->ctas[GS_FIN], st);
    return rc;
}

}  // namespace

extern "C" {

int bgb_version(void) { return 200; }

int bgb_kernel_matrix(const bgb_gp_t* gp, const double* X1, int64_t m, const double* X2,
                      int64_t n2, double diag_add, double* K, int64_t ldk, void* stream) {
    if (!valid_gp(gp) || X1 == nullptr || X2 == nullptr || K == nullptr || m < 0 || n2 < 0 ||
        ldk < n2)
        return BGB_ERR_ARG;
    return launch_kernel_matrix<double, double, double>(X1, m, X2, n2, gp->d, gp->inv_lengthscale,
                                                        gp->outputscale, gp->kernel, diag_add,
                                                        X1 == X2, K, ldk, as_stream(stream));
}

size_t bgb_cholesky_workspace_bytes(int64_t n) {
    (void)n;
    return align_up(64 * 64 * sizeof(double)) + align_up(2 * sizeof(int));
}

int bgb_cholesky(double* A, int64_t n, int64_t lda, int32_t* info_host, void* workspace,
                 size_t workspace_bytes, void* stream) {
    if (A == nullptr || n <= 0 || lda < n || info_host == nullptr) return BGB_ERR_ARG;
    if (workspace == nullptr || workspace_bytes < bgb_cholesky_workspace_bytes(n))
        return BGB_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    double* dws = ar.take<double>(64 * 64);
    int* dinfo = ar.take<int>(2);
    int rc = cholesky_f64(A, n, lda, dinfo, dws, st);
    if (rc) return rc;
    int hinfo[2] = {0, 0};
    BGB_CUDA_TRY(cudaMemcpyAsync(hinfo, dinfo, sizeof(hinfo), cudaMemcpyDeviceToHost, st));
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    *info_host = hinfo[0];
    return hinfo[0] == 0 ? BGB_OK : BGB_NOT_PSD;
}

int bgb_psd_safe_cholesky(const double* A, int64_t n, int64_t lda, double* L, int64_t ldl,
                          int32_t max_tries, double jitter, double* jitter_host, void* workspace,
                          size_t workspace_bytes, void* stream) {
    if (A == nullptr || L == nullptr || n <= 0 || lda < n || ldl < n || max_tries < 0)
        return BGB_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    if (jitter <= 0.0) jitter = 1e-8;
    double total = 0.0;
    int32_t info = 0;
    for (int t = -1; t < max_tries; ++t) {
        if (t >= 0) total = jitter * pow(10.0, (double)t);
        int rc = copy_matrix_f64(A, lda, L, ldl, n, n, total, st);
        if (rc) return rc;
        rc = bgb_cholesky(L, n, ldl, &info, workspace, workspace_bytes, stream);
        if (rc == BGB_OK) {
            if (jitter_host) *jitter_host = total;
            return BGB_OK;
        }
        if (rc != BGB_NOT_PSD) return rc;
    }
    if (jitter_host) *jitter_host = total;
    return BGB_NOT_PSD;
}

size_t bgb_tri_inverse_workspace_bytes(int64_t n) {
    return align_up(sizeof(double) * (size_t)tri_inverse_ws_doubles(n));
}

int bgb_tri_inverse(double* L, int64_t n, int64_t lda, void* workspace, size_t workspace_bytes,
                    void* stream) {
    if (L == nullptr || n <= 0 || lda < n) return BGB_ERR_ARG;
    if (workspace == nullptr || workspace_bytes < bgb_tri_inverse_workspace_bytes(n))
        return BGB_ERR_WORKSPACE;
    return tri_inverse_f64(L, n, lda, static_cast<double*>(workspace), as_stream(stream));
}

size_t bgb_gp_fit_workspace_bytes(int64_t n) {
    return align_up(sizeof(double) * n * n) + bgb_cholesky_workspace_bytes(n) +
           bgb_tri_inverse_workspace_bytes(n) + 3 * align_up(sizeof(double) * n);
}

int bgb_gp_fit(const bgb_gp_t* gp, const double* y, double noise, int32_t max_tries, double* L,
               double* Linv, double* alpha, double* beta, double* jitter_host, void* workspace,
               size_t workspace_bytes, void* stream) {
    if (!valid_gp(gp) || y == nullptr || L == nullptr || Linv == nullptr || alpha == nullptr ||
        beta == nullptr)
        return BGB_ERR_ARG;
    const int64_t n = gp->n;
    if (workspace == nullptr || workspace_bytes < bgb_gp_fit_workspace_bytes(n))
        return BGB_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    double* K = ar.take<double>(n * n);
    void* chol_ws = ar.take<char>(bgb_cholesky_workspace_bytes(n));
    double* tri_ws = ar.take<double>(bgb_tri_inverse_workspace_bytes(n) / sizeof(double));
    double* yc = ar.take<double>(n);
    double* res = ar.take<double>(n);
    double* t = ar.take<double>(n);
    // K = k(Xt, Xt) + noise I
    int rc = launch_kernel_matrix<double, double, double>(gp->train_X, n, gp->train_X, n, gp->d,
                                                          gp->inv_lengthscale, gp->outputscale,
                                                          gp->kernel, noise, 1, K, n, st);
    if (rc) return rc;
    double jit = 0.0;
    rc = bgb_psd_safe_cholesky(K, n, n, L, n, max_tries, 1e-8, &jit, chol_ws,
                               bgb_cholesky_workspace_bytes(n), stream);
    if (rc) return rc;
    if (jitter_host) *jitter_host = jit;
    // Linv = L^-1
    rc = copy_matrix_f64(L, n, Linv, n, n, n, 0.0, st);
    if (rc) return rc;
    rc = tri_inverse_f64(Linv, n, n, tri_ws, st);
    if (rc) return rc;
    // alpha = Linv^T (Linv (y - m)), then one refinement step against K_eff = K + jitter I
    sub_const_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(y, gp->mean_constant, yc, n);
    BGB_CHECK_LAUNCH();
    rc = gemv_f64(n, n, 1.0, Linv, n, yc, 0.0, t, st);
    if (rc) return rc;
    rc = gemv_t_f64(n, n, 1.0, Linv, n, t, 0.0, alpha, st);
    if (rc) return rc;
    if (jit > 0.0) {
        rc = launch_kernel_matrix<double, double, double>(gp->train_X, n, gp->train_X, n, gp->d,
                                                          gp->inv_lengthscale, gp->outputscale,
                                                          gp->kernel, noise + jit, 1, K, n, st);
        if (rc) return rc;
    }
    // res = yc - K alpha;  alpha += Linv^T (Linv res)
    BGB_CUDA_TRY(cudaMemcpyAsync(res, yc, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    rc = gemv_f64(n, n, -1.0, K, n, alpha, 1.0, res, st);
    if (rc) return rc;
    rc = gemv_f64(n, n, 1.0, Linv, n, res, 0.0, t, st);
    if (rc) return rc;
    rc = gemv_t_f64(n, n, 1.0, Linv, n, t, 1.0, alpha, st);
    if (rc) return rc;
    // beta = L^T alpha (= L^-1 (y - m) for the refined alpha)
    rc = gemv_t_f64(n, n, 1.0, L, n, alpha, 0.0, beta, st);
    if (rc) return rc;
    BGB_CUDA_TRY(cudaStreamSynchronize(st));
    return BGB_OK;
}

int bgb_gp_operands(const bgb_gp_t* gp, const double* Linv, const double* beta, double* B64,
                    float* B32, int64_t ldb, float* Linv32, float* beta32, double* Xs64,
                    float* Xs32, void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || beta == nullptr || B64 == nullptr || Xs64 == nullptr)
        return BGB_ERR_ARG;
    const int64_t n = gp->n;
    if (ldb < n) return BGB_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    fill_b_kernel<<<(unsigned)ceil_div(n * ldb, 256), 256, 0, st>>>(Linv, n, B64, ldb);
    BGB_CHECK_LAUNCH();
    int rc;
    if (B32 != nullptr && (rc = convert_f64_f32(B64, B32, n * ldb, st)) != BGB_OK) return rc;
    if (Linv32 != nullptr && (rc = convert_f64_f32(Linv, Linv32, n * n, st)) != BGB_OK) return rc;
    if (beta32 != nullptr && (rc = convert_f64_f32(beta, beta32, n, st)) != BGB_OK) return rc;
    scale_inputs_kernel<<<(unsigned)ceil_div(n * gp->d, 256), 256, 0, st>>>(
        gp->train_X, gp->inv_lengthscale, n, gp->d, Xs64, Xs32);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int bgb_gp_tc_operands(const bgb_gp_t* gp, const double* Linv, int64_t ldl, uint16_t* Lhi,
                       uint16_t* Llo, uint16_t* LThi, uint16_t* LTlo, float* Lmul, float* LTmul,
                       void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || Lhi == nullptr || Llo == nullptr || LThi == nullptr ||
        LTlo == nullptr || Lmul == nullptr || LTmul == nullptr)
        return BGB_ERR_ARG;
    const int64_t n = gp->n;
    if (ldl < n || (ldl % 8) != 0) return BGB_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    int rc = split_f64_f16(Linv, n, n, n, 0, reinterpret_cast<__half*>(Lhi),
                           reinterpret_cast<__half*>(Llo), ldl, Lmul, st);
    if (rc) return rc;
    return split_f64_f16(Linv, n, n, n, 1, reinterpret_cast<__half*>(LThi),
                         reinterpret_cast<__half*>(LTlo), ldl, LTmul, st);
}

int bgb_crosscov_gemm_f16x3(int64_t M, int64_t N, int64_t K, const uint16_t* A_hi,
                            const uint16_t* A_lo, int64_t lda, const uint16_t* B_hi,
                            const uint16_t* B_lo, int64_t ldbs, float* C, int64_t ldc,
                            const float* row_mul, float row_mul_const, const float* col_mul,
                            int32_t kmode, int32_t* err_dev, void* stream) {
    if (M < 0 || N < 0 || K <= 0 || A_hi == nullptr || A_lo == nullptr || B_hi == nullptr ||
        B_lo == nullptr || C == nullptr || col_mul == nullptr || (lda % 8) || (ldbs % 8) ||
        (ldc % 4) || lda < K || ldbs < K || ldc < N)
        return BGB_ERR_ARG;
    if (kmode != KB_UPPER && kmode != KB_LOWER && kmode != KFULL) return BGB_ERR_ARG;
    if (!tc_gemm_available()) return BGB_ERR_UNSUPPORTED;
    return tc_gemm_f16x3(M, N, K, reinterpret_cast<const __half*>(A_hi),
                         reinterpret_cast<const __half*>(A_lo), lda,
                         reinterpret_cast<const __half*>(B_hi), reinterpret_cast<const __half*>(B_lo),
                         ldbs, C, ldc, kmode, row_mul, row_mul_const, col_mul, err_dev,
                         as_stream(stream));
}

size_t bgb_baseline_operands_workspace_bytes(int64_t n, int32_t r) {
    return align_up(sizeof(double) * n * (r > 0 ? r : 1));
}

int bgb_baseline_operands(const bgb_gp_t* gp, const double* Linv, const double* X_baseline,
                          int32_t r, double* Vb64, float* Vb32, double* VbT64, float* VbT32,
                          void* workspace, size_t workspace_bytes, void* stream) {
    if (!valid_gp(gp) || Linv == nullptr || X_baseline == nullptr || r <= 0 || Vb64 == nullptr ||
        VbT64 == nullptr)
        return BGB_ERR_ARG;
    const int64_t n = gp->n;
    if (workspace == nullptr || workspace_bytes < bgb_baseline_operands_workspace_bytes(n, r))
        return BGB_ERR_WORKSPACE;
    cudaStream_t st = as_stream(stream);
    double* Kbt = static_cast<double*>(workspace);
    int rc = launch_kernel_matrix<double, double, double>(X_baseline, r, gp->train_X, n, gp->d,
                                                          gp->inv_lengthscale, gp->outputscale,
                                                          gp->kernel, 0.0, 0, Kbt, n, st);
    if (rc) return rc;
    rc = gemm_f64(r, n, n, 1.0, Kbt, n, 0, Linv, n, 1, 0.0, Vb64, n, KB_UPPER, 0, nullptr, st, n);
    if (rc) return rc;
    rc = transpose_f64(Vb64, r, n, n, VbT64, r, st);
    if (rc) return rc;
    if (Vb32 != nullptr && (rc = convert_f64_f32(Vb64, Vb32, (int64_t)r * n, st)) != BGB_OK)
        return rc;
    if (VbT32 != nullptr && (rc = convert_f64_f32(VbT64, VbT32, (int64_t)r * n, st)) != BGB_OK)
        return rc;
    return BGB_OK;
}

size_t bgb_gp_mll_workspace_bytes(int64_t n, int32_t d) { return mll_workspace_bytes(n, d); }

int bgb_gp_mll(const bgb_gp_t* gp, const double* y, const double* L, const double* Linv,
               const double* alpha, double* out_host, void* workspace, size_t workspace_bytes,
               void* stream) {
    if (!valid_gp(gp) || y == nullptr || L == nullptr || Linv == nullptr || alpha == nullptr ||
        out_host == nullptr)
        return BGB_ERR_ARG;
    if (gp->d > 64) return BGB_ERR_UNSUPPORTED;
    cudaStream_t st = as_stream(stream);
    int rc = gp_mll(gp->train_X, gp->n, gp->d, gp->inv_lengthscale, gp->outputscale, gp->kernel,
                    gp->mean_constant, y, L, Linv, alpha, out_host, workspace, workspace_bytes, st);
    if (rc) return rc;
    double il[64];
    BGB_CUDA_TRY(cudaMemcpy(il, gp->inv_lengthscale, sizeof(double) * gp->d, cudaMemcpyDeviceToHost));
    for (int k = 0; k < gp->d; ++k) out_host[1 + k] *= il[k];  // d r2 / d l_k = -2 dz_k^2 / l_k
    return BGB_OK;
}

size_t bgb_acq_workspace_bytes(const bgb_acq_t* acq, int64_t b) {
    if (acq == nullptr || b <= 0) return 0;
    return acq_ws_layout(acq, b, nullptr, nullptr, nullptr, nullptr, nullptr);
}

int bgb_posterior(const bgb_acq_t* acq, const double* X, int64_t b, double* mean, double* covar,
                  void* workspace, size_t workspace_bytes, void* stream) {
    if (!valid_acq(acq) || X == nullptr || mean == nullptr || covar == nullptr || b < 0 ||
        acq->r != 0)
        return BGB_ERR_ARG;
    if (b == 0) return BGB_OK;
    cudaStream_t st = as_stream(stream);
    Arena ar{static_cast<char*>(workspace), workspace_bytes, 0};
    QBatchArgs qa;
    memset(&qa, 0, sizeof(qa));
    void *Kc = nullptr, *C = nullptr, *P = nullptr;
    int* err = nullptr;
    if (workspace == nullptr || acq_ws_layout(acq, b, &ar, &qa, &Kc, &C, &P, &err) == 0)
        return BGB_ERR_WORKSPACE;
    fill_qargs(acq, X, b, &qa);
    BGB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    qa.dev_err = err;
    int rc;
    if (acq->precision == BGB_PREC_MIXED)
        rc = run_front<float>(acq, X, b, &qa, static_cast<float*>(Kc), static_cast<float*>(C),
                              static_cast<float*>(P), st, nullptr);
    else
        rc = run_front<double>(acq, X, b, &qa, static_cast<double*>(Kc), static_cast<double*>(C),
                               static_cast<double*>(P), st, nullptr);
    if (rc) return rc;
    return launch_posterior_out(qa, mean, covar, st);
}

int bgb_acq_forward(const bgb_acq_t* acq, const double* X, int64_t b, double* value,
                    int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
    return acq_call(acq, X, b, value, nullptr, status, workspace, workspace_bytes,
                    as_stream(stream));
}

int bgb_acq_forward_backward(const bgb_acq_t* acq, const double* X, int64_t b, double* value,
                             double* grad, int32_t* status, void* workspace,
                             size_t workspace_bytes, void* stream) {
    if (grad == nullptr) return BGB_ERR_ARG;
    return acq_call(acq, X, b, value, grad, status, workspace, workspace_bytes,
                    as_stream(stream));
}

int bgb_acq_forward_backward_noalloc(const bgb_acq_t* acq, const double* X, int64_t b,
                                     double* value, double* grad, int32_t* status, void* stream) {
    if (!valid_acq(acq) || X == nullptr || value == nullptr || grad == nullptr ||
        status == nullptr || b < 0)
        return BGB_ERR_ARG;
    if (b == 0) return BGB_OK;
    // size check first: an oversized call launches nothing and touches no device
    if (acq_ws_layout(acq, b, nullptr, nullptr, nullptr, nullptr, nullptr) >
        BGB_NOALLOC_SCRATCH_BYTES)
        return BGB_ERR_SCRATCH_LIMIT;
    void* scratch = nullptr;
    int rc = noalloc_scratch(as_stream(stream), &scratch);
    if (rc) return rc;
    // acq_call clears the device error word on `stream` before its first launch
    return acq_call(acq, X, b, value, grad, status, scratch, BGB_NOALLOC_SCRATCH_BYTES,
                    as_stream(stream));
}

unsigned long long bgb_launch_count(void) { return g_launches.load(); }

int bgb_acq_forward_backward_timed(const bgb_acq_t* acq, const double* X, int64_t b,
                                   double* value, double* grad, int32_t* status, void* workspace,
                                   size_t workspace_bytes, float* stage_ms_host, void* stream) {
    if (grad == nullptr || stage_ms_host == nullptr) return BGB_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    cudaEvent_t ev[kStages + 1];
    for (int i = 0; i <= kStages; ++i) BGB_CUDA_TRY(cudaEventCreate(&ev[i]));
    int rc = acq_call(acq, X, b, value, grad, status, workspace, workspace_bytes, st, ev);
    if (rc == BGB_OK) {
        if (cudaEventSynchronize(ev[kStages]) != cudaSuccess) rc = BGB_ERR_CUDA;
        for (int i = 0; rc == BGB_OK && i < kStages; ++i)
            if (cudaEventElapsedTime(&stage_ms_host[i], ev[i], ev[i + 1]) != cudaSuccess)
                rc = BGB_ERR_CUDA;
    }
    for (int i = 0; i <= kStages; ++i) cudaEventDestroy(ev[i]);
    return rc;
}

size_t bgb_group_workspace_bytes(const bgb_acq_t* acqs, const int64_t* b, int32_t count) {
    if (acqs == nullptr || b == nullptr || count <= 0) return 0;
    for (int i = 0; i < count; ++i)
        if (group_member_ok(&acqs[i], b[i]) != BGB_OK) return 0;
    return group_sizes(acqs, b, count).total;
}

int bgb_group_create(const bgb_acq_t* acqs, const int64_t* b, int32_t count,
                     const double* const* X, double* const* value, double* const* grad,
                     int32_t* const* status, void* workspace, size_t workspace_bytes, void* stream,
                     bgb_group_t** out) {
    try {
        return group_create(acqs, b, count, X, value, grad, status, workspace, workspace_bytes,
                            as_stream(stream), out);
    } catch (const std::bad_alloc&) {
        return BGB_ERR_ARG;
    }
}

int bgb_group_run(const bgb_group_t* group, void* stream) {
    if (group == nullptr) return BGB_ERR_ARG;
    return group_run(group, as_stream(stream));
}

int32_t bgb_group_launches(const bgb_group_t* group) { return group ? group->launches : 0; }

void bgb_group_destroy(bgb_group_t* group) { delete group; }

}  // extern "C"
