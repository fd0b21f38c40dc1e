// Batched L-BFGS-B on the device: launches and C ABI.
//
// One CTA per restart advances that restart's optimiser (lbfgsb_core.cuh)
// between two evaluations of the objective, so that the per-restart mode of
// the reference's optimiser (botorch/generation/gen.py:226-247 with
// botorch/optim/batched_lbfgs_b.py:169-636) keeps its points, gradients and
// limited-memory pairs in HBM and needs no host round trip per round but a
// four-integer summary.
#include <cuda_runtime.h>

#include <atomic>

#include "bgb_common.cuh"
#include "lbfgsb_core.cuh"

namespace bgb {
namespace {

using bgb_lb::Layout;

__global__ void __launch_bounds__(LB_NT) lbfgsb_init_kernel(const __grid_constant__ bgb_lb::InitArgs a) {
    __shared__ bgb_lb::Shm sh;
    bgb_lb::init_restart(a, blockIdx.x, sh);
}

__global__ void __launch_bounds__(LB_NT) lbfgsb_step_kernel(const __grid_constant__ bgb_lb::StepArgs a, int n2) {
    __shared__ bgb_lb::Shm sh;
    extern __shared__ __align__(16) unsigned char lb_dyn[];
    bgb_lb::step_restart(a, blockIdx.x, sh, lb_dyn, n2);
}

__global__ void __launch_bounds__(LB_NT)
    lbfgsb_summary_kernel(Layout L, const char* ws, long long R, int* out) {
    __shared__ bgb_lb::Shm sh;
    bgb_lb::summarize(L, ws, R, sh, out);
}

__global__ void lbfgsb_results_kernel(Layout L, const char* ws, long long R, double* f, int64_t* nit,
                                      int64_t* nfev, int32_t* code) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const bgb_lb::State& s = reinterpret_cast<const bgb_lb::State*>(ws + L.states)[r];
    if (f) f[r] = s.f;
    if (nit) nit[r] = s.nit;
    if (nfev) nfev[r] = s.nfev;
    if (code) code[r] = s.code;
}

int check_opts(const bgb_lbfgsb_opts* o) {
    if (o == nullptr || o->restarts < 1 || o->n < 1 || o->m < 1 || o->maxls < 1 || o->maxiter < 0 ||
        o->maxfun < 0 || !(o->factr >= 0.0) || !(o->pgtol >= 0.0))
        return BGB_ERR_ARG;
    if (o->n > bgb_lb::kMaxN || o->m > bgb_lb::kMaxM || o->restarts > (1LL << 30)) return BGB_ERR_UNSUPPORTED;
    return BGB_OK;
}

Layout layout_of(const bgb_lbfgsb_opts* o) { return bgb_lb::make_layout(o->restarts, o->n, o->m); }

size_t step_smem_bytes(int n2) { return (size_t)bgb_lb::step_dyn_bytes(n2); }

// The step's static plus dynamic shared memory exceeds the default 48 KB: allow
// the largest size (n = kMaxN) once per device, outside any stream work.
bool allow_step_smem() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    const unsigned long long bit = 1ULL << dev;
    if (done.load() & bit) return true;
    const int bytes = (int)step_smem_bytes(bgb_lb::sort_len(bgb_lb::kMaxN));
    if (cudaFuncSetAttribute(lbfgsb_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
        cudaSuccess)
        return false;
    done.fetch_or(bit);
    return true;
}

}  // namespace
}  // namespace bgb

extern "C" {

size_t bgb_lbfgsb_workspace_bytes(const bgb_lbfgsb_opts* o) {
    if (bgb::check_opts(o) != BGB_OK) return 0;
    return (size_t)bgb::layout_of(o).total;
}

int bgb_lbfgsb_init(const bgb_lbfgsb_opts* o, double* X, const double* lower, const double* upper, void* ws,
                    size_t ws_bytes, void* stream) {
    int rc = bgb::check_opts(o);
    if (rc != BGB_OK) return rc;
    if (X == nullptr || lower == nullptr || upper == nullptr || ws == nullptr) return BGB_ERR_ARG;
    const bgb_lb::Layout L = bgb::layout_of(o);
    if (ws_bytes < (size_t)L.total) return BGB_ERR_WORKSPACE;
    bgb_lb::InitArgs a;
    a.L = L;
    a.R = o->restarts;
    a.n = (int)o->n;
    a.m = o->m;
    a.ws = static_cast<char*>(ws);
    a.X = X;
    a.lo = lower;
    a.hi = upper;
    if (!bgb::allow_step_smem()) return BGB_ERR_CUDA;
    bgb::lbfgsb_init_kernel<<<(unsigned)o->restarts, LB_NT, 0, static_cast<cudaStream_t>(stream)>>>(a);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int bgb_lbfgsb_step(const bgb_lbfgsb_opts* o, double* X, const double* value, double sign, const double* grad,
                    const int32_t* status, int32_t ignore_status, void* ws, size_t ws_bytes, int32_t* summary,
                    void* stream) {
    int rc = bgb::check_opts(o);
    if (rc != BGB_OK) return rc;
    if (X == nullptr || value == nullptr || grad == nullptr || ws == nullptr) return BGB_ERR_ARG;
    const bgb_lb::Layout L = bgb::layout_of(o);
    if (ws_bytes < (size_t)L.total) return BGB_ERR_WORKSPACE;
    bgb_lb::StepArgs a;
    a.L = L;
    a.R = o->restarts;
    a.n = (int)o->n;
    a.m = o->m;
    a.maxls = o->maxls;
    a.maxiter = o->maxiter;
    a.maxfun = o->maxfun;
    a.factr = o->factr;
    a.pgtol = o->pgtol;
    a.ws = static_cast<char*>(ws);
    a.X = X;
    a.value = value;
    a.sign = sign;
    a.grad = grad;
    a.status = status;
    a.ignore_status = ignore_status;
    const int n2 = bgb_lb::sort_len(a.n);
    const size_t smem = bgb::step_smem_bytes(n2);
    if (!bgb::allow_step_smem()) return BGB_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bgb::lbfgsb_step_kernel<<<(unsigned)o->restarts, LB_NT, smem, s>>>(a, n2);
    BGB_CHECK_LAUNCH();
    if (summary != nullptr) {
        bgb::lbfgsb_summary_kernel<<<1, LB_NT, 0, s>>>(L, static_cast<const char*>(ws), o->restarts, summary);
        BGB_CHECK_LAUNCH();
    }
    return BGB_OK;
}

int bgb_lbfgsb_results(const bgb_lbfgsb_opts* o, const void* ws, size_t ws_bytes, double* f, int64_t* nit,
                       int64_t* nfev, int32_t* code, void* stream) {
    int rc = bgb::check_opts(o);
    if (rc != BGB_OK) return rc;
    if (ws == nullptr) return BGB_ERR_ARG;
    const bgb_lb::Layout L = bgb::layout_of(o);
    if (ws_bytes < (size_t)L.total) return BGB_ERR_WORKSPACE;
    const unsigned blocks = (unsigned)((o->restarts + 255) / 256);
    bgb::lbfgsb_results_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        L, static_cast<const char*>(ws), o->restarts, f, nit, nfev, code);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

}  // extern "C"
