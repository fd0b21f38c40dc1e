// Thin torch extension over the C ABI (include/botorch_gb300.h): the library's
// entry points for the hot path registered as dispatcher operators in the
// namespace botorch_gb300, with CUDA kernels only (no CPU implementation is
// registered, so CPU tensors raise in the dispatcher).
//
//   acq_forward_backward(acq, X, value!, grad!, status!, workspace!) -> int
//   acq_forward(acq, X, value!, status!, workspace!) -> int
//       the MC acquisition forward (and adjoint) on a b x q x d tensor, the
//       call botorch/generation/gen.py:466-469 makes through autograd; `acq` is
//       the packed bgb_acq_t (a CPU uint8 tensor); returns the C ABI's code.
//   log_areas_forward(obj, cell_lower, cell_upper, tau_relu, tau_max) -> Tensor
//   log_areas_backward(grad_out, obj, cell_lower, cell_upper, tau_relu, tau_max) -> Tensor
//       the contract of the reference's fused extension (botorch/csrc/logei_fused.cpp:
//       fused_log_areas_forward :184-264, fused_log_areas_backward :266-374, bound
//       as _C.forward / _C.backward at botorch/acquisition/multi_objective/logei.py:65-104),
//       with the same argument checks and messages.
//
// Built by botorch_gb300/build.py with the host compiler and torch's headers;
// loaded with torch.ops.load_library.
#include <ATen/ATen.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/library.h>

#include <cstring>

#include "botorch_gb300.h"

namespace {

constexpr int64_t kMaxI = 32;  // the reference's MAX_I
constexpr int64_t kMaxM = 8;   // the reference's MAX_M

void* stream_of(const at::Tensor& t) { return c10::cuda::getCurrentCUDAStream(t.device().index()).stream(); }

bgb_acq_t unpack_acq(const at::Tensor& acq) {
    TORCH_CHECK(acq.device().is_cpu() && acq.scalar_type() == at::kByte && acq.is_contiguous() &&
                    acq.numel() == (int64_t)sizeof(bgb_acq_t),
                "acq must be the packed bgb_acq_t as a contiguous CPU uint8 tensor of ", sizeof(bgb_acq_t),
                " bytes");
    bgb_acq_t a;
    std::memcpy(&a, acq.data_ptr(), sizeof(bgb_acq_t));
    return a;
}

void check_cuda_f64(const at::Tensor& t, const char* what) {
    TORCH_CHECK(t.is_cuda() && t.scalar_type() == at::kDouble && t.is_contiguous(), what,
                " must be a contiguous float64 CUDA tensor");
}

int64_t acq_forward_backward(const at::Tensor& acq, const at::Tensor& X, const at::Tensor& value,
                             const at::Tensor& grad, const at::Tensor& status, const at::Tensor& workspace) {
    const bgb_acq_t a = unpack_acq(acq);
    check_cuda_f64(X, "X");
    check_cuda_f64(value, "value");
    check_cuda_f64(grad, "grad");
    TORCH_CHECK(X.dim() == 3 && grad.sizes() == X.sizes() && value.numel() == X.size(0), "shape mismatch");
    TORCH_CHECK(status.is_cuda() && status.scalar_type() == at::kInt && status.numel() == X.size(0),
                "status must be an int32 CUDA tensor of b entries");
    TORCH_CHECK(workspace.is_cuda() && workspace.is_contiguous(), "workspace must be a contiguous CUDA tensor");
    const c10::cuda::CUDAGuard guard(X.device());
    return bgb_acq_forward_backward(&a, X.data_ptr<double>(), X.size(0), value.data_ptr<double>(),
                                    grad.data_ptr<double>(), status.data_ptr<int32_t>(), workspace.data_ptr(),
                                    (size_t)workspace.nbytes(), stream_of(X));
}

int64_t acq_forward(const at::Tensor& acq, const at::Tensor& X, const at::Tensor& value, const at::Tensor& status,
                    const at::Tensor& workspace) {
    const bgb_acq_t a = unpack_acq(acq);
    check_cuda_f64(X, "X");
    check_cuda_f64(value, "value");
    TORCH_CHECK(X.dim() == 3 && value.numel() == X.size(0), "shape mismatch");
    TORCH_CHECK(status.is_cuda() && status.scalar_type() == at::kInt && status.numel() == X.size(0),
                "status must be an int32 CUDA tensor of b entries");
    TORCH_CHECK(workspace.is_cuda() && workspace.is_contiguous(), "workspace must be a contiguous CUDA tensor");
    const c10::cuda::CUDAGuard guard(X.device());
    return bgb_acq_forward(&a, X.data_ptr<double>(), X.size(0), value.data_ptr<double>(),
                           status.data_ptr<int32_t>(), workspace.data_ptr(), (size_t)workspace.nbytes(),
                           stream_of(X));
}

struct Cells {
    at::Tensor obj, cl, cu;
    int64_t B, n_sub, isz, m, B_cells, nc;
};

// The argument checks of the reference's extension, for CUDA tensors.
Cells prepare(const at::Tensor& obj_subsets, const at::Tensor& cell_lower, const at::Tensor& cell_upper) {
    Cells c;
    c.obj = obj_subsets.contiguous();
    c.cl = cell_lower.contiguous();
    c.cu = cell_upper.contiguous();
    TORCH_CHECK(c.obj.dim() == 4, "obj_subsets must be 4-D");
    TORCH_CHECK((c.cl.dim() == 2 || c.cl.dim() == 3) && c.cl.dim() == c.cu.dim(), "cell bounds must be 2-D or 3-D");
    c.B = c.obj.size(0);
    c.n_sub = c.obj.size(1);
    c.isz = c.obj.size(2);
    c.m = c.obj.size(3);
    TORCH_CHECK(c.isz <= kMaxI && c.m <= kMaxM, "subset_size or m too large");
    TORCH_CHECK(c.obj.is_cuda(), "fused log-areas: the inputs must be CUDA tensors (no CPU path)");
    TORCH_CHECK(c.obj.scalar_type() == at::kDouble || c.obj.scalar_type() == at::kFloat,
                "fused log-areas: unsupported dtype");
    TORCH_CHECK(c.cl.scalar_type() == c.obj.scalar_type() && c.cu.scalar_type() == c.obj.scalar_type() &&
                    c.cl.device() == c.obj.device() && c.cu.device() == c.obj.device(),
                "fused log-areas: cell bounds must match obj_subsets in dtype and device");
    TORCH_CHECK(c.cl.sizes() == c.cu.sizes() && c.cl.size(-1) == c.m,
                "fused log-areas: cell bounds must be (..., num_cells, m) and of equal shape");
    c.B_cells = c.cl.dim() == 3 ? c.cl.size(0) : 1;
    c.nc = c.cl.size(-2);
    TORCH_CHECK(c.cl.dim() == 2 || c.B_cells == c.B,
                "fused log-areas: batched cell bounds need one batch per obj_subsets batch");
    return c;
}

// The C ABI's argument and launch errors, named as the Python layer names them.
void check_rc(int rc, const char* what) {
    const char* name = rc == BGB_ERR_ARG           ? "invalid argument"
                       : rc == BGB_ERR_WORKSPACE   ? "workspace too small"
                       : rc == BGB_ERR_CUDA        ? "CUDA error"
                       : rc == BGB_ERR_UNSUPPORTED ? "unsupported size"
                                                   : "error";
    TORCH_CHECK(rc == BGB_OK, what, ": ", name, " (code ", rc, ")");
}

at::Tensor log_areas_forward(const at::Tensor& obj_subsets, const at::Tensor& cell_lower,
                             const at::Tensor& cell_upper, double tau_relu, double tau_max) {
    Cells c = prepare(obj_subsets, cell_lower, cell_upper);
    const c10::cuda::CUDAGuard guard(c.obj.device());
    at::Tensor out = at::empty({c.B, c.nc, c.n_sub}, c.obj.options());
    int rc;
    if (c.obj.scalar_type() == at::kDouble)
        rc = bgb_log_areas_forward(c.obj.data_ptr<double>(), c.B, c.n_sub, c.isz, c.m, c.cl.data_ptr<double>(),
                                   c.cu.data_ptr<double>(), c.B_cells, c.nc, tau_relu, tau_max,
                                   out.data_ptr<double>(), stream_of(c.obj));
    else
        rc = bgb_log_areas_forward_f32(c.obj.data_ptr<float>(), c.B, c.n_sub, c.isz, c.m, c.cl.data_ptr<float>(),
                                       c.cu.data_ptr<float>(), c.B_cells, c.nc, tau_relu, tau_max,
                                       out.data_ptr<float>(), stream_of(c.obj));
    check_rc(rc, "bgb_log_areas_forward");
    return out;
}

at::Tensor log_areas_backward(const at::Tensor& grad_out, const at::Tensor& obj_subsets, const at::Tensor& cell_lower,
                              const at::Tensor& cell_upper, double tau_relu, double tau_max) {
    Cells c = prepare(obj_subsets, cell_lower, cell_upper);
    at::Tensor g = grad_out.contiguous();
    TORCH_CHECK(g.dim() == 3 && g.size(0) == c.B && g.size(1) == c.nc && g.size(2) == c.n_sub,
                "fused log-areas: grad_out must be (B, num_cells, n_sub)");
    TORCH_CHECK(g.scalar_type() == c.obj.scalar_type() && g.device() == c.obj.device(),
                "fused log-areas: grad_out must match obj_subsets in dtype and device");
    const c10::cuda::CUDAGuard guard(c.obj.device());
    at::Tensor grad_obj = at::empty_like(c.obj);
    int rc;
    if (c.obj.scalar_type() == at::kDouble)
        rc = bgb_log_areas_backward(g.data_ptr<double>(), c.obj.data_ptr<double>(), c.B, c.n_sub, c.isz, c.m,
                                    c.cl.data_ptr<double>(), c.cu.data_ptr<double>(), c.B_cells, c.nc, tau_relu,
                                    tau_max, grad_obj.data_ptr<double>(), stream_of(c.obj));
    else
        rc = bgb_log_areas_backward_f32(g.data_ptr<float>(), c.obj.data_ptr<float>(), c.B, c.n_sub, c.isz, c.m,
                                        c.cl.data_ptr<float>(), c.cu.data_ptr<float>(), c.B_cells, c.nc, tau_relu,
                                        tau_max, grad_obj.data_ptr<float>(), stream_of(c.obj));
    check_rc(rc, "bgb_log_areas_backward");
    return grad_obj;
}

}  // namespace

TORCH_LIBRARY(botorch_gb300, m) {
    m.def("acq_forward_backward(Tensor acq, Tensor X, Tensor(a!) value, Tensor(b!) grad, Tensor(c!) status, "
          "Tensor(d!) workspace) -> int");
    m.def("acq_forward(Tensor acq, Tensor X, Tensor(a!) value, Tensor(b!) status, Tensor(c!) workspace) -> int");
    m.def("log_areas_forward(Tensor obj_subsets, Tensor cell_lower, Tensor cell_upper, float tau_relu, "
          "float tau_max) -> Tensor");
    m.def("log_areas_backward(Tensor grad_out, Tensor obj_subsets, Tensor cell_lower, Tensor cell_upper, "
          "float tau_relu, float tau_max) -> Tensor");
}

TORCH_LIBRARY_IMPL(botorch_gb300, CUDA, m) {
    m.impl("acq_forward_backward", &acq_forward_backward);
    m.impl("acq_forward", &acq_forward);
    m.impl("log_areas_forward", &log_areas_forward);
    m.impl("log_areas_backward", &log_areas_backward);
}
