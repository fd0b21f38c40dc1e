// Scrambled Sobol points mapped to a box, on the device: the raw samples of the
// acquisition optimisation (botorch/utils/sampling.py:74-111, draw_sobol_samples,
// which draws torch.quasirandom.SobolEngine(q * d, scramble=True, seed) on the
// host and maps [0, 1) to the bounds).
//
// The engine's state (its scrambled direction numbers, the digital shift and
// its first point as it returns it) is built by torch on the host; point k >= 1
// of the sequence is shift XOR the direction numbers of the bits of the Gray
// code of k, times 2^-maxbit (the engine's recursion adds one direction number
// per step, rightmost zero bit of the step index, which reaches the same
// value). One thread owns one dimension over a run of consecutive points:
// the run's first point from its Gray code, the rest by that recursion; the
// threads of a warp cover consecutive dimensions, so each point's row is
// written in whole segments. The box map is lo + (hi - lo) * u with the same
// roundings as the elementwise tensor expression (no fused multiply-add).
#include <cuda_runtime.h>
#include <stdint.h>

#include "bgb_common.cuh"

namespace bgb {
namespace {

constexpr int kSobolRun = 64;  // points per thread

__global__ void sobol_box_kernel(const int64_t* __restrict__ state, const int64_t* __restrict__ shift,
                                 const double* __restrict__ first_point, int dim, int maxbit, int64_t first,
                                 int64_t n, const double* __restrict__ lower, const double* __restrict__ upper,
                                 int period, double* __restrict__ out) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t p0 = (int64_t)blockIdx.y * kSobolRun;
    if (d >= dim || p0 >= n) return;
    const int64_t p1 = p0 + kSobolRun < n ? p0 + kSobolRun : n;
    const int64_t* sd = state + (int64_t)d * maxbit;
    const double lo = lower[d % period], hi = upper[d % period];
    const double span = __dsub_rn(hi, lo);
    const double scale = 1.0 / (double)(1LL << maxbit);
    int64_t k = first + p0;  // index of the point in the sequence
    int64_t v = shift[d];
    for (int64_t g = k ^ (k >> 1), b = 0; g != 0; g >>= 1, ++b)
        if (g & 1) v ^= sd[b];
    for (int64_t p = p0; p < p1; ++p, ++k) {
        if (p > p0) v ^= sd[__ffsll((long long)k) - 1];  // bit that changes between k - 1 and k
        const double u = k == 0 ? first_point[d] : __dmul_rn((double)v, scale);
        out[p * dim + d] = __dadd_rn(lo, __dmul_rn(span, u));
    }
}

}  // namespace
}  // namespace bgb

extern "C" int bgb_sobol_box(const int64_t* state, const int64_t* shift, const double* first_point, int32_t dim,
                             int32_t maxbit, int64_t first, int64_t n, const double* lower, const double* upper,
                             int32_t period, double* out, void* stream) {
    if (dim < 1 || maxbit < 1 || maxbit > 62 || first < 0 || n < 0 || period < 1 || dim % period != 0)
        return BGB_ERR_ARG;
    if (n == 0) return BGB_OK;
    if (state == nullptr || shift == nullptr || first_point == nullptr || lower == nullptr || upper == nullptr ||
        out == nullptr)
        return BGB_ERR_ARG;
    if (bgb::ceil_div(n, bgb::kSobolRun) > 0x7fffffffLL || (first + n) >> maxbit != 0) return BGB_ERR_UNSUPPORTED;
    const dim3 grid((unsigned)bgb::ceil_div(dim, 256), (unsigned)bgb::ceil_div(n, bgb::kSobolRun));
    bgb::sobol_box_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        state, shift, first_point, dim, maxbit, first, n, lower, upper, period, out);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}
