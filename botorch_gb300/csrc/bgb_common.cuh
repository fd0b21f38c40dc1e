// Shared device helpers: stationary kernel values and derivatives, launch checks.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/botorch_gb300.h"

namespace bgb {
// Counts kernel launches made by this library (reported by bgb_launch_count).
void note_launch();
}  // namespace bgb

#define BGB_CHECK_LAUNCH()                                          \
    do {                                                            \
        bgb::note_launch();                                         \
        if (cudaGetLastError() != cudaSuccess) return BGB_ERR_CUDA; \
    } while (0)

#define BGB_CUDA_TRY(expr)                                  \
    do {                                                    \
        if ((expr) != cudaSuccess) return BGB_ERR_CUDA;     \
    } while (0)

namespace bgb {

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

// Floor on r^2 before the square root, as gpytorch's `dist` clamps at 1e-30:
// keeps the Matern gradient finite at coincident points.
constexpr double kMinSqDist = 1e-30;

template <typename T> __device__ __forceinline__ T dexp(T x);
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <typename T> __device__ __forceinline__ T dsqrt(T x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }

// kappa(r2): kernel value without the outputscale, r2 = squared scaled distance.
template <typename T>
__device__ __forceinline__ T kappa(int kind, T r2) {
    if (kind == BGB_KERNEL_RBF) return dexp<T>(T(-0.5) * r2);
    T rho = dsqrt<T>(r2 > T(kMinSqDist) ? r2 : T(kMinSqDist));
    if (kind == BGB_KERNEL_MATERN52) {
        T s = T(2.2360679774997896964) * rho;
        return (T(1) + s + T(5.0 / 3.0) * r2) * dexp<T>(-s);
    }
    if (kind == BGB_KERNEL_MATERN32) {
        T s = T(1.7320508075688772935) * rho;
        return (T(1) + s) * dexp<T>(-s);
    }
    return dexp<T>(-rho);  // Matern-1/2
}

// d kappa / d r2 (the adjoint of the kernel build). Below the r2 floor the
// distance is a constant in the reference's autograd graph, so only the terms
// that depend on r2 directly survive; the resulting gradient is multiplied by
// (x - y) = 0 there in every use.
template <typename T>
__device__ __forceinline__ T dkappa_dr2(int kind, T r2) {
    if (kind == BGB_KERNEL_RBF) return T(-0.5) * dexp<T>(T(-0.5) * r2);
    bool live = r2 > T(kMinSqDist);
    T rho = dsqrt<T>(live ? r2 : T(kMinSqDist));
    if (kind == BGB_KERNEL_MATERN52) {
        T s = T(2.2360679774997896964) * rho;
        T e = dexp<T>(-s);
        // d/dr2 [(1 + s + 5/3 r2) e^-s] with s = sqrt(5 r2): -(5/6)(1 + s) e^-s
        return live ? T(-5.0 / 6.0) * (T(1) + s) * e : T(5.0 / 3.0) * e;
    }
    if (kind == BGB_KERNEL_MATERN32) {
        T s = T(1.7320508075688772935) * rho;
        return live ? T(-1.5) * dexp<T>(-s) : T(0);
    }
    return live ? -dexp<T>(-rho) / (T(2) * rho) : T(0);
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// Bump allocator over a caller-provided workspace.
struct Arena {
    char* base;
    size_t cap;
    size_t off;
    template <typename T>
    T* take(size_t count) {
        size_t bytes = align_up(count * sizeof(T));
        if (off + bytes > cap) return nullptr;
        T* p = reinterpret_cast<T*>(base + off);
        off += bytes;
        return p;
    }
};

}  // namespace bgb
