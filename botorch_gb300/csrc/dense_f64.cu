// (b) Float64 dense linear algebra for the training side: tiled GEMM with
// triangular k-ranges, blocked right-looking Cholesky, blocked triangular
// inverse, GEMV. GB300 runs float64 at a small fraction of its float32 rate,
// so every routine here is DFMA-bound; the tiles are sized for register
// reuse, not for HBM traffic.
#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int GT = 64;   // output tile
constexpr int GK = 16;   // k step

__global__ void __launch_bounds__(256) gemm_f64_kernel(
    int64_t M, int64_t N, int64_t K, double alpha, const double* __restrict__ A, int64_t lda,
    int transA, const double* __restrict__ B, int64_t ldb, int transB, double beta,
    double* __restrict__ C, int64_t ldc, int kmode, int lower_only, const int* abort_flag,
    int64_t n_tri) {
    if (abort_flag != nullptr && *abort_flag != 0) return;
    const int64_t row0 = (int64_t)blockIdx.y * GT, col0 = (int64_t)blockIdx.x * GT;
    if (lower_only && col0 > row0 + GT - 1) return;
    __shared__ double As[GK][GT + 1];
    __shared__ double Bs[GK][GT + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double acc[4][4] = {};
    int64_t kbeg = 0, kend = K;
    if (kmode == KB_LOWER) kbeg = col0;
    else if (kmode == KAB_LOWER_T) kbeg = row0 > col0 ? row0 : col0;
    else if (kmode == KB_UPPER && col0 + GT <= n_tri) kend = col0 + GT < K ? col0 + GT : K;
    else if (kmode == KA_LOWER) kend = row0 + GT < K ? row0 + GT : K;
    kbeg = (kbeg / GK) * GK;
    for (int64_t k0 = kbeg; k0 < kend; k0 += GK) {
        for (int idx = threadIdx.x; idx < GK * GT; idx += 256) {
            int rr, kk;
            if (transA) { kk = idx / GT; rr = idx % GT; } else { rr = idx / GK; kk = idx % GK; }
            int64_t gr = row0 + rr, gk = k0 + kk;
            double v = 0.0;
            if (gr < M && gk < K) v = transA ? A[gk * lda + gr] : A[gr * lda + gk];
            As[kk][rr] = v;
        }
        for (int idx = threadIdx.x; idx < GK * GT; idx += 256) {
            int cc, kk;
            if (transB) { cc = idx / GK; kk = idx % GK; } else { kk = idx / GT; cc = idx % GT; }
            int64_t gc = col0 + cc, gk = k0 + kk;
            double v = 0.0;
            if (gc < N && gk < K) v = transB ? B[gc * ldb + gk] : B[gk * ldb + gc];
            Bs[kk][cc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { a[u] = As[kk][ty + 16 * u]; b[u] = Bs[kk][tx + 16 * u]; }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        int64_t i = row0 + ty + 16 * u;
        if (i >= M) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            int64_t j = col0 + tx + 16 * v;
            if (j >= N) continue;
            if (lower_only && j > i) continue;
            double out = alpha * acc[u][v];
            if (beta != 0.0) out = fma(beta, C[i * ldc + j], out);
            C[i * ldc + j] = out;
        }
    }
}

// Unblocked Cholesky of one diagonal block (kb <= 64) in shared memory, plus
// the inverse of the resulting triangular block (for the panel solve).
__global__ void __launch_bounds__(256) potrf_diag_kernel(double* A, int64_t lda, int kb,
                                                         int64_t k0, int* info, double* dinv) {
    if (info[1] != 0) return;  // an earlier block already failed
    __shared__ double S[64][65];
    __shared__ double X[64][65];
    __shared__ int fail;
    const int tid = threadIdx.x;
    if (tid == 0) fail = 0;
    for (int idx = tid; idx < 64 * 64; idx += 256) {
        int i = idx / 64, j = idx % 64;
        S[i][j] = (i < kb && j <= i) ? A[(int64_t)i * lda + j] : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        if (tid == 0) {
            double v = S[j][j];
            if (!(v > 0.0)) {
                fail = j + 1;
            } else {
                S[j][j] = sqrt(v);
            }
        }
        __syncthreads();
        if (fail) break;
        const double djj = S[j][j];
        for (int i = j + 1 + tid; i < kb; i += 256) S[i][j] /= djj;
        __syncthreads();
        const int rem = kb - j - 1;
        for (int idx = tid; idx < rem * rem; idx += 256) {
            int i = j + 1 + idx / rem, k = j + 1 + idx % rem;
            if (k <= i) S[i][k] = fma(-S[i][j], S[k][j], S[i][k]);
        }
        __syncthreads();
    }
    if (fail) {
        if (tid == 0) {
            info[0] = (int)(k0 + fail);
            info[1] = 1;
        }
        return;
    }
    // inverse of the lower-triangular block: column t by forward substitution
    if (tid < 64) {
        const int t = tid;
        for (int i = 0; i < 64; ++i) X[i][t] = 0.0;
        if (t < kb) {
            for (int i = t; i < kb; ++i) {
                double s = (i == t) ? 1.0 : 0.0;
                for (int k = t; k < i; ++k) s = fma(-S[i][k], X[k][t], s);
                X[i][t] = s / S[i][i];
            }
        }
    }
    __syncthreads();
    for (int idx = tid; idx < kb * kb; idx += 256) {
        int i = idx / kb, j = idx % kb;
        A[(int64_t)i * lda + j] = (j <= i) ? S[i][j] : 0.0;
        dinv[i * 64 + j] = X[i][j];
    }
}

// In-place: P (rows x kb) := P * Dinv^T (Dinv lower triangular kb x kb).
// Each CTA owns 32 rows, so reading and writing the same rows is safe.
__global__ void __launch_bounds__(256) panel_trsm_kernel(double* P, int64_t ldp, int64_t rows,
                                                         int kb, const double* __restrict__ dinv,
                                                         const int* info) {
    if (info[1] != 0) return;
    __shared__ double R[32][65];
    const int64_t r0 = (int64_t)blockIdx.x * 32;
    for (int idx = threadIdx.x; idx < 32 * 64; idx += 256) {
        int i = idx / 64, j = idx % 64;
        R[i][j] = (r0 + i < rows && j < kb) ? P[(r0 + i) * ldp + j] : 0.0;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < 32 * 64; idx += 256) {
        int i = idx / 64, c = idx % 64;
        if (r0 + i >= rows || c >= kb) continue;
        double s = 0.0;
        for (int k = 0; k <= c; ++k) s = fma(R[i][k], dinv[c * 64 + k], s);
        P[(r0 + i) * ldp + c] = s;
    }
}

__global__ void diag_inverse_blocks_kernel(const double* L, int64_t lda, int64_t n, double* D) {
    // one CTA per 64 x 64 diagonal block; D[blk] = inverse of L's diagonal block
    __shared__ double S[64][65];
    const int64_t k0 = (int64_t)blockIdx.x * 64;
    const int kb = (int)((n - k0) < 64 ? (n - k0) : 64);
    for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
        int i = idx / 64, j = idx % 64;
        S[i][j] = (i < kb && j < kb) ? L[(k0 + i) * lda + k0 + j] : 0.0;
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (t < 64) {
        double* out = D + (int64_t)blockIdx.x * 64 * 64;
        double col[64];
        for (int i = 0; i < 64; ++i) col[i] = 0.0;
        if (t < kb) {
            for (int i = t; i < kb; ++i) {
                double s = (i == t) ? 1.0 : 0.0;
                for (int k = t; k < i; ++k) s = fma(-S[i][k], col[k], s);
                col[i] = s / S[i][i];
            }
        }
        for (int i = 0; i < 64; ++i) out[i * 64 + t] = col[i];
    }
}

__global__ void copy_block_kernel(const double* src, int64_t lds, double* dst, int64_t ldd,
                                  int64_t m, int64_t n, double diag_add) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= m * n) return;
    int64_t i = idx / n, j = idx % n;
    double v = src[i * lds + j];
    if (i == j) v += diag_add;
    dst[i * ldd + j] = v;
}

__global__ void zero_upper_kernel(double* A, int64_t n, int64_t lda) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * n) return;
    int64_t i = idx / n, j = idx % n;
    if (j > i) A[i * lda + j] = 0.0;
}

__global__ void gemv_f64_kernel(int64_t m, int64_t n, double alpha, const double* __restrict__ A,
                                int64_t lda, const double* __restrict__ x, double beta,
                                double* __restrict__ y) {
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (row >= m) return;
    double s = 0.0;
    for (int64_t j = lane; j < n; j += 32) s = fma(A[row * lda + j], x[j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[row] = alpha * s + (beta != 0.0 ? beta * y[row] : 0.0);
}

__global__ void transpose_kernel(const double* src, int64_t rows, int64_t cols, int64_t lds,
                                 double* dst, int64_t ldd) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * cols) return;
    int64_t i = idx / cols, j = idx % cols;
    dst[j * ldd + i] = src[i * lds + j];
}

__global__ void convert_kernel(const double* src, float* dst, int64_t count) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < count) dst[idx] = (float)src[idx];
}

}  // namespace

int gemm_f64(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
             int transA, const double* B, int64_t ldb, int transB, double beta, double* C,
             int64_t ldc, int kmode, int lower_only, const int* abort_flag, cudaStream_t stream,
             int64_t n_tri) {
    if (M <= 0 || N <= 0) return BGB_OK;
    dim3 grid((unsigned)ceil_div(N, GT), (unsigned)ceil_div(M, GT));
    gemm_f64_kernel<<<grid, 256, 0, stream>>>(M, N, K, alpha, A, lda, transA, B, ldb, transB,
                                              beta, C, ldc, kmode, lower_only, abort_flag, n_tri);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int gemv_f64(int64_t m, int64_t n, double alpha, const double* A, int64_t lda, const double* x,
             double beta, double* y, cudaStream_t stream) {
    if (m <= 0) return BGB_OK;
    gemv_f64_kernel<<<(unsigned)ceil_div(m, 8), 256, 0, stream>>>(m, n, alpha, A, lda, x, beta, y);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

// Right-looking blocked Cholesky (block 64). dev_info[0] = failing pivot
// (1-based, 0 if none), dev_info[1] = abort flag read by the later launches.
// ws: 64*64 doubles (diagonal-block inverse).
int cholesky_f64(double* A, int64_t n, int64_t lda, int* dev_info, double* ws,
                 cudaStream_t stream) {
    BGB_CUDA_TRY(cudaMemsetAsync(dev_info, 0, 2 * sizeof(int), stream));
    for (int64_t k0 = 0; k0 < n; k0 += 64) {
        const int kb = (int)((n - k0) < 64 ? (n - k0) : 64);
        potrf_diag_kernel<<<1, 256, 0, stream>>>(A + k0 * lda + k0, lda, kb, k0, dev_info, ws);
        BGB_CHECK_LAUNCH();
        const int64_t rest = n - k0 - kb;
        if (rest <= 0) break;
        double* P = A + (k0 + kb) * lda + k0;
        panel_trsm_kernel<<<(unsigned)ceil_div(rest, 32), 256, 0, stream>>>(P, lda, rest, kb, ws,
                                                                            dev_info);
        BGB_CHECK_LAUNCH();
        double* T = A + (k0 + kb) * lda + (k0 + kb);
        int rc = gemm_f64(rest, rest, kb, -1.0, P, lda, 0, P, lda, 1, 1.0, T, lda, KFULL, 1,
                          dev_info + 1, stream);
        if (rc != BGB_OK) return rc;
    }
    return zero_upper_f64(A, n, lda, stream);
}

// In-place inverse of a lower-triangular matrix, blocked by 64 rows.
// ws: (n/64 + 1) * 64*64 diagonal inverses + 64 * n temporary.
int tri_inverse_f64(double* L, int64_t n, int64_t lda, double* ws, cudaStream_t stream) {
    const int64_t nb = ceil_div(n, 64);
    double* D = ws;
    double* T = ws + nb * 64 * 64;
    diag_inverse_blocks_kernel<<<(unsigned)nb, 64, 0, stream>>>(L, lda, n, D);
    BGB_CHECK_LAUNCH();
    for (int64_t ib = 0; ib < nb; ++ib) {
        const int64_t i0 = ib * 64;
        const int64_t kb = (n - i0) < 64 ? (n - i0) : 64;
        if (ib > 0) {
            // T = L[i-block, 0:i0] * Y[0:i0, 0:i0] (Y lower triangular, already in place)
            int rc = gemm_f64(kb, i0, i0, 1.0, L + i0 * lda, lda, 0, L, lda, 0, 0.0, T, i0,
                              KB_LOWER, 0, nullptr, stream);
            if (rc != BGB_OK) return rc;
            // Y[i-block, 0:i0] = -D_i * T
            rc = gemm_f64(kb, i0, kb, -1.0, D + ib * 64 * 64, 64, 0, T, i0, 0, 0.0, L + i0 * lda,
                          lda, KFULL, 0, nullptr, stream);
            if (rc != BGB_OK) return rc;
        }
        copy_block_kernel<<<(unsigned)ceil_div(kb * kb, 256), 256, 0, stream>>>(
            D + ib * 64 * 64, 64, L + i0 * lda + i0, lda, kb, kb, 0.0);
        BGB_CHECK_LAUNCH();
    }
    return zero_upper_f64(L, n, lda, stream);
}

int copy_matrix_f64(const double* src, int64_t lds, double* dst, int64_t ldd, int64_t m, int64_t n,
                    double diag_add, cudaStream_t stream) {
    if (m <= 0 || n <= 0) return BGB_OK;
    copy_block_kernel<<<(unsigned)ceil_div(m * n, 256), 256, 0, stream>>>(src, lds, dst, ldd, m, n,
                                                                         diag_add);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int zero_upper_f64(double* A, int64_t n, int64_t lda, cudaStream_t stream) {
    if (n <= 0) return BGB_OK;
    zero_upper_kernel<<<(unsigned)ceil_div(n * n, 256), 256, 0, stream>>>(A, n, lda);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int transpose_f64(const double* src, int64_t rows, int64_t cols, int64_t lds, double* dst,
                  int64_t ldd, cudaStream_t stream) {
    if (rows <= 0 || cols <= 0) return BGB_OK;
    transpose_kernel<<<(unsigned)ceil_div(rows * cols, 256), 256, 0, stream>>>(src, rows, cols, lds,
                                                                              dst, ldd);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int convert_f64_f32(const double* src, float* dst, int64_t count, cudaStream_t stream) {
    if (count <= 0) return BGB_OK;
    convert_kernel<<<(unsigned)ceil_div(count, 256), 256, 0, stream>>>(src, dst, count);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

}  // namespace bgb
