// (b) Float64 dense linear algebra for the training side: tiled GEMM with
// triangular k-ranges, blocked right-looking Cholesky, blocked triangular
// inverse, GEMV. GB300 runs float64 at a small fraction of its float32 rate,
// so every routine here is DFMA-bound; the tiles are sized for register
// reuse, not for HBM traffic.
#include <mutex>

#include "bgb_common.cuh"
#include "bgb_kernels.cuh"

namespace bgb {

namespace {

constexpr int GT = 64;   // output tile
constexpr int GK = 16;   // k step

// blockIdx.z: member of a batch of equal-shape products at element strides sA, sB, sC
__global__ void __launch_bounds__(256) gemm_f64_kernel(
    int64_t M, int64_t N, int64_t K, double alpha, const double* __restrict__ A, int64_t lda,
    int transA, const double* __restrict__ B, int64_t ldb, int transB, double beta,
    double* __restrict__ C, int64_t ldc, int kmode, int lower_only, const int* abort_flag,
    int64_t n_tri, int64_t sA, int64_t sB, int64_t sC) {
    if (abort_flag != nullptr && *abort_flag != 0) return;
    A += (int64_t)blockIdx.z * sA;
    B += (int64_t)blockIdx.z * sB;
    C += (int64_t)blockIdx.z * sC;
    // tile order: CTAs start in launch order, so with a triangular k range the
    // tiles with the longest range go first (KB_LOWER: the first columns;
    // KA_LOWER: the last rows), and the last wave holds short tiles only
    const int64_t lin = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
    int64_t tr = blockIdx.y, tc = blockIdx.x;
    if (kmode == KB_LOWER) {
        tc = lin / gridDim.y;
        tr = lin % gridDim.y;
    } else if (kmode == KA_LOWER) {
        tr = gridDim.y - 1 - lin / gridDim.x;
        tc = lin % gridDim.x;
    }
    const int64_t row0 = tr * GT, col0 = tc * GT;
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
// the inverse of the resulting triangular block (for the panel solve). Thread
// (r, cq) = (tid / 4, tid % 4) works on row r, columns cq, cq + 4, ...; both
// passes are right-looking with the pivot work (square root and reciprocal of
// the next diagonal entry; scaling of the next finished row of the inverse)
// done by the thread that updates that entry last, so each column costs two
// barriers (factor) and one (inverse). float64 runs at a small fraction of
// the float32 rate here, so the passes issue no redundant float64 work.
__global__ void __launch_bounds__(256) potrf_diag_kernel(double* A, int64_t lda, int kb,
                                                         int64_t k0, int* info, double* dinv) {
    if (info[1] != 0) return;  // an earlier block already failed
    __shared__ double S[64][65];
    __shared__ double X[64][65];
    __shared__ double rd[64];
    __shared__ int fail;
    const int tid = threadIdx.x;
    const int r = tid >> 2, cq = tid & 3;
    for (int idx = tid; idx < 64 * 64; idx += 256) {
        const int i = idx >> 6, j = idx & 63;
        S[i][j] = (i < kb && j <= i) ? A[(int64_t)i * lda + j] : 0.0;
        X[i][j] = (i == j) ? 1.0 : 0.0;
    }
    __syncthreads();
    if (tid == 0) {
        fail = 0;
        const double v = S[0][0];
        if (!(v > 0.0)) {
            fail = 1;
        } else {
            const double d = sqrt(v);
            S[0][0] = d;
            rd[0] = 1.0 / d;
        }
    }
    __syncthreads();
    for (int j = 0; j < kb && !fail; ++j) {
        // column j below the diagonal: L[r][j] = S[r][j] / L[j][j]
        if (cq == 0 && r > j && r < kb) S[r][j] *= rd[j];
        __syncthreads();
        // trailing update of the lower triangle; the thread of (j+1, j+1) then pivots
        if (r > j && r < kb) {
            const double lrj = S[r][j];
            for (int k = j + 1 + cq; k <= r; k += 4) S[r][k] = fma(-lrj, S[k][j], S[r][k]);
            if (r == j + 1 && cq == 0) {
                const double v = S[r][r];
                if (!(v > 0.0)) {
                    fail = r + 1;
                } else {
                    const double d = sqrt(v);
                    S[r][r] = d;
                    rd[r] = 1.0 / d;
                }
            }
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
    // X = L^-1 by rows: row k is final once rows < k are eliminated from it and it
    // is scaled by 1 / L[k][k]; eliminating row k from rows i > k finishes row k + 1
    if (tid == 0) X[0][0] = rd[0];
    __syncthreads();
    for (int k = 0; k + 1 < kb; ++k) {
        if (r > k && r < kb) {
            const double lrk = S[r][k];
            for (int c = cq; c <= k; c += 4) X[r][c] = fma(-lrk, X[k][c], X[r][c]);
            if (r == k + 1)
                for (int c = cq; c <= r; c += 4) X[r][c] *= rd[r];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < kb * kb; idx += 256) {
        int i = idx / kb, j = idx % kb;
        A[(int64_t)i * lda + j] = (j <= i) ? S[i][j] : 0.0;
        dinv[i * 64 + j] = (j <= i) ? X[i][j] : 0.0;
    }
}

// In-place: P (rows x kb) := P * Dinv^T (Dinv lower triangular kb x kb, staged in
// shared memory). Each CTA owns 16 rows, so reading and writing the same rows is safe.
constexpr int kTrsmRows = 16;
__global__ void __launch_bounds__(256) panel_trsm_kernel(double* P, int64_t ldp, int64_t rows,
                                                         int kb, const double* __restrict__ dinv,
                                                         const int* info) {
    if (info[1] != 0) return;
    __shared__ double R[kTrsmRows][65];
    __shared__ double D[64][65];
    const int64_t r0 = (int64_t)blockIdx.x * kTrsmRows;
    for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
        const int i = idx >> 6, j = idx & 63;
        D[i][j] = (i < kb && j <= i) ? dinv[i * 64 + j] : 0.0;
    }
    for (int idx = threadIdx.x; idx < kTrsmRows * 64; idx += 256) {
        const int i = idx >> 6, j = idx & 63;
        R[i][j] = (r0 + i < rows && j < kb) ? P[(r0 + i) * ldp + j] : 0.0;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < kTrsmRows * 64; idx += 256) {
        const int i = idx >> 6, c = idx & 63;
        if (r0 + i >= rows || c >= kb) continue;
        double s0 = 0.0, s1 = 0.0;
        int k = 0;
        for (; k + 1 <= c; k += 2) {
            s0 = fma(R[i][k], D[c][k], s0);
            s1 = fma(R[i][k + 1], D[c][k + 1], s1);
        }
        if (k <= c) s0 = fma(R[i][k], D[c][k], s0);
        P[(r0 + i) * ldp + c] = s0 + s1;
    }
}

// In place: every 64 x 64 diagonal block of the lower-triangular L (n x n) is
// replaced by its inverse (zeros above its diagonal); one CTA per block, 64
// threads, thread t solving column t by forward substitution.
__global__ void diag_inverse_inplace_kernel(double* L, int64_t lda, int64_t n) {
    __shared__ double S[64][65];
    const int64_t k0 = (int64_t)blockIdx.x * 64;
    const int kb = (int)((n - k0) < 64 ? (n - k0) : 64);
    for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
        int i = idx / 64, j = idx % 64;
        S[i][j] = (i < kb && j < kb) ? L[(k0 + i) * lda + k0 + j] : 0.0;
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= kb) return;
    double col[64];
    for (int i = 0; i < 64; ++i) col[i] = 0.0;
    for (int i = t; i < kb; ++i) {
        double s = (i == t) ? 1.0 : 0.0;
        for (int k = t; k < i; ++k) s = fma(-S[i][k], col[k], s);
        col[i] = s / S[i][i];
    }
    for (int i = 0; i < kb; ++i) L[(k0 + i) * lda + k0 + t] = col[i];
}

// y = alpha * A^T x + beta * y, A m x n row-major: one CTA per 32 columns, its
// 8 warps taking every 8th row (lane = column, so each row read is one 256-byte
// segment), the 8 partial sums added in a fixed order.
__global__ void __launch_bounds__(256) gemv_t_f64_kernel(int64_t m, int64_t n, double alpha,
                                                         const double* __restrict__ A, int64_t lda,
                                                         const double* __restrict__ x, double beta,
                                                         double* __restrict__ y) {
    __shared__ double part[8][33];
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const int64_t j = (int64_t)blockIdx.x * 32 + lane;
    double s0 = 0.0, s1 = 0.0;
    if (j < n) {
        int64_t i = w;
        for (; i + 8 < m; i += 16) {
            s0 = fma(A[i * lda + j], x[i], s0);
            s1 = fma(A[(i + 8) * lda + j], x[i + 8], s1);
        }
        if (i < m) s0 = fma(A[i * lda + j], x[i], s0);
    }
    part[w][lane] = s0 + s1;
    __syncthreads();
    if (w == 0 && j < n) {
        double t = 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) t += part[u][lane];
        y[j] = alpha * t + (beta != 0.0 ? beta * y[j] : 0.0);
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
    return gemm_f64_batched(M, N, K, alpha, A, lda, 0, transA, B, ldb, 0, transB, beta, C, ldc, 0,
                            kmode, lower_only, abort_flag, 1, stream, n_tri);
}

int gemm_f64_batched(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                     int64_t sA, int transA, const double* B, int64_t ldb, int64_t sB, int transB,
                     double beta, double* C, int64_t ldc, int64_t sC, int kmode, int lower_only,
                     const int* abort_flag, int64_t batch, cudaStream_t stream, int64_t n_tri) {
    if (M <= 0 || N <= 0 || batch <= 0) return BGB_OK;
    if (batch > 65535) return BGB_ERR_ARG;
    dim3 grid((unsigned)ceil_div(N, GT), (unsigned)ceil_div(M, GT), (unsigned)batch);
    gemm_f64_kernel<<<grid, 256, 0, stream>>>(M, N, K, alpha, A, lda, transA, B, ldb, transB,
                                              beta, C, ldc, kmode, lower_only, abort_flag, n_tri,
                                              sA, sB, sC);
    BGB_CHECK_LAUNCH();
    return BGB_OK;
}

int gemv_t_f64(int64_t m, int64_t n, double alpha, const double* A, int64_t lda, const double* x,
               double beta, double* y, cudaStream_t stream) {
    if (n <= 0) return BGB_OK;
    gemv_t_f64_kernel<<<(unsigned)ceil_div(n, 32), 256, 0, stream>>>(m, n, alpha, A, lda, x, beta,
                                                                     y);
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

// A high-priority side stream and two events per device for the lookahead of
// cholesky_f64; the mutex keeps each call's record / wait pairs together.
struct Lookahead {
    std::mutex mu;
    cudaStream_t side = nullptr;
    cudaEvent_t ready = nullptr, panel = nullptr;
};

Lookahead* lookahead_for_current_device() {
    static Lookahead per_dev[64];
    static std::mutex init_mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(init_mu);
    Lookahead& la = per_dev[dev];
    if (la.side == nullptr) {
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
            cudaStreamCreateWithPriority(&la.side, cudaStreamNonBlocking, greatest) != cudaSuccess ||
            cudaEventCreateWithFlags(&la.ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&la.panel, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            la.side = nullptr;
            return nullptr;
        }
    }
    return &la;
}

// Right-looking blocked Cholesky (block 64) with a lookahead of one panel: after
// panel k is solved, the next panel's column block is updated first, so the
// next panel's diagonal factor (one CTA) and panel solve run on a high-priority
// side stream while the rest of the trailing matrix is updated on `stream`.
// dev_info[0] = failing pivot (1-based, 0 if none), dev_info[1] = abort flag
// read by the later launches. ws: 64*64 doubles (diagonal-block inverse; panel
// k + 1's factor writes it after panel k's solve has read it, both on the side
// stream or in stream order before the first fork).
int cholesky_f64(double* A, int64_t n, int64_t lda, int* dev_info, double* ws,
                 cudaStream_t stream) {
    BGB_CUDA_TRY(cudaMemsetAsync(dev_info, 0, 2 * sizeof(int), stream));
    Lookahead* la = lookahead_for_current_device();
    std::unique_lock<std::mutex> lock;
    if (la != nullptr) lock = std::unique_lock<std::mutex>(la->mu);
    auto factor_panel = [&](int64_t k0, cudaStream_t st) -> int {
        const int kb = (int)((n - k0) < 64 ? (n - k0) : 64);
        potrf_diag_kernel<<<1, 256, 0, st>>>(A + k0 * lda + k0, lda, kb, k0, dev_info, ws);
        BGB_CHECK_LAUNCH();
        const int64_t rest = n - k0 - kb;
        if (rest > 0) {
            panel_trsm_kernel<<<(unsigned)ceil_div(rest, (int64_t)kTrsmRows), 256, 0, st>>>(
                A + (k0 + kb) * lda + k0, lda, rest, kb, ws, dev_info);
            BGB_CHECK_LAUNCH();
        }
        return BGB_OK;
    };
    int rc = factor_panel(0, stream);
    if (rc) return rc;
    for (int64_t k0 = 0; k0 < n; k0 += 64) {
        const int kb = (int)((n - k0) < 64 ? (n - k0) : 64);
        const int64_t rest = n - k0 - kb;
        if (rest <= 0) break;
        const double* P = A + (k0 + kb) * lda + k0;  // panel k below its diagonal block
        double* T = A + (k0 + kb) * lda + (k0 + kb);  // trailing matrix
        const int kb1 = (int)(rest < 64 ? rest : 64);
        if (la == nullptr) {
            rc = gemm_f64(rest, rest, kb, -1.0, P, lda, 0, P, lda, 1, 1.0, T, lda, KFULL, 1,
                          dev_info + 1, stream);
            if (rc) return rc;
            rc = factor_panel(k0 + kb, stream);
            if (rc) return rc;
            continue;
        }
        // next panel's column block, then its factor on the side stream
        rc = gemm_f64(rest, kb1, kb, -1.0, P, lda, 0, P, lda, 1, 1.0, T, lda, KFULL, 1,
                      dev_info + 1, stream);
        if (rc) return rc;
        BGB_CUDA_TRY(cudaEventRecord(la->ready, stream));
        BGB_CUDA_TRY(cudaStreamWaitEvent(la->side, la->ready, 0));
        rc = factor_panel(k0 + kb, la->side);
        if (rc) return rc;
        BGB_CUDA_TRY(cudaEventRecord(la->panel, la->side));
        // the rest of the trailing matrix meanwhile
        const int64_t rest2 = rest - kb1;
        if (rest2 > 0) {
            rc = gemm_f64(rest2, rest2, kb, -1.0, P + kb1 * lda, lda, 0, P + kb1 * lda, lda, 1, 1.0,
                          T + kb1 * lda + kb1, lda, KFULL, 1, dev_info + 1, stream);
            if (rc) return rc;
        }
        BGB_CUDA_TRY(cudaStreamWaitEvent(stream, la->panel, 0));
    }
    return zero_upper_f64(A, n, lda, stream);
}

// Workspace (doubles) of tri_inverse_f64: the largest level's products T.
int64_t tri_inverse_ws_doubles(int64_t n) {
    int64_t best = 64 * 64;
    for (int64_t s = 64; s < n; s *= 2) {
        int64_t need = 0;
        for (int64_t a0 = 0; a0 + s < n; a0 += 2 * s) {
            const int64_t sc = (n - a0 - s) < s ? (n - a0 - s) : s;
            need += sc * s;
        }
        best = need > best ? need : best;
    }
    return best;
}

// In-place inverse of a lower-triangular matrix (upper triangle zero), bottom up
// over block sizes s = 64, 128, ...: every 64 x 64 diagonal block is inverted,
// then at each level the pairs of adjacent inverted blocks [A 0; B C] become
//   [A^-1 0; -C^-1 (B A^-1)  C^-1]
// through two triangular GEMMs batched over all pairs of the level (one
// launch each for the pairs of full size, one each for a ragged last pair), so
// every level but the first few fills the GPU. ws: tri_inverse_ws_doubles(n).
int tri_inverse_f64(double* L, int64_t n, int64_t lda, double* ws, cudaStream_t stream) {
    if (n <= 0) return BGB_OK;
    int rc = zero_upper_f64(L, n, lda, stream);
    if (rc) return rc;
    diag_inverse_inplace_kernel<<<(unsigned)ceil_div(n, 64), 64, 0, stream>>>(L, lda, n);
    BGB_CHECK_LAUNCH();
    for (int64_t s = 64; s < n; s *= 2) {
        const int64_t full = n / (2 * s);               // pairs whose C block has s rows
        const int64_t a_last = full * 2 * s;            // A block of a ragged last pair
        const int64_t sc_last = n - a_last - s;         // its C rows (<= 0: no such pair)
        const int64_t step = 2 * s * lda + 2 * s;       // from one pair to the next
        // T_p = B_p A_p^-1  (A^-1 lower triangular: k >= column)
        if (full > 0) {
            rc = gemm_f64_batched(s, s, s, 1.0, L + s * lda, lda, step, 0, L, lda, step, 0, 0.0, ws,
                                  s, s * s, KB_LOWER, 0, nullptr, full, stream);
            if (rc) return rc;
        }
        if (sc_last > 0) {
            rc = gemm_f64(sc_last, s, s, 1.0, L + (a_last + s) * lda + a_last, lda, 0,
                          L + a_last * lda + a_last, lda, 0, 0.0, ws + full * s * s, s, KB_LOWER, 0,
                          nullptr, stream);
            if (rc) return rc;
        }
        // B_p := -C_p^-1 T_p  (C^-1 lower triangular: k <= row)
        if (full > 0) {
            rc = gemm_f64_batched(s, s, s, -1.0, L + s * lda + s, lda, step, 0, ws, s, s * s, 0, 0.0,
                                  L + s * lda, lda, step, KA_LOWER, 0, nullptr, full, stream);
            if (rc) return rc;
        }
        if (sc_last > 0) {
            rc = gemm_f64(sc_last, s, sc_last, -1.0, L + (a_last + s) * lda + a_last + s, lda, 0,
                          ws + full * s * s, s, 0, 0.0, L + (a_last + s) * lda + a_last, lda,
                          KA_LOWER, 0, nullptr, stream);
            if (rc) return rc;
        }
    }
    return BGB_OK;
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
