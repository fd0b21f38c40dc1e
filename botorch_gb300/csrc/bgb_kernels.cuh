// Internal launchers shared between the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bgb {

// kernel_build.cu
// K_lo non-null (float32 output only): write the tf32 hi/lo split (K = hi).
template <typename TIn, typename TAcc, typename TOut>
int launch_kernel_matrix(const TIn* X1, int64_t m, const TIn* X2, int64_t n2, int d,
                         const double* inv_ls, double outputscale, int kind, double diag_add,
                         int same, TOut* K, int64_t ldk, cudaStream_t stream,
                         TOut* K_lo = nullptr);
// Float32 form over coordinates already scaled by 1 / lengthscale, both k-major
// (Z1T: d x m with leading dimension ldz1, Z2T: d x n2 with ldz2). Same tile
// arithmetic as the float instantiation above, without rescaling per tile.
int launch_kernel_matrix_zt(const float* Z1T, int64_t ldz1, int64_t m, const float* Z2T,
                            int64_t ldz2, int64_t n2, int d, double outputscale, int kind,
                            float* K, int64_t ldk, cudaStream_t stream, float* K_lo = nullptr);

// dense_f64.cu ------------------------------------------------------------
// k-range modes of the GEMMs (structure of triangular operands):
enum KMode : int {
    KFULL = 0,        // k in [0, K)
    KB_LOWER = 1,     // B lower triangular (op(B)[k][j] = 0 for k < j): k >= col
    KAB_LOWER_T = 2,  // C = A^T B with A, B lower triangular: k >= max(row, col)
    KB_UPPER = 3,     // op(B) upper triangular in its first n_tri columns: k <= col there
    KA_LOWER = 4,     // op(A) lower triangular: k <= row
};
// C (M x N) = alpha * op(A) * op(B) + beta * C, row-major, float64.
// transA: op(A) = A^T (A stored K x M). transB: op(B) = B^T (B stored N x K).
// lower_only: tiles strictly above the diagonal are skipped (SYRK-style update).
int gemm_f64(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
             int transA, const double* B, int64_t ldb, int transB, double beta, double* C,
             int64_t ldc, int kmode, int lower_only, const int* abort_flag, cudaStream_t stream,
             int64_t n_tri = 0);

// y = alpha * A x + beta * y (A: m x n row-major), float64
int gemv_f64(int64_t m, int64_t n, double alpha, const double* A, int64_t lda, const double* x,
             double beta, double* y, cudaStream_t stream);

int cholesky_f64(double* A, int64_t n, int64_t lda, int* dev_info, double* dinv_ws,
                 cudaStream_t stream);
int tri_inverse_f64(double* L, int64_t n, int64_t lda, double* ws, cudaStream_t stream);
int copy_matrix_f64(const double* src, int64_t lds, double* dst, int64_t ldd, int64_t m, int64_t n,
                    double diag_add, cudaStream_t stream);
int zero_upper_f64(double* A, int64_t n, int64_t lda, cudaStream_t stream);
int convert_f64_f32(const double* src, float* dst, int64_t count, cudaStream_t stream);

// crosscov.cu --------------------------------------------------------------
// C (M x N) = A (M x K) * B (K x N), float32 SIMT path, row-major.
// kmode: KFULL, KB_LOWER or KB_UPPER (with n_tri) as for gemm_f64.
int gemm_f32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
             int64_t ldb, float* C, int64_t ldc, int kmode, int64_t n_tri, cudaStream_t stream);
int transpose_f64(const double* src, int64_t rows, int64_t cols, int64_t lds, double* dst,
                  int64_t ldd, cudaStream_t stream);

// crosscov_tc.cu ------------------------------------------------------------
bool tc_gemm_available();
// C = A op(B) on tcgen05 tensor cores, 3xTF32. A: hi/lo (M x K, lda); B given by its
// K-major storage Bs (N x K, hi/lo, ldbs), op(B)[k][j] = Bs[j][k]; kmode KB_UPPER/KB_LOWER.
// err: device int set non-zero when a bounded wait expired.
int tc_gemm_tf32x3(int64_t M, int64_t N, int64_t K, const float* A_hi, const float* A_lo,
                   int64_t lda, const float* B_hi, const float* B_lo, int64_t ldbs, float* C,
                   int64_t ldc, int kmode, int* err, cudaStream_t stream);
int split_tf32(const float* src, int64_t rows, int64_t cols, int64_t lds, float* hi, float* lo,
               int64_t ldd, cudaStream_t stream);
int split_f64_tf32(const double* src, int64_t rows, int64_t cols, int64_t lds, int transpose,
                   float* hi, float* lo, int64_t ldd, cudaStream_t stream);

}  // namespace bgb
