// Internal launchers shared between the translation units of the library.
#pragma once

#include <vector>
#include <cuda_fp16.h>

#include <cuda_runtime.h>
#include <stdint.h>

namespace bgb {

// kernel_build.cu
template <typename TIn, typename TAcc, typename TOut>
int launch_kernel_matrix(const TIn* X1, int64_t m, const TIn* X2, int64_t n2, int d,
                         const double* inv_ls, double outputscale, int kind, double diag_add,
                         int same, TOut* K, int64_t ldk, cudaStream_t stream);
// Float32 form over coordinates already scaled by 1 / lengthscale, both k-major
// (Z1T: d x m with leading dimension ldz1, Z2T: d x n2 with ldz2), without
// rescaling per tile. Output: K (float32), or with K16 set the float16 split
// of k16_scale * K into K16 / K16_lo; leading dimension ldk either way.
int launch_kernel_matrix_zt(const float* Z1T, int64_t ldz1, int64_t m, const float* Z2T,
                            int64_t ldz2, int64_t n2, int d, double outputscale, int kind,
                            float* K, __half* K16, __half* K16_lo, float k16_scale, int64_t ldk,
                            cudaStream_t stream);

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

// gemm_f64 over `batch` equal-shape products, member z at A + z sA, B + z sB, C + z sC.
int gemm_f64_batched(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                     int64_t sA, int transA, const double* B, int64_t ldb, int64_t sB, int transB,
                     double beta, double* C, int64_t ldc, int64_t sC, int kmode, int lower_only,
                     const int* abort_flag, int64_t batch, cudaStream_t stream, int64_t n_tri = 0);
// y = alpha * A^T x + beta * y (A: m x n row-major, y: n), float64
int gemv_t_f64(int64_t m, int64_t n, double alpha, const double* A, int64_t lda, const double* x,
               double beta, double* y, cudaStream_t stream);
int64_t tri_inverse_ws_doubles(int64_t n);

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

// mll.cu ---------------------------------------------------------------------
// Exact MLL of y under the GP and its gradient (float64, from L, L^-1, alpha):
// out_host[0] = mll / n, [1 + k] = -s sum W kappa' dz_k^2 / n (to be scaled by
// 1 / l_k), [1 + d] outputscale, [2 + d] noise, [3 + d] mean-constant gradient.
size_t mll_workspace_bytes(int64_t n, int d);
int gp_mll(const double* X, int64_t n, int d, const double* inv_ls, double outputscale, int kind,
           double mean_constant, const double* y, const double* L, const double* Linv,
           const double* alpha, double* out_host, void* ws, size_t ws_bytes, cudaStream_t st);

// crosscov_tc.cu ------------------------------------------------------------
bool tc_gemm_available();
// One GEMM of a grouped tensor-core launch (the operands of tc_gemm_f16x3).
struct TcGroupGemm {
    int64_t M, N, K;
    const __half* A_hi;
    const __half* A_lo;
    int64_t lda;
    const __half* B_hi;
    const __half* B_lo;
    int64_t ldbs;
    float* C;
    int64_t ldc;
    int kmode;
    const float* row_mul;
    float row_mul_const;
    const float* col_mul;
};
size_t tc_group_entry_bytes();
// tiles of one GEMM (M x N) in a grouped launch
int64_t tc_group_tiles(int64_t M, int64_t N);
// Device tables of a grouped launch: `entries` (tc_group_entry_bytes() per GEMM,
// to be copied to dev_entries, 64-byte aligned), per-cluster tile ranges `off`
// (clusters + 1) and the tile list `tiles`.
int tc_group_build(const TcGroupGemm* gemms, int count, uintptr_t dev_entries,
                   std::vector<unsigned char>& entries, std::vector<int>& off,
                   std::vector<uint64_t>& tiles, int& clusters);
int tc_group_launch(const void* dev_entries, const int* dev_off, const uint64_t* dev_tiles,
                    int clusters, int* err, cudaStream_t stream);
// C = diag(row_mul) A op(B) diag(col_mul) on tcgen05 tensor cores from float16
// hi/lo splits (ah*bh + ah*bl + al*bh, float32 accumulation). A: hi/lo (M x K,
// lda); B given by its K-major storage Bs (N x K, hi/lo, ldbs), op(B)[k][j] =
// Bs[j][k]; row_mul nullptr: row_mul_const for every row; kmode KB_UPPER /
// KB_LOWER / KFULL. err: device int set non-zero when a bounded wait expired.
int tc_gemm_f16x3(int64_t M, int64_t N, int64_t K, const __half* A_hi, const __half* A_lo,
                  int64_t lda, const __half* B_hi, const __half* B_lo, int64_t ldbs, float* C,
                  int64_t ldc, int kmode, const float* row_mul, float row_mul_const,
                  const float* col_mul, int* err, cudaStream_t stream);
// Row-scaled float16 split of a float64 matrix (or of its transpose): per
// storage row i a power-of-two s_i bringing max |x_i.| to at most 2^14,
// hi = f16(s_i x), lo = f16(s_i x - hi) (ldd-strided rows, columns >= cols
// zero), mul[i] = 1 / s_i.
int split_f64_f16(const double* src, int64_t rows, int64_t cols, int64_t lds, int transpose,
                  __half* hi, __half* lo, int64_t ldd, float* mul, cudaStream_t stream);

}  // namespace bgb
