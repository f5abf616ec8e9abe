// dense.cuh -- dense linear algebra on the GPU for the BEM systems.
//
// Replaces the LAPACK/BLAS calls of the reference (src/utils/linalg.hpp:17-78):
//   gemm      -> dgemm_          C = alpha op(A) op(B) + beta C, column-major
//   LUFactor  -> dgetrf_/dgetrs_ LU with partial pivoting and solves
//   solve     -> dgesv_          (factor + solve)
//
// LU design.  Partial pivoting on the BEM blocks of this problem never swaps a
// row (the matrices are diagonally dominant in the pivoting sense), so the
// factorisation runs a blocked right-looking LU WITHOUT row exchanges and
// certifies on the fly that partial pivoting would have chosen the same pivots:
// dgetrf keeps the diagonal pivot exactly when no multiplier exceeds 1 in
// magnitude (idamax returns the first maximum, so ties keep the diagonal).  If
// any |l_ij| > 1 (or a pivot is zero) the certificate fails and the matrix is
// refactored from a saved copy by an unblocked partial-pivoting LU that swaps
// rows exactly like dgetrf.  Either way the factors and pivots are those of
// dgetrf up to rounding.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"

namespace sqbem {

constexpr int LU_NB = 64;  // panel width of the blocked LU (FP64)

// C(MxN) = alpha * op(A) * op(B) + beta * C   (column-major, FP64)
void gemm64(bool ta, bool tb, int M, int N, int K, double alpha, const double* A, long long lda,
            const double* B, long long ldb, double beta, double* C, long long ldc, cudaStream_t st);

// LU factorisation (dgetrf semantics) of an n x n column-major matrix, kept on
// the device with the inverses of its diagonal blocks (used by the solves).
struct LU64 {
    int n = 0;
    long long ld = 0;
    DevBuf<double> A;      // factors (unit L below the diagonal, U on and above)
    DevBuf<double> Linv;   // per diagonal block: inverse of the unit-lower block (LU_NB x LU_NB)
    DevBuf<double> Uinv;   // per diagonal block: inverse of the upper block
    DevBuf<int> ipiv;      // 0-based pivot rows (dgetrf convention, only if pivoted)
    bool pivoted = false;  // true if the certificate failed and rows were exchanged

    // Factor M (n x n, leading dimension ld, device); M is copied.
    // Throws Error(SQBEM_ERR_SINGULAR, what) on a zero pivot.
    void factor(const double* M, int n, long long ld, cudaStream_t st, const char* what);
    // Take ownership of a device buffer (n x n, leading dimension n) and factor it in place.
    void factor_inplace(DevBuf<double>&& M, int n, cudaStream_t st, const char* what);
    // B <- A^{-1} B for B (n x nrhs, leading dimension ldb, device)
    void solve(double* B, long long ldb, int nrhs, cudaStream_t st) const;
    // B <- A^{-T} B (dgetrs 'T'): U^T then L^T solves, then the row exchanges undone
    void solve_transpose(double* B, long long ldb, int nrhs, cudaStream_t st) const;
};

// Solve with the certified LU; helpers shared with the mixed path.
void copy_matrix64(const double* src, long long lds, double* dst, long long ldd, int rows, int cols, cudaStream_t st);
// max |A| over a column-major block (result written to *out on the device)
void max_abs64(const double* A, long long lda, int rows, int cols, double* out, cudaStream_t st);

}  // namespace sqbem
