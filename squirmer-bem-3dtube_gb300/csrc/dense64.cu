// dense64.cu -- FP64 GEMM, certified no-exchange blocked LU with a partial-
// pivoting fallback, and blocked LU solves (the SQBEM_FP64 path; replaces the
// reference's dgemm_/dgetrf_/dgetrs_/dgesv_, src/utils/linalg.hpp:17-78).
//
// GB300 executes FP64 at roughly 1 TFLOP/s (CUDA-core DFMA and DMMA alike), so
// these kernels are register-tiled DFMA loops sized to keep that pipe busy; the
// fast path of the solver is the mixed-precision tensor-core code (tc_gemm.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dense.cuh"

namespace sqbem {

// ---------------------------------------------------------------- GEMM
constexpr int GB_M = 64, GB_N = 64, GB_K = 16;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) dgemm_kernel(int M, int N, int K, double alpha, const double* __restrict__ A,
                                                    long long lda, const double* __restrict__ B, long long ldb,
                                                    double beta, double* __restrict__ C, long long ldc) {
    __shared__ double As[GB_K][GB_M + 1];
    __shared__ double Bs[GB_K][GB_N + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.x * GB_M, n0 = blockIdx.y * GB_N;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < K; k0 += GB_K) {
#pragma unroll
        for (int r = 0; r < (GB_M * GB_K) / 256; ++r) {
            const int e = tid + r * 256;
            const int m = TA ? e / GB_K : e % GB_M;
            const int k = TA ? e % GB_K : e / GB_M;
            const int gm = m0 + m, gk = k0 + k;
            double v = 0.0;
            if (gm < M && gk < K) v = TA ? A[gk + gm * lda] : A[gm + gk * lda];
            As[k][m] = v;
        }
#pragma unroll
        for (int r = 0; r < (GB_N * GB_K) / 256; ++r) {
            const int e = tid + r * 256;
            const int n = TB ? e % GB_N : e / GB_K;
            const int k = TB ? e / GB_N : e % GB_K;
            const int gn = n0 + n, gk = k0 + k;
            double v = 0.0;
            if (gk < K && gn < N) v = TB ? B[gn + gk * ldb] : B[gk + gn * ldb];
            Bs[k][n] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < GB_K; ++k) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[k][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[k][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int gn = n0 + ty + 16 * j;
        if (gn >= N) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int gm = m0 + tx + 16 * i;
            if (gm >= M) continue;
            double* c = C + gm + gn * ldc;
            *c = beta == 0.0 ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *c);
        }
    }
}

void gemm64(bool ta, bool tb, int M, int N, int K, double alpha, const double* A, long long lda, const double* B,
            long long ldb, double beta, double* C, long long ldc, cudaStream_t st) {
    if (M <= 0 || N <= 0) return;
    if (K <= 0) {
        // C = beta C
        if (beta == 1.0) return;
        K = 0;
    }
    dim3 grid(ceil_div(M, GB_M), ceil_div(N, GB_N));
    const double fl = 2.0 * M * N * K;
    const double by = 8.0 * ((double)M * K + (double)K * N + (beta == 0.0 ? 1.0 : 2.0) * M * N);
    if (!ta && !tb)
        TIMED_LAUNCH("dgemm", fl, by, (dgemm_kernel<false, false>), grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb,
                     beta, C, ldc);
    else if (ta && !tb)
        TIMED_LAUNCH("dgemm", fl, by, (dgemm_kernel<true, false>), grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb,
                     beta, C, ldc);
    else if (!ta && tb)
        TIMED_LAUNCH("dgemm", fl, by, (dgemm_kernel<false, true>), grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb,
                     beta, C, ldc);
    else
        TIMED_LAUNCH("dgemm", fl, by, (dgemm_kernel<true, true>), grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb,
                     beta, C, ldc);
}

// ---------------------------------------------------------------- small helpers
__global__ void copy_kernel(const double* __restrict__ s, long long lds, double* __restrict__ d, long long ldd, int rows,
                            int cols) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)rows * cols) return;
    const int r = (int)(t % rows), c = (int)(t / rows);
    d[r + c * ldd] = s[r + c * lds];
}

void copy_matrix64(const double* src, long long lds, double* dst, long long ldd, int rows, int cols, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return;
    LAUNCH(copy_kernel, ceil_div((long long)rows * cols, 256), 256, 0, st, src, lds, dst, ldd, rows, cols);
}

// non-negative doubles order like their bit patterns
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

__global__ void max_abs_kernel(const double* __restrict__ A, long long lda, int rows, int cols, double* out) {
    double m = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)rows * cols;
         t += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(t % rows), c = (int)(t / rows);
        m = fmax(m, fabs(A[r + c * lda]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(out, m);
}

void max_abs64(const double* A, long long lda, int rows, int cols, double* out, cudaStream_t st) {
    CUDA_CHECK(cudaMemsetAsync(out, 0, sizeof(double), st));
    if (rows <= 0 || cols <= 0) return;
    LAUNCH(max_abs_kernel, std::min(ceil_div((long long)rows * cols, 256), 152 * 8), 256, 0, st, A, lda, rows, cols,
           out);
}

// copy W (rows x cols, ld rows) into A and flag |entry| > 1 (bit 0) or a
// non-finite entry (bit 1)
__global__ void copy_check_kernel(const double* __restrict__ W, double* __restrict__ A, long long lda, int rows,
                                  int cols, int* flag) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)rows * cols) return;
    const int r = (int)(t % rows), c = (int)(t / rows);
    const double v = W[t];
    A[r + c * lda] = v;
    if (!(fabs(v) <= 1.0)) atomicOr(flag, isfinite(v) ? 1 : 2);
}

// ---------------------------------------------------------------- diagonal blocks
// Inverses of the unit-lower and upper triangles of the kb x kb block a (shared,
// row stride LU_NB + 1), written column-major with leading dimension LU_NB.
__device__ void block_inverses(const double (*a)[LU_NB + 1], int kb, double* Linv, double* Uinv) {
    const int c = threadIdx.x;
    if (c < kb) {
        // column c of L^{-1}: X(c,c) = 1, X(i,c) = -sum_{k=c}^{i-1} L(i,k) X(k,c)
        for (int i = 0; i < LU_NB; ++i) Linv[i + c * LU_NB] = i == c ? 1.0 : 0.0;
        for (int i = c + 1; i < kb; ++i) {
            double s = 0.0;
            for (int k = c; k < i; ++k) s = fma(a[i][k], Linv[k + c * LU_NB], s);
            Linv[i + c * LU_NB] = -s;
        }
        // column c of U^{-1}: X(c,c) = 1/U(c,c), X(i,c) = -sum_{k=i+1}^{c} U(i,k) X(k,c) / U(i,i)
        for (int i = 0; i < LU_NB; ++i) Uinv[i + c * LU_NB] = 0.0;
        Uinv[c + c * LU_NB] = 1.0 / a[c][c];
        for (int i = c - 1; i >= 0; --i) {
            double s = 0.0;
            for (int k = i + 1; k <= c; ++k) s = fma(a[i][k], Uinv[k + c * LU_NB], s);
            Uinv[i + c * LU_NB] = -s / a[i][i];
        }
    } else if (c < LU_NB) {
        for (int i = 0; i < LU_NB; ++i) {
            Linv[i + c * LU_NB] = 0.0;
            Uinv[i + c * LU_NB] = 0.0;
        }
    }
}

// Factor the kb x kb diagonal block in place without exchanges; flag bit 0 if
// a multiplier exceeds 1 in magnitude, bit 1 on a zero / non-finite pivot.
__global__ void __launch_bounds__(256) lu_diag_kernel(double* A, long long lda, int kb, double* Linv, double* Uinv,
                                                      int* flag) {
    __shared__ double a[LU_NB][LU_NB + 1];
    const int tid = threadIdx.x;
    for (int e = tid; e < kb * kb; e += blockDim.x) a[e % kb][e / kb] = A[(e % kb) + (e / kb) * lda];
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        const double piv = a[j][j];
        if (tid == 0 && !(piv != 0.0 && isfinite(piv))) atomicOr(flag, 2);
        for (int i = j + 1 + tid; i < kb; i += blockDim.x) {
            const double l = a[i][j] / piv;
            a[i][j] = l;
            if (!(fabs(l) <= 1.0)) atomicOr(flag, isfinite(l) ? 1 : 2);
        }
        __syncthreads();
        const int w = kb - j - 1;
        for (int e = tid; e < w * w; e += blockDim.x) {
            const int i = j + 1 + e % w, c = j + 1 + e / w;
            a[i][c] = fma(-a[i][j], a[j][c], a[i][c]);
        }
        __syncthreads();
    }
    for (int e = tid; e < kb * kb; e += blockDim.x) A[(e % kb) + (e / kb) * lda] = a[e % kb][e / kb];
    block_inverses(a, kb, Linv, Uinv);
}

// Inverses of all diagonal blocks of a factored matrix (after the pivoted path).
__global__ void __launch_bounds__(LU_NB) diag_inv_kernel(const double* A, long long lda, int n, double* Linv,
                                                         double* Uinv) {
    __shared__ double a[LU_NB][LU_NB + 1];
    const int k0 = blockIdx.x * LU_NB, kb = min(LU_NB, n - k0);
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x)
        a[e % kb][e / kb] = A[(k0 + e % kb) + (long long)(k0 + e / kb) * lda];
    __syncthreads();
    block_inverses(a, kb, Linv + (long long)blockIdx.x * LU_NB * LU_NB, Uinv + (long long)blockIdx.x * LU_NB * LU_NB);
}

// ---------------------------------------------------------------- pivoted fallback
// Column j of an unblocked right-looking LU with partial pivoting (dgetf2 order).
__global__ void __launch_bounds__(1024) pivot_kernel(const double* A, long long lda, int n, int j, int* ipiv, int* flag) {
    __shared__ double bv[32];
    __shared__ int bi[32];
    double best = -1.0;
    int bidx = n;
    for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
        const double v = fabs(A[i + j * lda]);
        if (v > best) { best = v; bidx = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
    }
    if ((threadIdx.x & 31) == 0) { bv[threadIdx.x >> 5] = best; bi[threadIdx.x >> 5] = bidx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (bv[w] > best || (bv[w] == best && bi[w] < bidx)) { best = bv[w]; bidx = bi[w]; }
        // first maximum, as idamax; a zero column keeps the diagonal
        if (!(best > 0.0)) { bidx = j; atomicOr(flag, 2); }
        ipiv[j] = bidx;
    }
}

__global__ void swap_rows_kernel(double* A, long long lda, int n, int j, const int* ipiv) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int p = ipiv[j];
    if (c >= n || p == j) return;
    const double t = A[j + c * lda];
    A[j + c * lda] = A[p + c * lda];
    A[p + c * lda] = t;
}

__global__ void rank1_kernel(double* A, long long lda, int n, int j) {
    const int i = j + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int c = j + 1 + blockIdx.y;
    if (i >= n || c >= n) return;
    const double piv = A[j + j * lda];
    if (piv == 0.0) return;
    const double l = A[i + j * lda] / piv;
    A[i + c * lda] = fma(-l, A[j + c * lda], A[i + c * lda]);
}

__global__ void scale_col_kernel(double* A, long long lda, int n, int j) {
    const int i = j + 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double piv = A[j + j * lda];
    if (piv != 0.0) A[i + j * lda] = A[i + j * lda] / piv;
}

__global__ void laswp_kernel(double* B, long long ldb, int n, int nrhs, const int* ipiv) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nrhs) return;
    for (int j = 0; j < n; ++j) {
        const int p = ipiv[j];
        if (p != j) {
            const double t = B[j + c * ldb];
            B[j + c * ldb] = B[p + c * ldb];
            B[p + c * ldb] = t;
        }
    }
}

// ---------------------------------------------------------------- LU64
static void run_fast(double* A, long long ld, int n, double* Linv, double* Uinv, int* flag, cudaStream_t st) {
    DevBuf<double> W1((size_t)LU_NB * n, st), W2((size_t)LU_NB * n, st);
    for (int k0 = 0, b = 0; k0 < n; k0 += LU_NB, ++b) {
        const int kb = std::min(LU_NB, n - k0), n2 = n - k0 - kb;
        double* A11 = A + k0 + k0 * ld;
        double* Li = Linv + (long long)b * LU_NB * LU_NB;
        double* Ui = Uinv + (long long)b * LU_NB * LU_NB;
        LAUNCH(lu_diag_kernel, 1, 256, 0, st, A11, ld, kb, Li, Ui, flag);
        if (n2 == 0) break;
        double* A12 = A + k0 + (k0 + kb) * ld;
        double* A21 = A + (k0 + kb) + k0 * ld;
        double* A22 = A + (k0 + kb) + (k0 + kb) * ld;
        // U12 = L11^{-1} A12
        gemm64(false, false, kb, n2, kb, 1.0, Li, LU_NB, A12, ld, 0.0, W1.get(), kb, st);
        copy_matrix64(W1.get(), kb, A12, ld, kb, n2, st);
        // L21 = A21 U11^{-1}, certified |L21| <= 1
        gemm64(false, false, n2, kb, kb, 1.0, A21, ld, Ui, LU_NB, 0.0, W2.get(), n2, st);
        LAUNCH(copy_check_kernel, ceil_div((long long)n2 * kb, 256), 256, 0, st, W2.get(), A21, ld, n2, kb, flag);
        // A22 -= L21 U12
        gemm64(false, false, n2, n2, kb, -1.0, A21, ld, A12, ld, 1.0, A22, ld, st);
    }
}

static void run_pivoted(double* A, long long ld, int n, int* ipiv, double* Linv, double* Uinv, int* flag,
                        cudaStream_t st) {
    for (int j = 0; j < n; ++j) {
        LAUNCH(pivot_kernel, 1, 1024, 0, st, A, ld, n, j, ipiv, flag);
        LAUNCH(swap_rows_kernel, ceil_div(n, 256), 256, 0, st, A, ld, n, j, ipiv);
        if (j + 1 < n) {
            LAUNCH(rank1_kernel, dim3(ceil_div(n - j - 1, 256), n - j - 1), 256, 0, st, A, ld, n, j);
            LAUNCH(scale_col_kernel, ceil_div(n - j - 1, 256), 256, 0, st, A, ld, n, j);
        }
    }
    LAUNCH(diag_inv_kernel, ceil_div(n, LU_NB), LU_NB, 0, st, A, ld, n, Linv, Uinv);
}

static int read_flag(const int* flag, cudaStream_t st) {
    int h = 0;
    CUDA_CHECK(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    count_d2h(sizeof(int));
    CUDA_CHECK(cudaStreamSynchronize(st));
    return h;
}

void LU64::factor_inplace(DevBuf<double>&& M, int n_, cudaStream_t st, const char* what) {
    n = n_;
    ld = n_;
    A = std::move(M);
    const int nblk = ceil_div(n, LU_NB);
    Linv.alloc((size_t)nblk * LU_NB * LU_NB, st);
    Uinv.alloc((size_t)nblk * LU_NB * LU_NB, st);
    DevBuf<int> flag(1, st);
    flag.zero();
    DevBuf<double> saved((size_t)n * n, st);
    CUDA_CHECK(cudaMemcpyAsync(saved.get(), A.get(), sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, st));
    run_fast(A.get(), ld, n, Linv.get(), Uinv.get(), flag.get(), st);
    int f = read_flag(flag.get(), st);
    pivoted = false;
    if (f != 0) {
        // certificate failed: redo with row exchanges from the saved matrix
        CUDA_CHECK(cudaMemcpyAsync(A.get(), saved.get(), sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, st));
        ipiv.alloc((size_t)n, st);
        flag.zero();
        run_pivoted(A.get(), ld, n, ipiv.get(), Linv.get(), Uinv.get(), flag.get(), st);
        pivoted = true;
        f = read_flag(flag.get(), st);
        if (f & 2) fail(SQBEM_ERR_SINGULAR, "%s", what);
    }
}

void LU64::factor(const double* M, int n_, long long ldm, cudaStream_t st, const char* what) {
    DevBuf<double> a((size_t)n_ * n_, st);
    copy_matrix64(M, ldm, a.get(), n_, n_, n_, st);
    factor_inplace(std::move(a), n_, st, what);
}

void LU64::solve(double* B, long long ldb, int nrhs, cudaStream_t st) const {
    if (nrhs <= 0 || n == 0) return;
    // per-call scratch (stream-ordered), so handles sharing one factor on
    // different streams never share a buffer
    DevBuf<double> work((size_t)LU_NB * nrhs, st);
    double* W = work.get();
    if (pivoted) LAUNCH(laswp_kernel, ceil_div(nrhs, 128), 128, 0, st, B, ldb, n, nrhs, ipiv.get());
    const int nblk = ceil_div(n, LU_NB);
    for (int b = 0; b < nblk; ++b) {  // forward: unit lower L
        const int k0 = b * LU_NB, kb = std::min(LU_NB, n - k0);
        gemm64(false, false, kb, nrhs, kb, 1.0, Linv.get() + (long long)b * LU_NB * LU_NB, LU_NB, B + k0, ldb, 0.0, W,
               kb, st);
        copy_matrix64(W, kb, B + k0, ldb, kb, nrhs, st);
        if (k0 + kb < n)
            gemm64(false, false, n - k0 - kb, nrhs, kb, -1.0, A.get() + (k0 + kb) + k0 * ld, ld, B + k0, ldb, 1.0,
                   B + k0 + kb, ldb, st);
    }
    for (int b = nblk - 1; b >= 0; --b) {  // backward: U
        const int k0 = b * LU_NB, kb = std::min(LU_NB, n - k0);
        gemm64(false, false, kb, nrhs, kb, 1.0, Uinv.get() + (long long)b * LU_NB * LU_NB, LU_NB, B + k0, ldb, 0.0, W,
               kb, st);
        copy_matrix64(W, kb, B + k0, ldb, kb, nrhs, st);
        if (k0 > 0)
            gemm64(false, false, k0, nrhs, kb, -1.0, A.get() + k0 * ld, ld, B + k0, ldb, 1.0, B, ldb, st);
    }
}

}  // namespace sqbem

namespace sqbem {

// B <- P^T applied in reverse exchange order (undoes laswp)
__global__ void laswp_reverse_kernel(double* B, long long ldb, int n, int nrhs, const int* ipiv) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nrhs) return;
    for (int j = n - 1; j >= 0; --j) {
        const int p = ipiv[j];
        if (p != j) {
            const double t = B[j + c * ldb];
            B[j + c * ldb] = B[p + c * ldb];
            B[p + c * ldb] = t;
        }
    }
}

// A^T X = B with P A = L U:  A^T = U^T L^T P, so X = P^T L^{-T} U^{-T} B.
// U^T is lower triangular (forward, block inverses transposed), L^T unit upper
// (backward); the off-diagonal blocks enter as transposed GEMM operands.
void LU64::solve_transpose(double* B, long long ldb, int nrhs, cudaStream_t st) const {
    if (nrhs <= 0 || n == 0) return;
    DevBuf<double> work((size_t)LU_NB * nrhs, st);
    double* W = work.get();
    const int nblk = ceil_div(n, LU_NB);
    for (int b = 0; b < nblk; ++b) {  // forward with U^T
        const int k0 = b * LU_NB, kb = std::min(LU_NB, n - k0);
        if (k0 > 0)  // B_k -= (U_{0:k0, k})^T X_{0:k0}
            gemm64(true, false, kb, nrhs, k0, -1.0, A.get() + k0 * ld, ld, B, ldb, 1.0, B + k0, ldb, st);
        gemm64(true, false, kb, nrhs, kb, 1.0, Uinv.get() + (long long)b * LU_NB * LU_NB, LU_NB, B + k0, ldb, 0.0, W,
               kb, st);
        copy_matrix64(W, kb, B + k0, ldb, kb, nrhs, st);
    }
    for (int b = nblk - 1; b >= 0; --b) {  // backward with L^T (unit)
        const int k0 = b * LU_NB, kb = std::min(LU_NB, n - k0);
        if (k0 + kb < n)  // B_k -= (L_{k0+kb:n, k})^T X_{k0+kb:n}
            gemm64(true, false, kb, nrhs, n - k0 - kb, -1.0, A.get() + (k0 + kb) + k0 * ld, ld, B + k0 + kb, ldb, 1.0,
                   B + k0, ldb, st);
        gemm64(true, false, kb, nrhs, kb, 1.0, Linv.get() + (long long)b * LU_NB * LU_NB, LU_NB, B + k0, ldb, 0.0, W,
               kb, st);
        copy_matrix64(W, kb, B + k0, ldb, kb, nrhs, st);
    }
    if (pivoted) LAUNCH(laswp_reverse_kernel, ceil_div(nrhs, 128), 128, 0, st, B, ldb, n, nrhs, ipiv.get());
}

}  // namespace sqbem
