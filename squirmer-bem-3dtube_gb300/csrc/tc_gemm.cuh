// tc_gemm.cuh -- split-BF16 tensor-core GEMM (tcgen05 + TMA, sm_103a).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"

namespace sqbem {

using bf16 = __nv_bfloat16;

// A matrix split into two BF16 planes, hi = bf16(x), lo = bf16(x - hi), so that
// hi + lo carries ~16 significant bits of the FP32 value.  Layout:
//   rows x k with the k index contiguous ("K-major"), leading dimension ld
//   (elements, multiple of 8 so rows start on 16-byte boundaries for TMA).
struct SplitMat {
    bf16* hi = nullptr;
    bf16* lo = nullptr;
    int rows = 0, k = 0;
    long long ld = 0;
};

// One GEMM of a grouped launch:
//   C (M x N, FP32) = alpha * A(M x K) * B(K x N) + beta * C
// with A given K-major (a row of A is contiguous: A.rows = M, A.k = K) and B
// given K-major along its columns (B.rows = N, B.k = K, i.e. B^T row-major).
// The products use hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory.
// C may be column-major (c_rs = 1, c_cs = ldc) or row-major (c_rs = ldc, c_cs = 1),
// or absent; optional split outputs write the result as BF16 hi/lo planes.
struct TcProblem {
    int M = 0, N = 0, K = 0;
    float alpha = 1.f, beta = 0.f;
    float* C = nullptr;
    long long c_rs = 1, c_cs = 0;
    bf16* O_hi = nullptr;  // optional split output (same element addressing)
    bf16* O_lo = nullptr;
    long long o_rs = 1, o_cs = 0;
    bf16* P_hi = nullptr;  // optional second split output (e.g. the other layout)
    bf16* P_lo = nullptr;
    long long p_rs = 1, p_cs = 0;
    int check_unit = 0;    // flag |C| > 1 into the certificate word (LU multipliers)
    int tiles_n = 0;       // filled by the launcher
    int tile_start = 0;    // filled by the launcher
    int products = 3;      // 3: hi*hi + hi*lo + lo*hi; 2: hi*hi + hi*lo (A rounded to BF16)
};

struct TcOperands {
    SplitMat A, B;
};

// Launch all problems as one persistent grouped GEMM on stream st.
// err (device int) receives 1 if a bounded wait timed out; flag (device int,
// may be null) receives bit 0 if a check_unit problem saw |C| > 1.  variant:
// the kernel's tile variant (tc_gemm_variants()), or -1 for the one the tuning
// table gives for the problems' shape class.
void tc_gemm(const std::vector<TcProblem>& probs, const std::vector<TcOperands>& ops, int* err, int* flag,
             cudaStream_t st, int variant = -1);

// Tile variants of the GEMM kernel: count, and the tile width (N) and pipeline
// depth of one.
int tc_gemm_variants();
void tc_gemm_variant_info(int variant, int* bn, int* stages);
// The variant the tuning table gives for launches whose largest K and N are
// kmax and nmax.
int tc_gemm_choose(int kmax, int nmax);

// Convert an FP32 matrix (element (r, c) at src[r * s_rs + c * s_cs]) into split
// BF16 planes with element (r, c) at dst[r * d_rs + c * d_cs].
void split_convert(const float* src, long long s_rs, long long s_cs, int rows, int cols, bf16* hi, bf16* lo,
                   long long d_rs, long long d_cs, cudaStream_t st);

// Round a leading dimension up for TMA / swizzle friendliness.
inline long long pad_ld(long long n) { return (n + 63) / 64 * 64; }

}  // namespace sqbem
