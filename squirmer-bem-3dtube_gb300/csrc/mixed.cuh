// mixed.cuh -- mixed-precision dense factorisation for the SQBEM_MIXED path:
// LU without row exchanges (certified: every multiplier |l| <= 1, i.e. partial
// pivoting would keep the diagonal) of FP32 matrices, with every O(n^3) step on
// the split-BF16 tensor-core GEMM, recursive so that most of the work runs at
// large K.  All routines act on a GROUP of equally sized matrices (one per
// problem instance), one grouped launch per step.
#pragma once
#include <cuda_bf16.h>

#include <vector>

#include "common.cuh"
#include "tc_gemm.cuh"

namespace sqbem {

constexpr int MX_NB = 128;  // leaf block of the recursive LU / TRSM

inline int pad128(int n) { return (n + MX_NB - 1) / MX_NB * MX_NB; }

// One n x n matrix (n a multiple of 128; rows/columns beyond n_true hold the
// identity) with its split-BF16 copies and the inverses of its diagonal blocks.
struct MixedLU {
    int n = 0, n_true = 0;
    DevBuf<float> A;        // FP32, column-major, ld n; factored in place (unit L below, U on and above)
    DevBuf<bf16> Rh, Rl;    // split copy, row-major (ld n): L blocks and U blocks used as the left operand
    DevBuf<bf16> Ch, Cl;    // split copy, column-major (ld n): U blocks used as the right operand
    DevBuf<float> Li, Ui;   // per diagonal block: L^{-1} and U^{-1} (128 x 128, column-major)
    DevBuf<bf16> LiRh, LiRl, UiRh, UiRl, UiCh, UiCl, LiCh, LiCl;  // their split copies (row- / column-major)
    // the inverses of the factor's 256 x 256 diagonal blocks (row-major split,
    // ld 256, one per pair of 128-blocks), composed after the factorization for
    // the solves' 256-wide leaves
    DevBuf<bf16> L2h, L2l, U2h, U2l;
    bool wide = false;
    void alloc(int n_true, cudaStream_t st);
};

// Right-hand sides being solved in place: X (FP32, column-major, leading
// dimension ldx, n rows, nrhs columns) and a split column-major copy (Sh/Sl,
// leading dimension lds) that the solve keeps equal to the final X, so X can be
// the right operand of a following GEMM.  Optional row-major copy (Rh/Rl, ldr).
struct Rhs {
    float* X = nullptr;
    long long ldx = 0;
    int nrhs = 0;
    bf16* Sh = nullptr;
    bf16* Sl = nullptr;
    long long lds = 0;
    bf16* Rh = nullptr;
    bf16* Rl = nullptr;
    long long ldr = 0;
};

struct MixedCtx {
    cudaStream_t st = nullptr;
    int* err = nullptr;   // device: bounded-wait expiry in a GEMM
    int* flag = nullptr;  // device: bit 0 certificate failed (|l| > 1), bit 1 zero / non-finite pivot
};

// Factor every matrix of the group (A already filled, padding = identity).
void mixed_lu_factor(const std::vector<MixedLU*>& g, const MixedCtx& cx);
// X_k <- A_k^{-1} X_k for every member k.  identity_rhs: X_k holds the identity
// (an inversion), whose zeros above the diagonal the lower solve skips.
void mixed_lu_solve(const std::vector<MixedLU*>& g, const std::vector<Rhs>& rhs, const MixedCtx& cx,
                    bool identity_rhs = false);

// Grouped FP32 -> split-BF16 conversion.
struct ConvJob {
    const float* src;
    long long s_rs, s_cs;
    int rows, cols;
    bf16* hi;
    bf16* lo;
    long long d_rs, d_cs;
};
void convert_group(const std::vector<ConvJob>& jobs, cudaStream_t st);

// out <- A^{-1} in for every member's factor (n_true[k] x r, r <= 8, FP64 in and
// out, leading dimension n_true[k]), one 4-CTA cluster per member: the block
// forward and backward substitutions with the split factor and the block
// inverses, for refinement corrections and few-column solves.
void trsv_group(const std::vector<const MixedLU*>& g, const std::vector<const double*>& in,
                const std::vector<double*>& out, const std::vector<int>& n_true, int r, cudaStream_t st);
// The same with explicit leading dimensions of in and out per member.
struct TrsvIO {
    const double* in = nullptr;
    long long ldi = 0;
    double* out = nullptr;
    long long ldo = 0;
    int n_true = 0;
};
void trsv_group_io(const std::vector<const MixedLU*>& g, const std::vector<TrsvIO>& io, int r, cudaStream_t st);

}  // namespace sqbem
