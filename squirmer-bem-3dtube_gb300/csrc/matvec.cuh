// matvec.cuh -- grouped products of FP32 (or FP64) column-major matrices with
// FP64 vectors, accumulated in FP64 (the refinement residuals and the small
// dense products of the mixed path).  HBM-bound: each matrix byte is read once.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"

namespace sqbem {

// y (m x r) = alpha * A (m x n) * x (n x r) + beta * y, r <= 8.
// A column-major with leading dimension lda, FP32 (A32) or FP64 (A64, one set).
struct MvJob {
    const float* A32 = nullptr;
    const double* A64 = nullptr;
    long long lda = 0;
    int m = 0, n = 0, r = 0;
    const double* x = nullptr;
    long long ldx = 0;
    double* y = nullptr;
    long long ldy = 0;
    double alpha = 1, beta = 0;
    // FP32 matrices only: plain FP32 multiply-adds instead of the compensated
    // sum (for products whose error only enters a correction)
    bool plain = false;
};

void matvec_group(const std::vector<MvJob>& jobs, cudaStream_t st);

// y (m x 6, FP64, leading dimension ldy) = A K for the rigid-body map K of a
// sphere (swimmer.hpp:224-231): A (m x 3 Ns, FP32, column-major, lda), K's row
// 3p + b has 1 in column b and the entries of e_c x r_p in the rotation columns
// c = 3, 4, 5 (r_p = centroid of panel p - sphere centre, 3 per panel in rc).
// Compensated FP32 sums like the matvec: per element one error-free sum for
// the translation column and two compensated products for the rotation columns
// (K's zero entries are skipped).
struct RigidJob {
    const float* A = nullptr;
    long long lda = 0;
    int m = 0, np = 0;  // rows, panels (3 np columns)
    const double* rc = nullptr;
    double* y = nullptr;
    long long ldy = 0;
};
void rigid_product_group(const std::vector<RigidJob>& jobs, cudaStream_t st);

// Elementwise helpers on column-major FP64 / FP32 blocks of a group.
struct CopyJob {
    const double* s64 = nullptr;  // one of s64 / s32 as source
    const float* s32 = nullptr;
    long long lds = 0;
    double* d64 = nullptr;  // one of d64 / d32 as destination
    float* d32 = nullptr;
    long long ldd = 0;
    int rows = 0, cols = 0;
    double alpha = 1, beta = 0;  // d = alpha * s + beta * d
};
void copy_group(const std::vector<CopyJob>& jobs, cudaStream_t st);

// sum of squares per column of an FP64 block (rows x cols), written to out[c]
struct NormJob {
    const double* x = nullptr;
    long long ldx = 0;
    int rows = 0, cols = 0;
    double* out = nullptr;
};
void sumsq_group(const std::vector<NormJob>& jobs, cudaStream_t st);

}  // namespace sqbem
