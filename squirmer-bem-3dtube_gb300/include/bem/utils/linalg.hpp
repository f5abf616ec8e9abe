// linalg.hpp -- column-major dense matrix and the dense solves, drop-in for
// src/utils/linalg.hpp:31-78.  The solves run on the GPU (sqbem_solve_dense:
// certified no-exchange LU with a partial-pivoting fallback, dgesv semantics).
#pragma once
#include <stdexcept>
#include <vector>
#include "sqbem_cxx.hpp"

namespace bem {

// element (i, j) at a[i + j * n]
struct Mat {
    int n = 0, m = 0;
    std::vector<double> a;
    Mat() = default;
    Mat(int rows, int cols) : n(rows), m(cols), a((size_t)rows * cols, 0.0) {}
    double& operator()(int i, int j) { return a[i + (size_t)j * n]; }
    double operator()(int i, int j) const { return a[i + (size_t)j * n]; }
};

// C = alpha A B + beta C (host; small products)
inline void gemm(double alpha, const Mat& A, const Mat& B, double beta, Mat& C) {
    if (A.m != B.n || C.n != A.n || C.m != B.m) throw std::runtime_error("gemm: dimension mismatch");
    for (int j = 0; j < C.m; ++j)
        for (int i = 0; i < C.n; ++i) {
            double s = 0;
            for (int k = 0; k < A.m; ++k) s += A(i, k) * B(k, j);
            C(i, j) = alpha * s + (beta == 0 ? 0.0 : beta * C(i, j));
        }
}

// B <- A^{-1} B on the GPU
inline void solve_dense(Mat A, Mat& B) {
    if (A.n != A.m || B.n != A.n) throw std::runtime_error("dgesv failed");
    if (sqbem_solve_dense(A.n, B.m, A.a.data(), B.a.data(), nullptr) != SQBEM_OK)
        throw std::runtime_error("dgesv failed");
}

// keeps the matrix; every solve factors it on the GPU (compatibility type)
struct LUFactor {
    Mat LU;
    void factor(Mat A) { LU = std::move(A); }
    void solve(Mat& B) const {
        if (B.m == 0) return;
        solve_dense(LU, B);
    }
};

}  // namespace bem
