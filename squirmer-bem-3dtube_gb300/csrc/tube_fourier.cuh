// tube_fourier.cuh -- solves with the tube block through its rotational symmetry.
//
// With every panel's 3-vectors written in the frame of its sector (x~ = R_s^T x),
// the deflated tube block T (n_theta-fold symmetric, see tube_sym.cuh) becomes
// block-circulant: T~[(s, a), (t, b)] = C_{t - s}[a, b], C_d[a, b] =
// T[(0, a), (d, b)] R_d, blocks of order n3 = 3 nb.  A discrete Fourier transform
// over the sector index turns it block-diagonal:
//     x^_f = (1 / n) sum_s w^{-f s} x~_s,   y^_f = C^_f x^_f,   y~_s = sum_f w^{f s} y^_f,
//     C^_f = sum_d w^{f d} C_d,  w = exp(2 pi i / n_theta),
// and, T being real, C^_{n - f} = conj(C^_f): n_theta / 2 + 1 complex blocks of
// order n3 determine T^{-1}.  Their inverses are formed once per tube (FP32
// Gauss-Jordan with partial pivoting on a thread-block cluster) and kept as the
// split-BF16 real forms [[Re, -Im], [Im, Re]]; Y = T^{-1} X is then a forward
// transform, one tensor-core GEMM of order 2 n3 per frequency and an inverse
// transform.  For the 128-instance sweep (n_theta = 24, nb = 50 .. 58) this
// replaces the LU of T (3 Nt = 3600 .. 4176) and the triangular solves with it.
#pragma once
#include <cuda_bf16.h>

#include <vector>

#include "common.cuh"
#include "mixed.cuh"
#include "tube_sym.cuh"

namespace sqbem {

constexpr int FT_MAX_SECTORS = 36;   // n_theta handled (frequencies held: n_theta / 2 + 1 <= 19)
constexpr int FT_MAX_ORDER = 256;    // largest block order n3

struct FourierTube {
    int nth = 0, nb = 0, nf = 0;  // sectors, panels per sector, frequencies held
    int n3 = 0;                   // 3 nb: order of a complex block
    int m2 = 0;                   // 2 n3: order of its real form
    int ldk = 0;                  // m2 rounded up to a multiple of 8
    int nt = 0;                   // 3 Nt
    DevBuf<int> panel;            // nb x nth: panel[a * nth + s] = representative a rotated by s sectors
    DevBuf<float2> tw;            // (cos, sin) of 2 pi k / nth, k < nth
    DevBuf<bf16> Ah, Al;          // nf real forms of the block inverses, m2 x m2 row-major (ld ldk), split
};

// Whether a tube with this symmetry takes the Fourier path (n_theta and block
// order within the kernels' limits).
bool fourier_supported(const TubeSymmetry& sym);

// The inverses of the Fourier blocks of every tube, from the sector-0 rows of its
// deflated block (T0: 3 nb x 3 Nt, column-major, leading dimension 3 nb).  A zero
// pivot sets bit 1 of *cx.flag.
void fourier_build(const std::vector<FourierTube*>& ft, const std::vector<const TubeSymmetry*>& sym,
                   const std::vector<const float*>& T0, const MixedCtx& cx);

// Y = T^{-1} X for one tube: X (3 Nt x nc, column-major, leading dimension ldx)
// in FP32 or FP64, Y likewise, and optionally a split copy of Y with any row and
// column strides (column-major for a right operand, row-major for a left one).
struct FourierJob {
    const FourierTube* ft = nullptr;
    const float* x32 = nullptr;
    const double* x64 = nullptr;
    long long ldx = 0;
    int nc = 0;
    float* y32 = nullptr;
    double* y64 = nullptr;
    long long ldy = 0;
    bf16* yh = nullptr;           // split copy: element (r, j) at r * srs + j * scs
    bf16* yl = nullptr;
    long long srs = 1, scs = 0;
};
// Every job of one call: the same input and output precisions.
void fourier_solve(const std::vector<FourierJob>& jobs, const MixedCtx& cx);

}  // namespace sqbem
