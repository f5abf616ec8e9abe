// mixed_solver.cuh -- state of the SQBEM_MIXED swimmer path.
//
// Full system (t = tube, s = sphere, w = (U, Omega)), as in swimmer.hpp:11-16:
//   [ T  B  Ct ] [f_t]   [b_t]        b_t = -A_uBt u_s
//   [ D  E  Cs ] [f_s] = [b_s]        b_s = -A_uBs u_s
//   [ 0  F  0  ] [ w ]   [ 0 ]        F: force-free / torque-free rows
// Blocks are assembled in FP32 and kept for the FP64 residual.  The
// preconditioner is the Schur elimination on split-BF16 tensor cores: the LU of
// T; Y = T^{-1}[B | Ct] by the LU solves (a tube serving one swimmer) or as one
// GEMM with an explicit T^{-1} (a tube shared by many swimmers); G = [E | Cs] -
// D Y factored (its inverse is never formed: Z = G_s^{-1} G_c and every
// refinement step's G_s^{-1} r come from block substitutions with the factor),
// and the 6 x 6 rigid-body system S6 = F Z solved in FP64.  Every refinement
// step is one triangular solve with T's factor (or a product with T^{-1}), one
// with G_s's factor and a handful of HBM-bound products.
// Iterative refinement on the full system, residuals accumulated in FP64,
// stops when the relative residual reaches REFINE_TOL.
#pragma once
#include <cuda_bf16.h>

#include <memory>
#include <vector>

#include "common.cuh"
#include "mixed.cuh"
#include "sphere_share.cuh"
#include "tube_fourier.cuh"

namespace sqbem {

// Relative FP64 residual |b - A x| / |b| at which the refinement stops.  The
// mixed result differs from the FP64 one mainly through the FP32 storage of the
// assembled blocks (U, Omega: ~2e-7 relative on the sweep workload); a residual
// of 1e-8 lies an order of magnitude below that floor (two refinement steps,
// each contracting the residual ~3e-5; the U, Omega error is the same as at
// 1e-11 to three digits).
constexpr double REFINE_TOL = 1e-8;
// The cap on refinement steps is refine_max_iterations() (sqbem_set_limits).

struct MixedTube {
    int nt = 0, ntp = 0;          // 3 Nt and its multiple of 128
    DevBuf<float> T;              // deflated T (nt x nt, column-major, ld nt), FP32
    // explicit inverse (a tube shared by many swimmers: trajectories, the
    // single-swimmer API) ...
    DevBuf<float> Ti;             // T^{-1}, ntp x ntp column-major (padding: identity)
    DevBuf<bf16> TiRh, TiRl;      // T^{-1} split row-major (left operand of Y = T^{-1}[B | Ct])
    // ... or, for a tube used by one swimmer (the batches), its factor only: Y and
    // the refinement's T^{-1} r come from LU solves, which saves forming T^{-1}
    std::unique_ptr<MixedLU> lu;  // split factor and diagonal-block inverses (A, Ch, Cl released)
    // ... or, for a rotationally symmetric tube (every tube this library meshes),
    // the inverses of its Fourier blocks: T^{-1} X is a transform, one small GEMM
    // per frequency and the inverse transform, for one swimmer or many
    std::unique_ptr<FourierTube> ft;
    bool fourier() const { return ft != nullptr; }
    // T^{-1} formed explicitly (a tube shared by many swimmers, also with Fourier
    // blocks: Y = T^{-1} [B | Ct] is then one large-K GEMM per swimmer, and the
    // refinement's T^{-1} r still goes through the blocks)
    bool explicit_inverse() const { return Ti.get() != nullptr; }
};

struct MixedSwimmer {
    int ns = 0, nt = 0, nc = 0;   // 3 Ns, 3 Nt, 3 Ns + 6
    int nsp = 0;                  // multiple of 128 >= ns
    DevBuf<float> B, AuBt;        // nt x ns
    DevBuf<float> D;              // ns x nt
    DevBuf<float> E, AuBs;        // ns x ns (E unused while `sphere` provides it)
    std::shared_ptr<const SphereBlocks> sphere;  // the call's shared sphere-sphere blocks, if they fit
    const float* e() const { return sphere ? sphere->E.get() : E.get(); }
    DevBuf<float> Ct, Cs;         // nt x 6, ns x 6
    DevBuf<float> Y;              // T^{-1} [B | Ct], nt x nc, leading dimension ldY
    long long ldY = 0;            // nt (explicit T^{-1}) or the padded ntp (the LU solve's buffer)
    std::unique_ptr<MixedLU> glu; // G_s's split factor and diagonal-block inverses (A, Ch, Cl released):
                                  // G_s^{-1} is applied by block substitutions (trsv_group_io)
    DevBuf<double> Z64;           // G_s^{-1} G_c (ns x 6), FP64
    DevBuf<double> F;             // 6 x ns, column-major (ld 6), unscaled
    DevBuf<double> S6i;           // (F Z)^{-1}, 6 x 6 column-major
    DevBuf<double> K;             // rigid-body map, ns x 6
};

}  // namespace sqbem

struct sqbem_tube;
struct sqbem_swimmer;

namespace sqbem {
struct MixedCtx;
// Build the mixed tubes / swimmers of a group (equal padded tube size; for the
// swimmers also equal sphere size).  The assembly runs per member, the dense
// steps as grouped launches.
void mixed_build_tubes(const std::vector<sqbem_tube*>& tubes, const MixedCtx& cx, bool explicit_inverse = true);
// share (may be null): sphere-sphere blocks assembled once for the call; a
// member whose sphere matches them copies / reads them instead of assembling.
void mixed_build_swimmers(const std::vector<sqbem_swimmer*>& sw, const MixedCtx& cx,
                          const std::shared_ptr<const SphereBlocks>& share = nullptr);
// Refined solve of every member for nrhs right-hand sides; x = [f_t; f_s; w]
// per member (device, FP64, (nt + nc) x nrhs), plus the iterations used and the
// final relative residual (max over members and right-hand sides).
//   prescribed = false: force- and torque-free swimming, in = slip fields
//                       (device, ns x nrhs FP64), swimmer.hpp:107-139;
//   prescribed = true:  rigid motion given, in = (U, Omega) (device, 6 x nrhs),
//                       no slip and no constraint rows, swimmer.hpp:142-153.
void mixed_solve(const std::vector<sqbem_swimmer*>& sw, bool prescribed, const std::vector<const double*>& in,
                 int nrhs, const std::vector<double*>& x, const MixedCtx& cx, int* iterations, double* residual);
}  // namespace sqbem
