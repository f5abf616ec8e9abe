// adjoint.cu -- derivatives of the free-swimming (U, Omega) with respect to a
// rigid translation c of the sphere, by the adjoint of the full BEM system.
//
// The system (swimmer.hpp:107-139, 188-249), unknowns z = [f_t; f_s; w], w = (U, Omega):
//   [ T  B   A_uBt K ] [f_t]   [-A_uBt u]
//   [ D  E   A_uBs K ] [f_s] = [-A_uBs u]       A z = b
//   [ 0  F   0       ] [ w ]   [ 0      ]
// Under a translation of the sphere (panels and xc move together, the tube stays)
// T, E, K, F, the slip u and the sphere-sphere part of A_uBs are invariant; B,
// A_uBt (tube rows <- sphere sources), D (sphere rows <- tube sources) and the
// tube part of the completed double layer on the diagonal of A_uBs change.  For
// an output g.z,
//   d(g.z)/dc = lam.(db/dc - dA/dc z),   A^T lam = g,
// and with v = u + K w (the sphere surface velocity) the right side reduces to
//   -lam_t.(dB f_s + dA_uBt v) - lam_s.(dD f_t + d(A_uBs)_diag v),
// one sum over the sphere-tube panel pairs (assemble.cu, adjoint_pairs) with
// the kernel gradients integrated by the assembly's own quadrature.
//
// Transpose solve by block elimination with the stored LU factors:
//   M^T [lam_s; lam_c] = [0; g_w]   (M = [Gs Gc; F 0], the reduced system)
//   lam_t = -T^{-T} D^T lam_s
// lam_c does not enter (the constraint rows do not depend on c).  dU/dB2 needs
// no adjoint: U is linear in the slip, so it is the B2-mode solution itself
// (trajectory.hpp:9-10).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "assemble.cuh"
#include "common.cuh"
#include "dense.cuh"
#include "solver.cuh"

using namespace sqbem;

void sqbem_swimmer::adjoint(int nrhs, const double* slips, double* U, double* Om, double* dU, double* dOm) {
    if (precision != SQBEM_FP64) fail(SQBEM_ERR_ARG, "adjoint: needs an FP64 swimmer (stored LU factors)");
    const int ns = 3 * Ns, nt = 3 * Nt, n = ns + 6;
    std::vector<double> fs((size_t)ns * nrhs), ft((size_t)std::max(nt, 1) * nrhs);
    solve_free(nrhs, slips, U, Om, fs.data(), tube ? ft.data() : nullptr);
    std::fill(dU, dU + 9 * (size_t)nrhs, 0.0);
    std::fill(dOm, dOm + 9 * (size_t)nrhs, 0.0);
    if (!tube) return;  // unbounded fluid: translation invariant
    // sphere surface velocity v = u + U + Omega x (c_p - xc)
    std::vector<double> v((size_t)ns * nrhs);
    for (int k = 0; k < nrhs; ++k)
        for (int p = 0; p < Ns; ++p) {
            const double rx = host_panels[p].c[0] - xc[0], ry = host_panels[p].c[1] - xc[1],
                         rz = host_panels[p].c[2] - xc[2];
            const double* u = slips + (size_t)k * ns + 3 * p;
            const double* w = Om + 3 * k;
            double* o = v.data() + (size_t)k * ns + 3 * p;
            o[0] = u[0] + U[3 * k] + (w[1] * rz - w[2] * ry);
            o[1] = u[1] + U[3 * k + 1] + (w[2] * rx - w[0] * rz);
            o[2] = u[2] + U[3 * k + 2] + (w[0] * ry - w[1] * rx);
        }
    // adjoint vectors for the six outputs (U, Omega)
    std::vector<double> g((size_t)n * 6, 0.0);
    for (int o = 0; o < 6; ++o) g[(size_t)o * n + ns + o] = 1.0;
    DevBuf<double> ls((size_t)n * 6, st), lt((size_t)nt * 6, st);
    ls.upload(g.data(), g.size());
    luM.solve_transpose(ls.get(), n, 6, st);
    gemm64(true, false, nt, 6, ns, -1.0, D.get(), ns, ls.get(), n, 0.0, lt.get(), nt, st);
    tube->lu.solve_transpose(lt.get(), nt, 6, st);
    DevBuf<double> dfs(fs.size(), st), dft(ft.size(), st), dv(v.size(), st), out(6 * ADJ_MAX_MODES * 3, st);
    dfs.upload(fs.data(), fs.size());
    dft.upload(ft.data(), ft.size());
    dv.upload(v.data(), v.size());
    const double gsc = 1.0 / (EIGHT_PI * mu), tsc = 1.0 / EIGHT_PI;
    for (int j0 = 0; j0 < nrhs; j0 += ADJ_MAX_MODES) {
        const int nm = std::min(ADJ_MAX_MODES, nrhs - j0);
        AdjTerm t[2];
        // tube rows <- sphere sources: -lam_t.(dB f_s + dA_uBt v), sources move (+dr)
        t[0].tgt = tube->panels.cent.get(); t[0].nT = Nt;
        t[0].lam = lt.get(); t[0].lam_ld = nt;
        t[0].src = panels.rec.get(); t[0].nS = Ns;
        t[0].f = dfs.get() + (size_t)j0 * ns; t[0].f_ld = ns;
        t[0].v = dv.get() + (size_t)j0 * ns; t[0].v_ld = ns; t[0].v_src = 1;
        t[0].gs = -gsc; t[0].ts = tsc;
        // sphere rows <- tube sources: -lam_s.(dD f_t + d(A_uBs)_diag v), targets move (-dr)
        t[1].tgt = panels.cent.get(); t[1].nT = Ns;
        t[1].lam = ls.get(); t[1].lam_ld = n;
        t[1].src = tube->panels.rec.get(); t[1].nS = Nt;
        t[1].f = dft.get() + (size_t)j0 * nt; t[1].f_ld = nt;
        t[1].v = dv.get() + (size_t)j0 * ns; t[1].v_ld = ns; t[1].v_src = 0;
        t[1].gs = gsc; t[1].ts = tsc;
        adjoint_pairs(t, 2, nm, out.get(), st);
        double h[6 * ADJ_MAX_MODES * 3];
        out.download(h, 6 * ADJ_MAX_MODES * 3);
        CUDA_CHECK(cudaStreamSynchronize(st));
        for (int j = 0; j < nm; ++j)
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < 3; ++k) {
                    dU[9 * (j0 + j) + 3 * a + k] = h[a * ADJ_MAX_MODES * 3 + j * 3 + k];
                    dOm[9 * (j0 + j) + 3 * a + k] = h[(3 + a) * ADJ_MAX_MODES * 3 + j * 3 + k];
                }
    }
}
