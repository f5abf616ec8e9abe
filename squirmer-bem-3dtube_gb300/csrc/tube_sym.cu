// tube_sym.cu -- the tube block of the mixed path from the rows of one sector
// (see tube_sym.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "mixed.cuh"
#include "solver.cuh"
#include "tube_fourier.cuh"
#include "tube_sym.cuh"

namespace sqbem {

TubeSymmetry tube_symmetry(const std::vector<PanelRec>& P, int nth) {
    TubeSymmetry S;
    const int n = (int)P.size();
    if (nth < 2 || n == 0 || n % nth != 0) return S;
    const double al = 2.0 * 3.14159265358979323846 / nth;
    double size = 0;
    for (const PanelRec& r : P)
        for (int k = 0; k < 9; ++k) size = std::max(size, std::fabs(r.v[k]));
    const double tol = 1e-10 * size;
    S.nth = nth;
    S.sector.assign(n, -1);
    S.rep.assign(n, -1);
    // sector of a panel: the angular interval of its centroid (the wall, fan and
    // ring triangles of the tube have centroids at least a third of a sector
    // from the interval ends)
    for (int p = 0; p < n; ++p) {
        double phi = std::atan2(P[p].c[1], P[p].c[0]);
        if (phi < 0) phi += 2.0 * 3.14159265358979323846;
        int s = (int)std::floor(phi / al);
        S.sector[p] = std::min(std::max(s, 0), nth - 1);
    }
    for (int p = 0; p < n; ++p)
        if (S.sector[p] == 0) {
            S.rep[p] = (int)S.rep_panel.size();
            S.rep_panel.push_back(p);
        }
    S.nb = (int)S.rep_panel.size();
    if (S.nb * nth != n) return S;
    S.panel.assign((size_t)S.nb * nth, -1);
    for (int p = 0; p < n; ++p) {
        const int s = S.sector[p];
        const double c = std::cos(s * al), sn = std::sin(s * al);
        double v[9];  // the vertices rotated back by s sectors
        for (int k = 0; k < 3; ++k) {
            const double x = P[p].v[3 * k], y = P[p].v[3 * k + 1];
            v[3 * k] = c * x + sn * y;
            v[3 * k + 1] = -sn * x + c * y;
            v[3 * k + 2] = P[p].v[3 * k + 2];
        }
        int found = -1;
        for (int a = 0; a < S.nb && found < 0; ++a) {
            const PanelRec& r = P[S.rep_panel[a]];
            bool eq = true;
            for (int k = 0; k < 9 && eq; ++k) eq = std::fabs(v[k] - r.v[k]) <= tol;
            if (eq) found = a;
        }
        if (found < 0 || S.panel[(size_t)found * nth + s] >= 0) return S;
        S.rep[p] = found;
        S.panel[(size_t)found * nth + s] = p;
    }
    S.ok = true;
    return S;
}

namespace {

// One 3 x 3 block per thread: target panel p (blockIdx.x, threadIdx.x), source
// panel q (blockIdx.y).  T[p, q] = R T0[rep(p), q0] R^T with q0 = rep(q) rotated
// by sector(q) - sector(p), R the rotation of sector(p).
__global__ void tube_fill_kernel(float* __restrict__ T, long long ld, const float* __restrict__ T0, int ld0, int Nt,
                                 int nth, const int* __restrict__ sector, const int* __restrict__ rep,
                                 const int* __restrict__ panel, const float2* __restrict__ rot) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (p >= Nt) return;
    const int sp = sector[p], a = rep[p];
    int s = sector[q] - sp;
    if (s < 0) s += nth;
    const int q0 = panel[rep[q] * nth + s];
    const float2 r = rot[sp];
    const float c = r.x, sn = r.y;
    float A[3][3];
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int al = 0; al < 3; ++al) A[al][b] = T0[(3 * a + al) + (long long)(3 * q0 + b) * ld0];
    // M = A R^T, then R M; R = [[c, -s, 0], [s, c, 0], [0, 0, 1]]
    float M[3][3];
#pragma unroll
    for (int al = 0; al < 3; ++al) {
        M[al][0] = c * A[al][0] - sn * A[al][1];
        M[al][1] = sn * A[al][0] + c * A[al][1];
        M[al][2] = A[al][2];
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        float* col = T + 3LL * p + (long long)(3 * q + b) * ld;
        col[0] = c * M[0][b] - sn * M[1][b];
        col[1] = sn * M[0][b] + c * M[1][b];
        col[2] = M[2][b];
    }
}

// Deflation of the sector-0 rows (swimmer.hpp:64-74, as deflate_kernel does for
// the whole block): T0[3a + al, 3q + b] += sc n_rep(a)[al] n_q[b] area_q.
__global__ void deflate_rows_kernel(float* __restrict__ T0, int ld0, const int* __restrict__ rep_panel, int nb,
                                    const PanelRec* __restrict__ P, int Nt, double sc) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;  // row of T0
    const int c = blockIdx.y;                             // column of T0
    if (r >= 3 * nb) return;
    const int i = rep_panel[r / 3], al = r % 3, q = c / 3, b = c % 3;
    const double v = sc * P[i].n[al] * P[q].n[b] * P[q].area;
    float* e = T0 + r + (long long)c * ld0;
    *e = (float)((double)*e + v);
}

}  // namespace

void assemble_tube_symmetric(const sqbem_tube* t, const TubeSymmetry& sym, float* T, long long ld,
                             cudaStream_t st, DevBuf<float>* T0_out) {
    const int Nt = t->Nt, nb = sym.nb, nth = sym.nth;
    if (!sym.ok || nb * nth != Nt) fail(SQBEM_ERR_ARG, "tube assembly: the panels have no rotational symmetry");
    // rows of sector 0: targets are the representatives' centroids, sources all panels
    std::vector<double> hc(3 * (size_t)nb);
    for (int a = 0; a < nb; ++a)
        for (int k = 0; k < 3; ++k) hc[3 * a + k] = t->host_panels[sym.rep_panel[a]].c[k];
    DevBuf<double> tc(hc.size(), st);
    tc.upload(hc.data(), hc.size());
    DevBuf<int> self(nb, st);
    self.upload(sym.rep_panel.data(), nb);
    const int ld0 = 3 * nb;
    DevBuf<float> T0((size_t)ld0 * 3 * Nt, st);
    T0.zero();
    BlockJob<float> j;
    j.tgt = tc.get();
    j.nT = nb;
    j.src = t->panels.rec.get();
    j.nS = Nt;
    j.self_of = self.get();
    j.S = T0.get();
    j.s_rs = 1;
    j.s_cs = ld0;
    j.sscale = 1.0 / (EIGHT_PI * t->mu);
    j.dscale = -1.0 / EIGHT_PI;
    assemble_block(j, (int)std::min<long long>((long long)nb * Nt, 64LL << 20), st, true);
    const double sc = 1.0 / (EIGHT_PI * t->mu * std::sqrt(t->panels.area_total));
    LAUNCH(deflate_rows_kernel, dim3(ceil_div(ld0, 128), 3 * Nt), 128, 0, st, T0.get(), ld0, self.get(), nb,
           t->panels.rec.get(), Nt, sc);
    // the rotation of every sector and the panel maps
    std::vector<float2> hr(nth);
    const double al = 2.0 * 3.14159265358979323846 / nth;
    for (int s = 0; s < nth; ++s) hr[s] = make_float2((float)std::cos(s * al), (float)std::sin(s * al));
    DevBuf<float2> rot(nth, st);
    rot.upload(hr.data(), nth);
    DevBuf<int> sector(Nt, st), rep(Nt, st), panel((size_t)nb * nth, st);
    sector.upload(sym.sector.data(), Nt);
    rep.upload(sym.rep.data(), Nt);
    panel.upload(sym.panel.data(), (size_t)nb * nth);
    const double bytes = 4.0 * 9.0 * Nt * (double)Nt;
    TIMED_LAUNCH("tube_fill", 0.0, bytes, tube_fill_kernel, dim3(ceil_div(Nt, 128), Nt), 128, 0, st, T, ld, T0.get(),
                 ld0, Nt, nth, sector.get(), rep.get(), panel.get(), rot.get());
    if (T0_out) *T0_out = std::move(T0);
}

}  // namespace sqbem

using namespace sqbem;

// The deflated FP32 tube block of the mixed path (3 Nt x 3 Nt, column-major),
// assembled directly or, with symmetric != 0, from the rows of one sector; for
// tests of the symmetric assembly.  No counterpart in the reference.
extern "C" int sqbem_tube_block_f32(double R, double L, double a, int n_theta, int n_r, double mu, int symmetric,
                                    float* out) {
    return guarded([&] {
        if (!out || !(R > 0) || !(L > 0) || n_theta < 3 || n_r < 1 || !(mu > 0))
            fail(SQBEM_ERR_ARG, "tube_block_f32: bad arguments");
        require_device();
        sqbem_tube t;
        t.R = R; t.L = L; t.a = a; t.n_theta = n_theta; t.n_r = n_r; t.mu = mu;
        t.precision = SQBEM_MIXED;
        t.mesh = bem::swimmer_tube_mesh(R, L, a, n_theta, n_r);
        t.set_panels();
        const int n = 3 * t.Nt;
        DevBuf<float> T((size_t)n * n, t.st);
        T.zero();
        if (symmetric) {  // deflated from the sector-0 rows
            const TubeSymmetry sym = tube_symmetry(t.host_panels, n_theta);
            assemble_tube_symmetric(&t, sym, T.get(), n, t.st);
        } else {
            BlockJob<float> j;
            j.tgt = t.panels.cent.get();
            j.nT = t.Nt;
            j.src = t.panels.rec.get();
            j.nS = t.Nt;
            j.same_mesh = 1;
            j.S = T.get();
            j.s_rs = 1;
            j.s_cs = n;
            j.sscale = 1.0 / (EIGHT_PI * mu);
            j.dscale = -1.0 / EIGHT_PI;
            assemble_block(j, (int)std::min<long long>((long long)t.Nt * t.Nt, 64LL << 20), t.st, true);
            deflate<float>(T.get(), 1, n, t.panels, mu, t.st);
        }
        T.download(out, (size_t)n * n);
        CUDA_CHECK(cudaStreamSynchronize(t.st));
    });
}

// The rotational symmetry the mixed assembly finds in the tube mesh of these
// parameters (host only, no device needed): *nb = panels per sector (0: none);
// sector and rep (Nt ints each, may be null) as in TubeSymmetry.  No
// counterpart in the reference.
extern "C" int sqbem_tube_symmetry(double R, double L, double a, int n_theta, int n_r, int* nb, int* sector, int* rep) {
    return guarded([&] {
        if (!nb || !(R > 0) || !(L > 0) || n_theta < 3 || n_r < 1) fail(SQBEM_ERR_ARG, "tube_symmetry: bad arguments");
        const bem::Mesh m = bem::swimmer_tube_mesh(R, L, a, n_theta, n_r);
        const auto V = mesh_vertices(m);
        const TubeSymmetry S = tube_symmetry(make_panels(V.data(), m.P()), n_theta);
        *nb = S.ok ? S.nb : 0;
        if (!S.ok) return;
        if (sector) std::copy(S.sector.begin(), S.sector.end(), sector);
        if (rep) std::copy(S.rep.begin(), S.rep.end(), rep);
    });
}

// Y = T^{-1} X through the Fourier blocks of the tube of these parameters (X, Y:
// 3 Nt x nc, column-major, host FP64), T the deflated FP32 block that
// sqbem_tube_block_f32 returns with symmetric = 1; for tests of the Fourier
// path.  No counterpart in the reference.
extern "C" int sqbem_tube_fourier_solve(double R, double L, double a, int n_theta, int n_r, double mu, int nc,
                                        const double* X, double* Y) {
    return guarded([&] {
        if (!X || !Y || nc < 1 || !(R > 0) || !(L > 0) || n_theta < 3 || n_r < 1 || !(mu > 0))
            fail(SQBEM_ERR_ARG, "tube_fourier_solve: bad arguments");
        require_device();
        sqbem_tube t;
        t.R = R; t.L = L; t.a = a; t.n_theta = n_theta; t.n_r = n_r; t.mu = mu;
        t.precision = SQBEM_MIXED;
        t.mesh = bem::swimmer_tube_mesh(R, L, a, n_theta, n_r);
        t.set_panels();
        const TubeSymmetry sym = tube_symmetry(t.host_panels, n_theta);
        if (!fourier_supported(sym)) fail(SQBEM_ERR_ARG, "tube_fourier_solve: no Fourier path for this tube");
        const int n = 3 * t.Nt;
        DevBuf<float> T((size_t)n * n, t.st), T0;
        assemble_tube_symmetric(&t, sym, T.get(), n, t.st, &T0);
        DevBuf<int> flags(2, t.st);
        flags.zero();
        MixedCtx cx{t.st, flags.get(), flags.get() + 1};
        FourierTube ft;
        fourier_build({&ft}, {&sym}, {T0.get()}, cx);
        DevBuf<double> dx((size_t)n * nc, t.st), dy((size_t)n * nc, t.st);
        dx.upload(X, (size_t)n * nc);
        FourierJob j;
        j.ft = &ft;
        j.x64 = dx.get(); j.ldx = n; j.nc = nc;
        j.y64 = dy.get(); j.ldy = n;
        fourier_solve({j}, cx);
        dy.download(Y, (size_t)n * nc);
        int h[2] = {};
        flags.download(h, 2);
        CUDA_CHECK(cudaStreamSynchronize(t.st));
        if (h[0]) fail(SQBEM_ERR_TIMEOUT, "tube_fourier_solve: a bounded wait in the tensor-core GEMM expired");
        if (h[1] & 2) fail(SQBEM_ERR_SINGULAR, "tube_fourier_solve: zero pivot in a Fourier block");
    });
}
