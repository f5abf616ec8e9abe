// solver.cu -- Tube, SwimmerSolver and DuctFlow on the GPU (FP64 path).
//
// Follows the reference's algebra step by step (src/swimmer.hpp:48-288,
// src/duct_flow.hpp:41-108); every block is assembled by assemble.cu and every
// dense step runs in dense64.cu.  Matrices are column-major like the
// reference's Mat (linalg.hpp:30-37).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "assemble.cuh"
#include "common.cuh"
#include "dense.cuh"
#include "solver.cuh"

using namespace sqbem;

namespace {

template <class T>
BlockJob<T> block_job(const DevPanels& tgt, const DevPanels& src, bool same, double mu, T* S, long long lds, T* D,
                      long long ldd) {
    BlockJob<T> j;
    j.tgt = tgt.cent.get();
    j.nT = tgt.P;
    j.src = src.rec.get();
    j.nS = src.P;
    j.same_mesh = same ? 1 : 0;
    j.S = S;
    j.s_rs = 1;
    j.s_cs = lds;
    j.D = D;
    j.d_rs = 1;
    j.d_cs = ldd;
    j.sscale = 1.0 / (EIGHT_PI * mu);
    j.dscale = -1.0 / EIGHT_PI;
    return j;
}

int near_capacity(int nT, int nS) {
    const long long pairs = (long long)nT * nS;
    return (int)std::min<long long>(pairs, 64LL << 20);
}

// copy selected columns: dst(:, k) = src(:, cols[k])
__global__ void gather_cols_kernel(const double* __restrict__ src, long long lds, const int* __restrict__ cols, int ncol,
                                   int rows, double* __restrict__ dst, long long ldd) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)rows * ncol) return;
    const int r = (int)(t % rows), k = (int)(t / rows);
    dst[r + k * ldd] = src[r + (long long)cols[k] * lds];
}

// dst(:, cols[k]) = src(:, cols[k])
__global__ void copy_cols_kernel(const double* __restrict__ src, long long lds, const int* __restrict__ cols, int ncol,
                                 int rows, double* __restrict__ dst, long long ldd) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)rows * ncol) return;
    const int r = (int)(t % rows), k = (int)(t / rows);
    dst[r + (long long)cols[k] * ldd] = src[r + (long long)cols[k] * lds];
}

}  // namespace

// ---------------------------------------------------------------- Tube
void sqbem_tube::build(double R_, double L_, double a_, int nth, int nr, double mu_, int prec) {
    R = R_; L = L_; a = a_; n_theta = nth; n_r = nr; mu = mu_; precision = prec;
    mesh = bem::swimmer_tube_mesh(R, L, a, nth, nr);
    build_device();
}

void sqbem_tube::set_panels() {
    Nt = mesh.P();
    const auto V = mesh_vertices(mesh);
    host_panels = make_panels(V.data(), Nt);
    panels.set(host_panels, st);
}

void sqbem_tube::build_device() {
    set_panels();
    const int n = 3 * Nt;
    if (precision == SQBEM_MIXED) {
        DevBuf<int> flags(2, st);
        flags.zero();
        MixedCtx cx{st, flags.get(), flags.get() + 1};
        mixed_build_tubes({this}, cx);
        CUDA_CHECK(cudaStreamSynchronize(st));
        return;
    }
    DevBuf<double> T((size_t)n * n, st);
    auto job = block_job<double>(panels, panels, true, mu, T.get(), n, nullptr, 0);
    assemble_block(job, near_capacity(Nt, Nt), st, false);
    deflate(T.get(), 1, n, panels, mu, st);
    lu.factor_inplace(std::move(T), n, st, "dgetrf failed");
    CUDA_CHECK(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------- SwimmerSolver
void sqbem_swimmer::set_geometry(const sqbem_tube* t, int Ns_, const double* V, const double* center, double mu_,
                                 int prec) {
    tube = t;
    Ns = Ns_;
    Nt = t ? t->Nt : 0;
    mu = mu_;
    precision = prec;
    std::memcpy(xc, center, 3 * sizeof(double));
    host_panels = make_panels(V, Ns);
    panels.set(host_panels, st);
}

void sqbem_swimmer::build(const sqbem_tube* t, int Ns_, const double* V, const double* center, double mu_, int prec) {
    set_geometry(t, Ns_, V, center, mu_, prec);
    if (precision == SQBEM_MIXED) {
        if (tube && tube->precision != SQBEM_MIXED)
            fail(SQBEM_ERR_ARG, "SwimmerSolver: a mixed-precision swimmer needs a mixed-precision tube");
        EventTimer clock;
        clock.start(st);
        DevBuf<int> flags(2, st);
        flags.zero();
        MixedCtx cx{st, flags.get(), flags.get() + 1};
        mixed_build_swimmers({this}, cx);
        clock.stop(st);
        t_assembly = 0;
        t_schur = clock.seconds();
        return;
    }
    if (tube && tube->precision != SQBEM_FP64)
        fail(SQBEM_ERR_ARG, "SwimmerSolver: an FP64 swimmer needs an FP64 tube");
    build_fp64();
}

void sqbem_swimmer::build_fp64() {
    const int ns = 3 * Ns, nt = 3 * Nt;
    EventTimer clock, clock2;
    clock.start(st);
    DevBuf<double> E((size_t)ns * ns, st), Dt;
    AuBs.alloc((size_t)ns * ns, st);
    DevBuf<double> rsum((size_t)ns * 3, st);
    rsum.zero();
    if (tube) {
        // tube rows <- sphere sources: B (into Y) and A_uBt   (swimmer.hpp:188-198)
        Y.alloc((size_t)nt * (ns + 6), st);
        AuBt.alloc((size_t)nt * ns, st);
        auto j1 = block_job<double>(tube->panels, panels, false, mu, Y.get(), nt, AuBt.get(), nt);
        assemble_block(j1, near_capacity(Nt, Ns), st, false);
        // sphere rows <- tube sources: D and its double-layer row sums (199-207)
        D.alloc((size_t)ns * nt, st);
        Dt.alloc((size_t)ns * nt, st);
        auto j2 = block_job<double>(panels, tube->panels, false, mu, D.get(), ns, Dt.get(), ns);
        assemble_block(j2, near_capacity(Ns, Nt), st, false);
        add_rowsums(Dt.get(), 1, ns, ns, Nt, rsum.get(), st);
        Dt.release();
    }
    // sphere rows <- sphere sources: E and A_uBs (208-216)
    auto j3 = block_job<double>(panels, panels, true, mu, E.get(), ns, AuBs.get(), ns);
    assemble_block(j3, near_capacity(Ns, Ns), st, false);
    add_rowsums(AuBs.get(), 1, ns, ns, Ns, rsum.get(), st);
    // completed double layer; unbounded fluid adds -I (218-220)
    diag_complete(AuBs.get(), 1, ns, Ns, rsum.get(), tube ? 0.0 : 1.0, nullptr, st);
    deflate(E.get(), 1, ns, panels, mu, st);
    // rigid-body map and C = A_u K (222-234)
    const auto Kh = rigid_map(host_panels, xc);
    DevBuf<double> K((size_t)ns * 6, st);
    K.upload(Kh.data(), Kh.size());
    Gc.alloc((size_t)ns * 6, st);
    gemm64(false, false, ns, 6, ns, 1.0, AuBs.get(), ns, K.get(), ns, 0.0, Gc.get(), ns, st);
    if (tube) gemm64(false, false, nt, 6, ns, 1.0, AuBt.get(), nt, K.get(), ns, 0.0, Y.get() + (size_t)nt * ns, nt, st);
    clock.stop(st);
    clock2.start(st);
    Gs = std::move(E);
    if (tube) {
        // Y = T^{-1} [B | Ct];  Gs = E - D Y_s;  Gc = Cs - D Y_c  (238-249)
        tube->lu.solve(Y.get(), nt, ns + 6, st);
        gemm64(false, false, ns, ns, nt, -1.0, D.get(), ns, Y.get(), nt, 1.0, Gs.get(), ns, st);
        gemm64(false, false, ns, 6, nt, -1.0, D.get(), ns, Y.get() + (size_t)nt * ns, nt, 1.0, Gc.get(), ns, st);
    }
    clock2.stop(st);
    t_assembly = clock.seconds();
    t_schur = clock2.seconds();
}

void sqbem_swimmer::factor_M() {
    if (haveM) return;
    const int ns = 3 * Ns, n = ns + 6;
    // M = [Gs | Gc ; scaled force/torque rows | 0]   (swimmer.hpp:108-125)
    DevBuf<double> M((size_t)n * n, st);
    M.zero();
    copy_matrix64(Gs.get(), ns, M.get(), n, ns, ns, st);
    copy_matrix64(Gc.get(), ns, M.get() + (size_t)n * ns, n, ns, 6, st);
    DevBuf<double> amax(1, st);
    max_abs64(Gs.get(), ns, ns, ns, amax.get(), st);
    double h_amax = 0;
    amax.download(&h_amax, 1);
    CUDA_CHECK(cudaStreamSynchronize(st));
    const double sc = h_amax / panels.area_max;
    const auto F = constraint_rows(host_panels, xc, sc);
    count_h2d(F.size() * sizeof(double));
    CUDA_CHECK(cudaMemcpy2DAsync(M.get() + ns, sizeof(double) * n, F.data(), sizeof(double) * 6, sizeof(double) * 6,
                                 ns, cudaMemcpyHostToDevice, st));
    luM.factor_inplace(std::move(M), n, st, "dgesv failed");
    haveM = true;
}

void sqbem_swimmer::solve_free(int nrhs, const double* slips, double* U, double* Om, double* f_sphere,
                               double* f_tube) {
    const int ns = 3 * Ns, nt = 3 * Nt, n = ns + 6;
    if (precision == SQBEM_MIXED) {
        solve_mixed(false, nrhs, slips, U, Om, f_sphere, f_tube);
        return;
    }
    factor_M();
    // reduced right-hand sides (swimmer.hpp:256-269)
    DevBuf<double> u((size_t)ns * nrhs, st), Rh((size_t)n * nrhs, st), rt;
    u.upload(slips, (size_t)ns * nrhs);
    Rh.zero();
    gemm64(false, false, ns, nrhs, ns, -1.0, AuBs.get(), ns, u.get(), ns, 0.0, Rh.get(), n, st);
    if (tube) {
        rt.alloc((size_t)nt * nrhs, st);
        gemm64(false, false, nt, nrhs, ns, -1.0, AuBt.get(), nt, u.get(), ns, 0.0, rt.get(), nt, st);
        tube->lu.solve(rt.get(), nt, nrhs, st);
        gemm64(false, false, ns, nrhs, nt, -1.0, D.get(), ns, rt.get(), nt, 1.0, Rh.get(), n, st);
    }
    luM.solve(Rh.get(), n, nrhs, st);
    // unpack: f_t = T^{-1} r_t - Y x   (swimmer.hpp:274-288)
    std::vector<double> x((size_t)n * nrhs);
    Rh.download(x.data(), x.size());
    if (tube && f_tube) {
        gemm64(false, false, nt, nrhs, n, -1.0, Y.get(), nt, Rh.get(), n, 1.0, rt.get(), nt, st);
        rt.download(f_tube, (size_t)nt * nrhs);
    }
    CUDA_CHECK(cudaStreamSynchronize(st));
    for (int k = 0; k < nrhs; ++k) {
        const double* xk = x.data() + (size_t)k * n;
        for (int c = 0; c < 3; ++c) {
            U[3 * k + c] = xk[ns + c];
            Om[3 * k + c] = xk[ns + 3 + c];
        }
        if (f_sphere) std::memcpy(f_sphere + (size_t)k * ns, xk, sizeof(double) * ns);
    }
    if (!tube && f_tube) { /* no tube panels */ }
    ir_iterations = 0;
    ir_residual = 0;
}

void sqbem_swimmer::solve_prescribed(const double* U, const double* Om, double* f_sphere, double* f_tube) {
    const int ns = 3 * Ns, nt = 3 * Nt, n = ns + 6;
    if (precision == SQBEM_MIXED) {
        const double w[6] = {U[0], U[1], U[2], Om[0], Om[1], Om[2]};
        double Uo[3], Oo[3];
        solve_mixed(true, 1, w, Uo, Oo, f_sphere, f_tube);
        return;
    }
    if (!haveGs) {
        luGs.factor(Gs.get(), ns, ns, st, "dgesv failed");
        haveGs = true;
    }
    // rhs = -Gc w; Gs x = rhs; x = [rhs; w]   (swimmer.hpp:142-153)
    double w[6] = {U[0], U[1], U[2], Om[0], Om[1], Om[2]};
    DevBuf<double> dw(6, st), x((size_t)n, st);
    dw.upload(w, 6);
    gemm64(false, false, ns, 1, 6, -1.0, Gc.get(), ns, dw.get(), 6, 0.0, x.get(), n, st);
    luGs.solve(x.get(), n, 1, st);
    CUDA_CHECK(cudaMemcpyAsync(x.get() + ns, dw.get(), sizeof(double) * 6, cudaMemcpyDeviceToDevice, st));
    if (f_sphere) x.download(f_sphere, ns);
    if (tube && f_tube) {
        DevBuf<double> ft((size_t)nt, st);
        gemm64(false, false, nt, 1, n, -1.0, Y.get(), nt, x.get(), n, 0.0, ft.get(), nt, st);
        ft.download(f_tube, nt);
    }
    CUDA_CHECK(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------- DuctFlow
void sqbem_duct::build(double R_, double L_, int nth, int nz, int nr, double mu_, int prec) {
    R = R_; L = L_; mu = mu_; precision = prec;
    mesh = bem::tube_mesh(R, bem::uniform_z(0, L, nz), nth, nr);
    P = mesh.P();
    const auto V = mesh_vertices(mesh);
    const auto hp = make_panels(V.data(), P);
    panels.set(hp, st);
    const int n = 3 * P;
    cap.clear();
    for (int p = 0; p < P; ++p)
        if (mesh.tags[p] != bem::WALL) cap.push_back(p);
    const int ncap = (int)cap.size();
    // A_f = SL/(8 pi mu) into M, A_u = -DL/(8 pi) into Dsc   (duct_flow.hpp:373-397)
    DevBuf<double> M((size_t)n * n, st), Dsc((size_t)n * n, st);
    auto job = block_job<double>(panels, panels, true, mu, M.get(), n, Dsc.get(), n);
    assemble_block(job, near_capacity(P, P), st, false);
    DevBuf<double> rsum((size_t)n * 3, st);
    rsum.zero();
    add_rowsums(Dsc.get(), 1, n, n, P, rsum.get(), st);
    // known cap tractions f_z -> columns of Fk; unknown u_z columns come from A_u
    std::vector<int> zcols(ncap);
    std::vector<unsigned char> mask(P, 0);
    for (int k = 0; k < ncap; ++k) {
        zcols[k] = 3 * cap[k] + 2;
        mask[cap[k]] = 4;
    }
    DevBuf<int> dz(std::max(ncap, 1), st);
    if (ncap) dz.upload(zcols.data(), ncap);
    Fk.alloc((size_t)n * std::max(ncap, 1), st);
    if (ncap) {
        LAUNCH(gather_cols_kernel, ceil_div((long long)n * ncap, 256), 256, 0, st, M.get(), n, dz.get(), ncap, n,
               Fk.get(), n);
        LAUNCH(copy_cols_kernel, ceil_div((long long)n * ncap, 256), 256, 0, st, Dsc.get(), n, dz.get(), ncap, n,
               M.get(), n);
    }
    DevBuf<unsigned char> dmask(P, st);
    dmask.upload(mask.data(), P);
    diag_complete(M.get(), 1, n, P, rsum.get(), 0.0, dmask.get(), st);
    Dsc.release();
    lu.factor_inplace(std::move(M), n, st, "dgetrf failed");
    CUDA_CHECK(cudaStreamSynchronize(st));
}

void sqbem_duct::solve(double p_in, double p_out, double* u, double* f, double* Q) {
    const int n = 3 * P, ncap = (int)cap.size();
    std::vector<double> fk(ncap);
    for (int k = 0; k < ncap; ++k) fk[k] = mesh.tags[cap[k]] == bem::INLET ? p_in : -p_out;
    DevBuf<double> dfk(std::max(ncap, 1), st), rhs((size_t)n, st);
    if (ncap) dfk.upload(fk.data(), ncap);
    // rhs = -Fk fk (known u are all zero), x = M^{-1} rhs   (duct_flow.hpp:41-63)
    gemm64(false, false, n, 1, ncap, -1.0, Fk.get(), n, dfk.get(), std::max(ncap, 1), 0.0, rhs.get(), n, st);
    lu.solve(rhs.get(), n, 1, st);
    std::vector<double> x(n);
    rhs.download(x.data(), n);
    CUDA_CHECK(cudaStreamSynchronize(st));
    std::vector<double> uu((size_t)n, 0.0), ff((size_t)n, 0.0);
    for (int p = 0; p < P; ++p)
        for (int b = 0; b < 3; ++b) {
            const bool known = !(mesh.tags[p] != bem::WALL && b == 2);
            (known ? ff : uu)[3 * p + b] = x[3 * p + b];
        }
    double q = 0;
    for (int k = 0; k < ncap; ++k) {
        const int p = cap[k];
        ff[3 * p + 2] = fk[k];
        if (mesh.tags[p] == bem::OUTLET) q += uu[3 * p + 2] * mesh.area[p];
    }
    *Q = q;
    if (u) std::memcpy(u, uu.data(), sizeof(double) * n);
    if (f) std::memcpy(f, ff.data(), sizeof(double) * n);
}

// Mixed-precision solve for this swimmer alone (a group of one): in = slip
// fields (Ns x 3 per right-hand side) or, if prescribed, (U, Omega) (6 values).
void sqbem_swimmer::solve_mixed(bool prescribed, int nrhs, const double* in, double* U, double* Om, double* f_sphere,
                                double* f_tube) {
    const int ns = 3 * Ns, nt = 3 * Nt, nc = ns + 6;
    const size_t per_in = prescribed ? 6 : (size_t)ns;
    DevBuf<double> din(per_in * nrhs, st), x((size_t)(nt + nc) * nrhs, st);
    din.upload(in, per_in * nrhs);
    DevBuf<int> flags(2, st);
    flags.zero();
    MixedCtx cx{st, flags.get(), flags.get() + 1};
    mixed_solve({this}, prescribed, {din.get()}, nrhs, {x.get()}, cx, &ir_iterations, &ir_residual);
    std::vector<double> h((size_t)(nt + nc) * nrhs);
    x.download(h.data(), h.size());
    CUDA_CHECK(cudaStreamSynchronize(st));
    for (int k = 0; k < nrhs; ++k) {
        const double* xk = h.data() + (size_t)k * (nt + nc);
        for (int c = 0; c < 3; ++c) {
            U[3 * k + c] = xk[nt + ns + c];
            Om[3 * k + c] = xk[nt + ns + 3 + c];
        }
        if (f_sphere) std::memcpy(f_sphere + (size_t)k * ns, xk + nt, sizeof(double) * ns);
        if (f_tube && nt) std::memcpy(f_tube + (size_t)k * nt, xk, sizeof(double) * nt);
    }
}
