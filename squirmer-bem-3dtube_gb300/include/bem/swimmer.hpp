// swimmer.hpp -- a spherical squirmer in a closed rigid tube (or in unbounded
// fluid), drop-in for src/swimmer.hpp:33-289 (same classes, members and
// methods).
//
//   tube wall and caps: u = 0;  sphere: u = U + Omega x (x - xc) + u_s(x)
//   unknowns: tractions everywhere, U, Omega;  force- and torque-free closure
// Tube assembles and factors the tube block on the GPU once; SwimmerSolver
// assembles the swimmer couplings and eliminates them onto (f_s, U, Omega)
// through the Schur complement, all on the GPU.  The precision defaults to
// FP64 (SQBEM_PRECISION=mixed: split-BF16 tensor cores with FP64 refinement).
#pragma once
#include <memory>
#include <vector>
#include "utils/field.hpp"
#include "utils/io.hpp"
#include "utils/kernels.hpp"
#include "utils/linalg.hpp"
#include "utils/mesh.hpp"
#include "utils/sqbem_cxx.hpp"

namespace bem {

struct Tube {
    Mesh mesh;
    int Nt = 0;
    double R = 1, L = 4, mu = 1;
    int precision = SQBEM_FP64;

    Tube() = default;
    Tube(double R_, double L_, double a, int n_theta, int n_r = 4, double mu_ = 1, int prec = default_precision())
        : R(R_), L(L_), mu(mu_), precision(prec) {
        mesh = swimmer_tube_mesh(R, L, a, n_theta, n_r);
        Nt = mesh.P();
        sqbem_tube* h = nullptr;
        check(sqbem_tube_create(R, L, a, n_theta, n_r, mu, precision, &h));
        handle_.reset(h, sqbem_tube_destroy);
    }
    const sqbem_tube* handle() const { return handle_.get(); }

    // rank-one deflation of the null mode f = c m on panels [p0, p0 + np) of M
    // (host form, for matrices a caller assembles itself)
    static void deflate(const Mesh& M, int p0, int np, Mat& A, int off, double mu) {
        double At = 0;
        for (int p = p0; p < p0 + np; ++p) At += M.area[p];
        const double sc = 1.0 / (EIGHT_PI * mu * std::sqrt(At));
        for (int i = 0; i < np; ++i)
            for (int p = 0; p < np; ++p)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        A(off + 3 * i + a, off + 3 * p + b) +=
                            sc * M.normal[p0 + i][a] * M.normal[p0 + p][b] * M.area[p0 + p];
    }

private:
    std::shared_ptr<sqbem_tube> handle_;
};

struct SwimmerSolution {
    V3 U, Om;
    std::vector<V3> f_sphere, f_tube;  // tractions (f = sigma.m, m out of the fluid)
};

class SwimmerSolver {
public:
    const Tube* tube;  // nullptr -> unbounded fluid
    Mesh S;            // sphere mesh
    V3 xc;
    double mu;
    int Ns, Nt;
    double t_assembly = 0, t_schur = 0;

    SwimmerSolver(const Tube* t, const Mesh& sphere, V3 center, double mu_ = 1.0)
        : tube(t), S(sphere), xc(center), mu(mu_) {
        Ns = S.P();
        Nt = tube ? tube->Nt : 0;
        precision_ = tube ? tube->precision : default_precision();
        std::vector<double> V((size_t)Ns * 9);
        for (int p = 0; p < Ns; ++p)
            for (int k = 0; k < 3; ++k)
                for (int c = 0; c < 3; ++c) V[9 * p + 3 * k + c] = S.V[p][k][c];
        const double c[3] = {xc.x, xc.y, xc.z};
        sqbem_swimmer* h = nullptr;
        check(sqbem_swimmer_create(tube ? tube->handle() : nullptr, Ns, V.data(), S.tags.data(), c, mu, precision_,
                                   &h));
        handle_.reset(h, sqbem_swimmer_destroy);
        check(sqbem_swimmer_timings(h, &t_assembly, &t_schur));
    }

    // squirming slip on every sphere panel for orientation e and modes B1, B2
    std::vector<V3> slip(V3 e, double B1, double B2) const {
        std::vector<V3> u(Ns);
        for (int p = 0; p < Ns; ++p) u[p] = squirmer_slip(S.centroid[p], xc, e, B1, B2);
        return u;
    }

    // force- and torque-free swimming, one solution per slip field
    std::vector<SwimmerSolution> solve_free(const std::vector<std::vector<V3>>& slips) {
        const int nr = (int)slips.size();
        std::vector<double> in((size_t)nr * Ns * 3), U(3 * (size_t)nr), Om(3 * (size_t)nr), fs((size_t)nr * Ns * 3),
            ft((size_t)nr * Nt * 3);
        for (int k = 0; k < nr; ++k)
            for (int p = 0; p < Ns; ++p)
                for (int c = 0; c < 3; ++c) in[((size_t)k * Ns + p) * 3 + c] = slips[k][p][c];
        check(sqbem_swimmer_solve_free(handle_.get(), nr, in.data(), U.data(), Om.data(), fs.data(),
                                       Nt ? ft.data() : nullptr));
        std::vector<SwimmerSolution> out(nr);
        for (int k = 0; k < nr; ++k) unpack(&U[3 * k], &Om[3 * k], &fs[(size_t)k * Ns * 3], &ft[(size_t)k * Nt * 3], out[k]);
        return out;
    }

    // rigid sphere with prescribed (U, Omega) and no slip ("towed" problem)
    SwimmerSolution solve_prescribed(V3 U, V3 Om) {
        const double u[3] = {U.x, U.y, U.z}, w[3] = {Om.x, Om.y, Om.z};
        std::vector<double> fs((size_t)Ns * 3), ft((size_t)Nt * 3);
        check(sqbem_swimmer_solve_prescribed(handle_.get(), u, w, fs.data(), Nt ? ft.data() : nullptr));
        SwimmerSolution s;
        unpack(u, w, fs.data(), ft.data(), s);
        return s;
    }

    // hydrodynamic force ON the sphere: F = -sum f dA (m points into it)
    V3 force(const SwimmerSolution& s) const {
        V3 F{};
        for (int p = 0; p < Ns; ++p) F = F - S.area[p] * s.f_sphere[p];
        return F;
    }

    // velocity at points in the fluid (lab frame)
    std::vector<V3> velocity(const SwimmerSolution& s, const std::vector<V3>& slip_field,
                             const std::vector<V3>& pts) const {
        const Mesh all = tube ? merge(tube->mesh, S) : S;
        std::vector<V3> u(all.P()), f(all.P());
        for (int p = 0; p < Nt; ++p) f[p] = s.f_tube[p];
        for (int p = 0; p < Ns; ++p) {
            u[Nt + p] = s.U + cross(s.Om, S.centroid[p] - xc) + slip_field[p];
            f[Nt + p] = s.f_sphere[p];
        }
        return velocity_at(all, u, f, mu, pts, precision_);
    }

private:
    int precision_;
    std::shared_ptr<sqbem_swimmer> handle_;

    void unpack(const double* U, const double* Om, const double* fs, const double* ft, SwimmerSolution& s) const {
        s.U = {U[0], U[1], U[2]};
        s.Om = {Om[0], Om[1], Om[2]};
        s.f_sphere.resize(Ns);
        for (int p = 0; p < Ns; ++p) s.f_sphere[p] = {fs[3 * p], fs[3 * p + 1], fs[3 * p + 2]};
        s.f_tube.resize(Nt);
        for (int p = 0; p < Nt; ++p) s.f_tube[p] = {ft[3 * p], ft[3 * p + 1], ft[3 * p + 2]};
    }
};

}  // namespace bem
