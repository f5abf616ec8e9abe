// duct_flow.hpp -- pressure-driven Stokes flow in a finite rigid tube, drop-in
// for src/duct_flow.hpp:22-109 (same constructor, members and methods).
//
//   wall: u = 0; inlet: u_x = u_y = 0, f_z = p_in; outlet: u_x = u_y = 0, f_z = -p_out
// Assembly of the mixed-BC completed boundary integral equation and its LU run
// on the GPU once (constructor); every solve() is one more right-hand side.
#pragma once
#include <cmath>
#include <memory>
#include <vector>
#include "utils/field.hpp"
#include "utils/mesh.hpp"
#include "utils/sqbem_cxx.hpp"

namespace bem {

class DuctFlow {
public:
    Mesh mesh;
    double R, L, mu;

    struct Solution {
        std::vector<V3> u, f;
        double Q = 0;  // volume flow rate through the outlet
    };

    DuctFlow(double R_, double L_, int n_theta, int n_z, int n_r, double mu_ = 1.0, int precision = default_precision())
        : R(R_), L(L_), mu(mu_), precision_(precision) {
        mesh = tube_mesh(R, uniform_z(0, L, n_z), n_theta, n_r);
        sqbem_duct* h = nullptr;
        check(sqbem_duct_create(R, L, n_theta, n_z, n_r, mu, precision, &h));
        handle_.reset(h, sqbem_duct_destroy);
    }

    // true if the velocity component (panel p, component b) is prescribed
    bool u_known(int p, int b) const { return !(mesh.tags[p] != WALL && b == 2); }

    Solution solve(double p_in, double p_out) const {
        const int P = mesh.P();
        std::vector<double> u(3 * (size_t)P), f(3 * (size_t)P);
        Solution s;
        check(sqbem_duct_solve(handle_.get(), p_in, p_out, u.data(), f.data(), &s.Q));
        s.u.resize(P);
        s.f.resize(P);
        for (int p = 0; p < P; ++p) {
            s.u[p] = {u[3 * p], u[3 * p + 1], u[3 * p + 2]};
            s.f[p] = {f[3 * p], f[3 * p + 1], f[3 * p + 2]};
        }
        return s;
    }

    std::vector<V3> velocity(const Solution& s, const std::vector<V3>& pts) const {
        return velocity_at(mesh, s.u, s.f, mu, pts, precision_);
    }

    // Hagen-Poiseuille
    double exact_uz(double r, double dP) const { return dP / L * (R * R - r * r) / (4 * mu); }
    double exact_Q(double dP) const { return PI * std::pow(R, 4) * dP / L / (8 * mu); }

private:
    int precision_;
    std::shared_ptr<sqbem_duct> handle_;
};

}  // namespace bem
