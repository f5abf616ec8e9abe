// squirmer_bem.cpp -- the command-line program of the library: the same input
// files, modes and output files as the reference's squirmer_bem
// (src/main.cpp:27-175), so existing inputs/*.in run unchanged and write
// CSVs in the reference's layout (src/utils/io.hpp format, 10 digits).
//
//   squirmer_bem <input-file> [key=value ...]
//
//   mode = duct        pressure-driven flow in an empty tube: flow_rate.csv,
//                      panels.csv, profile.csv (src/main.cpp:27-62)
//   mode = kinematics  U, Omega of the B1 and B2 modes (and the towed drag on
//                      the axis) for every a/R x beta: kinematics.csv
//                      (src/main.cpp:69-101)
//   mode = field       lab-frame velocity on an x-z grid: field_B1.csv,
//                      field_B2.csv, field_info.csv (src/main.cpp:109-150)
//   mode = trajectory  one swimmer path: <name>.csv and <name>.ckpt
//                      (src/main.cpp:157-175, src/trajectory.hpp)
//
// Built on the drop-in headers over libsqbem.so.  The kinematics mode sends
// every (a/R, beta) of the input to the GPU in one batched call
// (sqbem_kinematics_batch) instead of one solve after another; its "seconds"
// column is the batch's device time divided evenly among the rows.  The
// precision key (fp64 | mixed; default: the SQBEM_PRECISION environment
// variable, else fp64) selects the arithmetic of the kinematics, field and
// trajectory modes; the duct mode is FP64.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "duct_flow.hpp"
#include "swimmer.hpp"
#include "trajectory.hpp"
#include "utils/config.hpp"
#include "utils/io.hpp"

using namespace bem;

namespace {

// the precision key, if given, becomes the drop-in classes' default
// (SQBEM_PRECISION) for the whole run
void apply_precision(const Config& c) {
    if (!c.has("precision")) return;
    const std::string p = c.str("precision");
    if (p != "mixed" && p != "fp64") throw std::runtime_error("unknown precision '" + p + "' (fp64|mixed)");
    setenv("SQBEM_PRECISION", p.c_str(), 1);
}

// ---------------------------------------------------------------- duct
void duct_mode(const Config& c, const std::string& out) {
    const double R = c.num("R", 1.0), L = c.num("L", 4.0), mu = c.num("mu", 1.0);
    const int n_theta = c.integer("n_theta", 24), n_z = c.integer("n_z", 24), n_r = c.integer("n_r", 6);
    const double p_out = c.num("p_out", 0.0), dP_detail = c.num("dP_detail", 1.0);
    const std::vector<double> drops = c.list("dP_list", {0.5, 1, 2, 4});
    const int n_profile = c.integer("n_profile", 20);
    Timer clock;
    const DuctFlow duct(R, L, n_theta, n_z, n_r, mu, SQBEM_FP64);  // one factor, a right-hand side per drop
    std::printf("duct flow: %d panels, %d unknowns, assembled + factorised in %.1f s\n", duct.mesh.P(),
                3 * duct.mesh.P(), clock.seconds());
    {
        Csv rates(out + "/flow_rate.csv", "dP,Q,Q_exact,rel_err");
        for (const double dP : drops) {
            const double Q = duct.solve(p_out + dP, p_out).Q, Qx = duct.exact_Q(dP);
            const double err = std::fabs(Q - Qx) / Qx;
            rates.row({dP, Q, Qx, err});
            std::printf("  dP = %-5g  Q = %.6f   exact %.6f   rel. error %.2e\n", dP, Q, Qx, err);
        }
    }
    const DuctFlow::Solution sol = duct.solve(p_out + dP_detail, p_out);
    write_panels(out + "/panels.csv", duct.mesh, sol.u, sol.f);
    // interior profile at mid-length along three azimuths
    std::vector<V3> pts;
    for (const double phi : {0.0, PI / 5, PI / 2})
        for (int k = 0; k < n_profile; ++k) {
            const double r = 0.95 * R * k / (n_profile - 1);
            pts.push_back({r * std::cos(phi), r * std::sin(phi), L / 2});
        }
    const std::vector<V3> vel = duct.velocity(sol, pts);
    Csv prof(out + "/profile.csv", "x,y,z,r,ux,uy,uz,uz_exact",
             {"interior velocity at z = L/2, dP = " + std::to_string(dP_detail)});
    for (size_t k = 0; k < pts.size(); ++k) {
        const double r = std::hypot(pts[k].x, pts[k].y);
        prof.row({pts[k].x, pts[k].y, pts[k].z, r, vel[k].x, vel[k].y, vel[k].z, duct.exact_uz(r, dP_detail)});
    }
    std::printf("wrote %s/{flow_rate,panels,profile}.csv  (%.1f s)\n", out.c_str(), clock.seconds());
}

// ---------------------------------------------------------------- kinematics
void kinematics_mode(const Config& c, const std::string& out) {
    const std::vector<double> ratios = c.list("a_over_R", {0.3}), betas = c.list("beta", {0.0});
    const int n_theta = c.integer("n_theta", 24), level = c.integer("sphere_level", 3);
    const double L_over_R = c.num("L_over_R", 4.0);
    const bool towed = c.integer("towed_drag", 1) != 0;
    const int prec = default_precision();
    // every (a/R, beta) pair as one instance of a single batched call
    std::vector<sqbem_instance> inst;
    for (const double lam : ratios)
        for (const double beta : betas) {
            sqbem_instance q{};
            q.a_over_R = lam;
            q.beta = lam > 0 ? beta : 0.0;  // unbounded fluid: the sphere sits at the origin
            q.L_over_R = L_over_R;
            q.e[2] = 1.0;
            q.n_theta = n_theta;
            q.n_r = 4;
            q.sphere_level = level;
            q.towed = towed ? 1 : 0;
            inst.push_back(q);
        }
    std::vector<double> res(inst.size() * SQBEM_RESULT_STRIDE);
    double secs = 0;
    check(sqbem_kinematics_batch((int)inst.size(), inst.data(), prec, res.data(), &secs));
    const double per_row = inst.empty() ? 0.0 : secs / inst.size();
    Csv table(out + "/kinematics.csv",
              "a_over_R,beta,panels,UB1x,UB1y,UB1z,OB1x,OB1y,OB1z,UB2x,UB2y,UB2z,OB2x,OB2y,OB2z,drag_K,seconds",
              {"U, Omega for B1=1 (neutral mode) and B2=1 (dipole mode); a=1, mu=1, e=z. "
               "Any squirmer: U = U_B1 + alpha*U_B2. drag_K = axial drag/(6 pi mu a U), sphere on axis only. "
               "a_over_R=0 means unbounded fluid."});
    const double U0 = 2.0 / 3;
    size_t k = 0;
    for (const double lam : ratios)
        for (const double beta : betas) {
            const double* r = res.data() + k++ * SQBEM_RESULT_STRIDE;
            std::vector<double> row = {lam, beta, r[13] + r[14]};
            row.insert(row.end(), r, r + 12);
            row.push_back(r[12]);
            row.push_back(per_row);
            table.row(row);
            std::printf("a/R=%.2f beta=%.2f: U_B1/U0=(%+.4f,%+.4f,%.4f) Om_B1=(%+.4f,%+.4f,%+.4f) "
                        "U_B2/U0=(%+.4f,%+.4f,%+.4f) K=%.4f [%.1fs]\n",
                        lam, beta, r[0] / U0, r[1] / U0, r[2] / U0, r[3], r[4], r[5], r[6] / U0, r[7] / U0, r[8] / U0,
                        r[12], per_row);
        }
}

// ---------------------------------------------------------------- field
void field_mode(const Config& c, const std::string& out) {
    const double a = 1.0;
    const double lam = c.num("a_over_R", 0.3), beta = c.num("beta", 0.0);
    const int n_theta = c.integer("n_theta", 24), level = c.integer("sphere_level", 3);
    const int nx = c.integer("nx", 25), nz = c.integer("nz", 57);
    const double z_extent = c.num("z_extent", 7.0);
    Timer clock;
    // unbounded fluid: the grid spans x_extent instead of the tube's 0.97 R
    const double R = lam > 0 ? a / lam : c.num("x_extent", 4.0) / 0.97;
    std::unique_ptr<Tube> tube;
    if (lam > 0) tube = std::make_unique<Tube>(R, c.num("L_over_R", 4.0) * R, a, n_theta);
    const double b = lam > 0 ? beta * (R - a) : 0.0;
    const V3 e{0, 0, 1}, centre{b, 0, 0};
    SwimmerSolver sw(tube.get(), icosphere(a, level, centre), centre);
    const std::vector<V3> slip1 = sw.slip(e, 1, 0), slip2 = sw.slip(e, 0, 1);
    const std::vector<SwimmerSolution> sol = sw.solve_free({slip1, slip2});
    // grid in the plane y = 0; points within 1.03 a of the centre are masked
    std::vector<V3> grid, fluid;
    std::vector<char> masked;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
            const V3 p{-0.97 * R + 1.94 * R * i / (nx - 1), 0, -z_extent + 2 * z_extent * j / (nz - 1)};
            const bool in = norm(p - centre) < 1.03 * a;
            grid.push_back(p);
            masked.push_back(in ? 1 : 0);
            if (!in) fluid.push_back(p);
        }
    for (int m = 0; m < 2; ++m) {
        const std::vector<V3> v = sw.velocity(sol[m], m == 0 ? slip1 : slip2, fluid);
        const SwimmerSolution& s = sol[m];
        Csv f(out + (m == 0 ? "/field_B1.csv" : "/field_B2.csv"), "x,z,ux,uy,uz",
              {"lab-frame velocity in the plane y=0 for B" + std::to_string(m + 1) +
                   "=1; points inside the sphere are NaN. a_over_R=" + std::to_string(lam) +
                   " beta=" + std::to_string(beta),
               "swimmer U=(" + std::to_string(s.U.x) + "," + std::to_string(s.U.y) + "," + std::to_string(s.U.z) +
                   ")"});
        size_t q = 0;
        for (size_t k = 0; k < grid.size(); ++k) {
            if (masked[k]) {
                f.row({grid[k].x, grid[k].z, NAN, NAN, NAN});
            } else {
                f.row({grid[k].x, grid[k].z, v[q].x, v[q].y, v[q].z});
                ++q;
            }
        }
    }
    Csv info(out + "/field_info.csv", "a_over_R,beta,R,UB1z,UB2z,OB1y");
    info.row({lam, beta, lam > 0 ? R : 0.0, sol[0].U.z, sol[1].U.z, sol[0].Om.y});
    std::printf("field: %zu points x 2 modes, U_B1 = %.5f  (%.1f s)\n", fluid.size(), sol[0].U.z, clock.seconds());
}

// ---------------------------------------------------------------- trajectory
void trajectory_mode(const Config& c, const std::string& out) {
    TrajectoryParams P;
    P.alpha = c.num("alpha", 0);
    P.a_over_R = c.num("a_over_R", 0.3);
    P.beta0 = c.num("beta0", 0.5);
    P.pitch0_deg = c.num("pitch0_deg", 0);
    P.yaw0_deg = c.num("yaw0_deg", 0);
    P.dt = c.num("dt", 0.5);
    P.t_max = c.num("t_max", 100);
    P.L_over_R = c.num("L_over_R", 4);
    P.n_theta = c.integer("n_theta", 30);
    P.sphere_level = c.integer("sphere_level", 2);
    P.beta_stop = c.num("beta_stop", 0.95);
    P.budget_s = c.num("budget_s", 0);
    ensure_dir(out);
    run_trajectory(P, out + "/" + c.str("name", "trajectory"));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <input-file> [key=value ...]\n", argv[0]);
        return 1;
    }
    try {
        Config cfg = Config::load(argv[1]);
        for (int i = 2; i < argc; ++i) cfg.parse_line(argv[i]);  // command-line settings win
        apply_precision(cfg);
        const std::string mode = cfg.str("mode");
        const std::string out = cfg.str("output_dir", "outputs/" + mode);
        ensure_dir(out);
        if (mode == "duct") duct_mode(cfg, out);
        else if (mode == "kinematics") kinematics_mode(cfg, out);
        else if (mode == "field") field_mode(cfg, out);
        else if (mode == "trajectory") trajectory_mode(cfg, out);
        else throw std::runtime_error("unknown mode '" + mode + "' (duct|kinematics|field|trajectory)");
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}
