// trajectory.hpp -- time integration of a squirmer's path in a tube, drop-in
// for src/trajectory.hpp:23-151 (same TrajectoryParams, same run_trajectory
// signature, files and status strings).
//
//   dX/dt = U(X, e),  de/dt = Omega(X, e) x e,  3 RK4 steps then Adams-Bashforth 4
// The tube is factored once; each evaluation rebuilds only the swimmer
// couplings on the GPU.  Writes <out_prefix>.csv and keeps <out_prefix>.ckpt
// for restart, byte-compatible with the reference's files.
#pragma once
#include <string>
#include "swimmer.hpp"
#include "utils/io.hpp"
#include "utils/sqbem_cxx.hpp"

namespace bem {

struct TrajectoryParams {
    double alpha = 0;         // B2/B1 (pusher < 0 < puller)
    double a_over_R = 0.3;    // confinement
    double beta0 = 0.5;       // initial offset from the axis, in units of (R - a)
    double pitch0_deg = 0;    // initial tilt toward +x (radial direction)
    double yaw0_deg = 0;      // initial tilt toward +y (azimuthal direction)
    double dt = 0.5;          // time step, units a/B1
    double t_max = 100;
    double L_over_R = 4;      // truncated tube length
    int n_theta = 30;         // tube panels around the circumference
    int sphere_level = 2;     // icosphere refinement (2 -> 320 panels)
    double beta_stop = 0.95;  // stop when the swimmer gets this close to the wall
    double budget_s = 0;      // wall-clock budget per call (0 = unlimited)
};

inline std::string run_trajectory(const TrajectoryParams& P, const std::string& out_prefix, bool verbose = true,
                                  int precision = default_precision()) {
    sqbem_traj_params q;
    q.alpha = P.alpha;
    q.a_over_R = P.a_over_R;
    q.beta0 = P.beta0;
    q.pitch0_deg = P.pitch0_deg;
    q.yaw0_deg = P.yaw0_deg;
    q.dt = P.dt;
    q.t_max = P.t_max;
    q.L_over_R = P.L_over_R;
    q.n_theta = P.n_theta;
    q.sphere_level = P.sphere_level;
    q.beta_stop = P.beta_stop;
    q.budget_s = P.budget_s;
    char status[64] = {0};
    check(sqbem_run_trajectory(&q, out_prefix.c_str(), verbose ? 1 : 0, precision, status, sizeof status));
    return status;
}

}  // namespace bem
