// dropin_driver.cpp -- exercises the drop-in header API (duct_flow.hpp,
// swimmer.hpp, trajectory.hpp) the way the reference's programs use it, and
// prints the results as one JSON object for tests/test_gpu_dropin.py.
#include <cstdio>
#include <string>
#include <vector>
#include "duct_flow.hpp"
#include "swimmer.hpp"
#include "trajectory.hpp"
#include "utils/config.hpp"

using namespace bem;

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    std::printf("{");
    {  // DuctFlow(1, 4, 8, 8, 3): Q per pressure drop
        DuctFlow d(1.0, 4.0, 8, 8, 3);
        std::printf("\"duct_P\":%d,\"duct_Q\":[", d.mesh.P());
        const double dps[4] = {0.5, 1, 2, 4};
        for (int k = 0; k < 4; ++k) std::printf("%s%.17g", k ? "," : "", d.solve(dps[k], 0.0).Q);
        std::printf("],");
    }
    {  // off-axis swimmer: a/R = 0.3, beta = 0.4, n_theta = 8, level 1 (main.cpp:69-101)
        const double a = 1.0, lam = 0.3, R = a / lam, b = 0.4 * (R - a);
        Tube tube(R, 4 * R, a, 8);
        SwimmerSolver s(&tube, icosphere(a, 1, {b, 0, 0}), {b, 0, 0});
        const V3 e{0, 0, 1};
        auto m = s.solve_free({s.slip(e, 1, 0), s.slip(e, 0, 1)});
        const double K = -s.force(s.solve_prescribed({0, 0, 1}, {})).z / (6 * PI);
        std::printf("\"U_B1\":[%.17g,%.17g,%.17g],\"Om_B1\":[%.17g,%.17g,%.17g],", m[0].U.x, m[0].U.y, m[0].U.z,
                    m[0].Om.x, m[0].Om.y, m[0].Om.z);
        std::printf("\"U_B2\":[%.17g,%.17g,%.17g],\"Om_B2\":[%.17g,%.17g,%.17g],", m[1].U.x, m[1].U.y, m[1].U.z,
                    m[1].Om.x, m[1].Om.y, m[1].Om.z);
        std::printf("\"drag_K\":%.17g,", K);
    }
    {  // config reader and trajectory (test_trajectory.cpp-style use)
        Config c;
        c.parse_line("alpha = -1.5   # pusher");
        c.parse_line("dP_list = 0.5, 1 2");
        TrajectoryParams P;
        P.alpha = c.num("alpha", 0);
        P.beta0 = 0.5;
        P.pitch0_deg = 5;
        P.yaw0_deg = 10;
        P.dt = 0.5;
        P.t_max = 3.0;
        P.n_theta = 12;
        P.sphere_level = 1;
        const std::string st = run_trajectory(P, dir + "/dropin_traj", false);
        std::printf("\"list\":[%g,%g,%g],\"traj_status\":\"%s\"", c.list("dP_list")[0], c.list("dP_list")[1],
                    c.list("dP_list")[2], st.c_str());
    }
    std::printf("}\n");
    return 0;
}
