// field.hpp -- velocity in the fluid from the boundary solution, drop-in for
// src/utils/field.hpp:18-34:
//   u_j(x0) = 1/(8 pi mu) sum_p SL_p,ij f_p,i - 1/(8 pi) sum_p DL_p,ij u_p,i
// evaluated on the GPU (one warp per point).
#pragma once
#include <vector>
#include "kernels.hpp"

namespace bem {

inline std::vector<V3> velocity_at(const Mesh& M, const std::vector<V3>& u, const std::vector<V3>& f, double mu,
                                   const std::vector<V3>& points, int precision = default_precision()) {
    std::vector<double> V((size_t)M.P() * 9), uu((size_t)M.P() * 3), ff((size_t)M.P() * 3), pts(points.size() * 3),
        out(points.size() * 3);
    for (int p = 0; p < M.P(); ++p) {
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) V[9 * p + 3 * k + c] = M.V[p][k][c];
        for (int c = 0; c < 3; ++c) {
            uu[3 * p + c] = u[p][c];
            ff[3 * p + c] = f[p][c];
        }
    }
    for (size_t n = 0; n < points.size(); ++n)
        for (int c = 0; c < 3; ++c) pts[3 * n + c] = points[n][c];
    check(sqbem_velocity_at(M.P(), V.data(), uu.data(), ff.data(), mu, (int)points.size(), pts.data(), out.data(),
                            precision));
    std::vector<V3> res(points.size());
    for (size_t n = 0; n < points.size(); ++n) res[n] = {out[3 * n], out[3 * n + 1], out[3 * n + 2]};
    return res;
}

}  // namespace bem
