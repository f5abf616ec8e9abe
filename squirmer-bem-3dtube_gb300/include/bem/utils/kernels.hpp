// kernels.hpp -- panel integrals of the Stokeslet and stresslet and the
// squirmer slip; drop-in for src/utils/kernels.hpp:29-111.
//
//   SL_ij = int_p d_ij/|r| + r_i r_j/|r|^3 dS,  DL_ij = int_p -6 r_i r_j (r.m)/|r|^5 dS
// with the reference's adaptive rule (7/28/112/448 points by distance / panel
// size, Duffy self integral).  panel_integrals runs on the GPU: one call per
// pair is supported for compatibility, batched work belongs in
// sqbem_panel_integrals.
#pragma once
#include <array>
#include <vector>
#include "mesh.hpp"
#include "quadrature.hpp"
#include "sqbem_cxx.hpp"
#include "vec3.hpp"

namespace bem {

inline void panel_integrals(const Mesh& M, int p, const V3& x0, bool self, double* SL, double* DL) {
    double V9[9];
    for (int k = 0; k < 3; ++k) {
        V9[3 * k] = M.V[p][k].x;
        V9[3 * k + 1] = M.V[p][k].y;
        V9[3 * k + 2] = M.V[p][k].z;
    }
    const double x[3] = {x0.x, x0.y, x0.z};
    const int s = self ? 1 : 0;
    check(sqbem_panel_integrals(1, V9, x, &s, SL, DL));
}

// u_s = (B1 + B2 cos th) sin th e_th,  sin th e_th = (cos th) rhat - e
inline V3 squirmer_slip(V3 x, V3 center, V3 e, double B1, double B2) {
    const V3 rh = unit(x - center);
    const double ct = dot(rh, e);
    return (B1 + B2 * ct) * (ct * rh - e);
}

}  // namespace bem
