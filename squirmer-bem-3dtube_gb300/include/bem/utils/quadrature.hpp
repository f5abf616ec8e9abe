// quadrature.hpp -- triangle and line quadrature used by the panel integrals.
//
// Same rules as the reference's src/utils/quadrature.hpp:
//   rules()[0..3]: the 7-point degree-5 Dunavant rule and its repetition on the
//   4, 16 and 64 sub-triangles of the reference triangle (7 / 28 / 112 / 448
//   points), barycentric coordinates, weights summing to 1 (quadrature.hpp:22-72);
//   gauss_legendre01(n): n-point Gauss-Legendre on [0, 1] by Newton iteration on
//   the Legendre recurrence (quadrature.hpp:79-99).
// The tables have to be the reference's (down to the point order and the
// operation order that generates them) so that FP64 panel integrals agree to
// rounding; the code that generates them is this project's own.
#pragma once
#include <array>
#include <cmath>
#include <vector>
#include "vec3.hpp"

namespace bem {

struct Rule {
    std::vector<std::array<double, 3>> L;  // barycentric coordinates
    std::vector<double> W;                 // weights, summing to 1
};

// Dunavant (1985) degree-5 rule: centroid + two orbits of three points.
inline Rule dunavant7() {
    const double a1 = 0.059715871789770, b1 = 0.470142064105115, w1 = 0.132394152788506;
    const double a2 = 0.797426985353087, b2 = 0.101286507323456, w2 = 0.125939180544827;
    Rule r;
    r.L.push_back({1. / 3, 1. / 3, 1. / 3});
    r.W.push_back(0.225);
    for (const auto& orbit : {std::array<double, 3>{a1, b1, w1}, std::array<double, 3>{a2, b2, w2}}) {
        const double a = orbit[0], b = orbit[1];
        r.L.push_back({a, b, b});
        r.L.push_back({b, a, b});
        r.L.push_back({b, b, a});
        for (int k = 0; k < 3; ++k) r.W.push_back(orbit[2]);
    }
    return r;
}

// Dunavant-7 on the 4^level congruent sub-triangles obtained by repeated
// midpoint subdivision (corner triangles first, then the central one).
inline Rule subdivided(int level) {
    using Bary = std::array<double, 3>;
    using Tri = std::array<Bary, 3>;
    std::vector<Tri> tris{Tri{Bary{1, 0, 0}, Bary{0, 1, 0}, Bary{0, 0, 1}}};
    auto half = [](const Bary& p, const Bary& q) {
        return Bary{(p[0] + q[0]) / 2, (p[1] + q[1]) / 2, (p[2] + q[2]) / 2};
    };
    for (int l = 0; l < level; ++l) {
        std::vector<Tri> finer;
        finer.reserve(tris.size() * 4);
        for (const Tri& t : tris) {
            const Bary ab = half(t[0], t[1]), bc = half(t[1], t[2]), ca = half(t[2], t[0]);
            finer.push_back({t[0], ab, ca});
            finer.push_back({ab, t[1], bc});
            finer.push_back({ca, bc, t[2]});
            finer.push_back({ab, bc, ca});
        }
        tris.swap(finer);
    }
    const Rule base = dunavant7();
    Rule r;
    for (const Tri& t : tris)
        for (size_t q = 0; q < base.W.size(); ++q) {
            Bary l{0, 0, 0};
            for (int k = 0; k < 3; ++k)
                for (int c = 0; c < 3; ++c) l[c] += base.L[q][k] * t[k][c];
            r.L.push_back(l);
            r.W.push_back(base.W[q] / tris.size());
        }
    return r;
}

// rules()[0] = 7 points, [1] = 28, [2] = 112, [3] = 448
inline const std::vector<Rule>& rules() {
    static const std::vector<Rule> table = {dunavant7(), subdivided(1), subdivided(2), subdivided(3)};
    return table;
}

// n-point Gauss-Legendre nodes x and weights w on [0, 1].
inline void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(PI * (i + 0.75) / (n + 0.5)), dp = 0;
        for (int it = 0; it < 100; ++it) {
            double pn = 1, pm = 0;  // P_j(z), P_{j-1}(z)
            for (int j = 1; j <= n; ++j) {
                const double pmm = pm;
                pm = pn;
                pn = ((2 * j - 1) * z * pm - (j - 1) * pmm) / j;
            }
            dp = n * (z * pn - pm) / (z * z - 1);
            const double step = pn / dp;
            z -= step;
            if (std::fabs(step) < 1e-15) break;
        }
        x[i] = 0.5 * (1 - z);
        w[i] = 1.0 / ((1 - z * z) * dp * dp);
    }
}

}  // namespace bem
