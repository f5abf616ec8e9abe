// mesh.hpp -- flat-triangle surface meshes for the BEM: closed tube (wall + two
// caps) and volume-corrected icosphere.  Host code; the GPU receives per-panel
// vertex triples.
//
// Drop-in for the reference's src/utils/mesh.hpp (same names, fields and
// conventions):
//   * normals point OUT OF THE FLUID: tube wall radially outward, inlet cap -z,
//     outlet cap +z, sphere toward its centre (mesh.hpp:4-6);
//   * tags WALL 0, INLET 1, OUTLET 2, SPHERE 10 (mesh.hpp:45);
//   * node order, triangle order and the floating-point operation order are the
//     reference's, so every coordinate, normal, centroid, area and h is
//     bit-identical (tests/test_abi.py::test_meshes_bitwise_match_reference
//     checks this against fixtures written by the reference).
#pragma once
#include <algorithm>
#include <array>
#include <cstdint>
#include <unordered_map>
#include <utility>
#include <vector>
#include "vec3.hpp"

namespace bem {

enum Tag { WALL = 0, INLET = 1, OUTLET = 2, SPHERE = 10 };

struct Mesh {
    std::vector<V3> nodes;
    std::vector<std::array<int, 3>> tris;
    std::vector<int> tags;
    // per-panel geometry, filled by geometry()
    std::vector<std::array<V3, 3>> V;
    std::vector<V3> normal, centroid;
    std::vector<double> area, h;  // h = sqrt(2 area)

    int P() const { return (int)tris.size(); }

    void geometry() {
        const int n = P();
        V.assign(n, {});
        normal.assign(n, {});
        centroid.assign(n, {});
        area.assign(n, 0.0);
        h.assign(n, 0.0);
        for (int p = 0; p < n; ++p) {
            const auto& t = tris[p];
            V[p] = {nodes[t[0]], nodes[t[1]], nodes[t[2]]};
            const V3 c = cross(V[p][1] - V[p][0], V[p][2] - V[p][0]);
            area[p] = 0.5 * norm(c);
            normal[p] = (1.0 / (2 * area[p])) * c;
            centroid[p] = (1.0 / 3) * (V[p][0] + V[p][1] + V[p][2]);
            h[p] = std::sqrt(2 * area[p]);
        }
    }

    // Flip every panel whose normal points against outward(centroid).
    template <class F>
    void orient(F outward) {
        geometry();
        for (int p = 0; p < P(); ++p)
            if (dot(normal[p], outward(centroid[p])) < 0) std::swap(tris[p][1], tris[p][2]);
        geometry();
    }

    void translate(V3 d) {
        for (auto& x : nodes) x = x + d;
        geometry();
    }

    double total_area() const {
        double s = 0;
        for (double A : area) s += A;
        return s;
    }
};

inline Mesh merge(const Mesh& a, const Mesh& b) {
    Mesh m = a;
    const int off = (int)a.nodes.size();
    m.nodes.insert(m.nodes.end(), b.nodes.begin(), b.nodes.end());
    m.tris.reserve(a.tris.size() + b.tris.size());
    for (const auto& t : b.tris) m.tris.push_back({t[0] + off, t[1] + off, t[2] + off});
    m.tags.insert(m.tags.end(), b.tags.begin(), b.tags.end());
    m.geometry();
    return m;
}

// nz + 1 equally spaced axial nodes on [z0, z1]
inline std::vector<double> uniform_z(double z0, double z1, int nz) {
    std::vector<double> z;
    z.reserve(nz + 1);
    for (int k = 0; k <= nz; ++k) z.push_back(z0 + (z1 - z0) * k / nz);
    return z;
}

// Axial nodes on [-L/2, L/2], symmetric about 0: spacing dzmin up to |z| = core,
// then growing by `growth` per panel up to dzmax.  A last panel thinner than
// 0.3 dz is absorbed into its neighbour.
inline std::vector<double> graded_z(double L, double dzmin, double dzmax, double core,
                                    double growth = 1.25) {
    const double half_len = L / 2;
    std::vector<double> pos{0.0};
    double dz = dzmin;
    while (pos.back() < half_len - 1e-12) {
        if (pos.back() >= core) dz = std::min(dz * growth, dzmax);
        pos.push_back(std::min(pos.back() + dz, half_len));
    }
    if (pos.size() > 2 && half_len - pos[pos.size() - 2] < 0.3 * dz) pos.erase(pos.end() - 2);
    std::vector<double> z;
    z.reserve(2 * pos.size() - 1);
    for (auto it = pos.rbegin(); it != pos.rend(); ++it) z.push_back(-*it);
    z.insert(z.end(), pos.begin() + 1, pos.end());
    return z;
}

namespace detail {

// Flat cap disc at height z0: centre node + nr rings of n_theta nodes.
inline Mesh tube_cap(double z0, int tag, double sign, double Rp, double al, int nth, int nr) {
    Mesh m;
    m.nodes.push_back({0, 0, z0});
    for (int k = 1; k <= nr; ++k)
        for (int i = 0; i < nth; ++i)
            m.nodes.push_back({Rp * k / nr * std::cos(i * al), Rp * k / nr * std::sin(i * al), z0});
    auto node = [nth](int ring, int i) { return 1 + ring * nth + i % nth; };
    for (int i = 0; i < nth; ++i) m.tris.push_back({0, node(0, i), node(0, i + 1)});
    for (int k = 0; k + 1 < nr; ++k)
        for (int i = 0; i < nth; ++i) {
            const int a = node(k, i), b = node(k, i + 1), c = node(k + 1, i + 1), d = node(k + 1, i);
            m.tris.push_back({a, d, c});
            m.tris.push_back({a, c, b});
        }
    m.tags.assign(m.tris.size(), tag);
    m.orient([sign](V3) { return V3{0, 0, sign}; });
    return m;
}

}  // namespace detail

// Closed tube of radius R around the z axis with axial nodes z.  Polygon vertices
// sit on the radius Rp = R sqrt(al / sin al) that gives the faceted cross-section
// the area of the circle.
inline Mesh tube_mesh(double R, const std::vector<double>& z, int nth, int nr) {
    const double al = 2 * PI / nth;
    const double Rp = R * std::sqrt(al / std::sin(al));
    const int nz = (int)z.size() - 1;
    Mesh wall;
    wall.nodes.reserve((size_t)nth * (nz + 1));
    for (int i = 0; i < nth; ++i)
        for (int k = 0; k <= nz; ++k) wall.nodes.push_back({Rp * std::cos(i * al), Rp * std::sin(i * al), z[k]});
    auto node = [nth, nz](int i, int k) { return (i % nth) * (nz + 1) + k; };
    for (int i = 0; i < nth; ++i)
        for (int k = 0; k < nz; ++k) {
            const int a = node(i, k), b = node(i + 1, k), c = node(i + 1, k + 1), d = node(i, k + 1);
            wall.tris.push_back({a, b, c});
            wall.tris.push_back({a, c, d});
        }
    wall.tags.assign(wall.tris.size(), WALL);
    wall.orient([](V3 x) { return V3{x.x, x.y, 0}; });
    const Mesh inlet = detail::tube_cap(z.front(), INLET, -1.0, Rp, al, nth, nr);
    const Mesh outlet = detail::tube_cap(z.back(), OUTLET, 1.0, Rp, al, nth, nr);
    return merge(merge(wall, inlet), outlet);
}

// Tube for the swimmer problems: centred on z = 0, graded axially with spacing
// 0.6 h inside |z| < a + R/2 growing to 1.4 h, h = 2 pi R / n_theta.
inline Mesh swimmer_tube_mesh(double R, double L, double a, int nth, int nr = 4) {
    const double h = 2 * PI * R / nth;
    return tube_mesh(R, graded_z(L, 0.6 * h, 1.4 * h, a + 0.5 * R), nth, nr);
}

// Icosphere of radius a (20 * 4^level panels) scaled to the volume of the sphere,
// normals pointing into the sphere.
inline Mesh icosphere(double a, int level, V3 center = {}, int tag = SPHERE) {
    const double g = (1 + std::sqrt(5.0)) / 2;
    std::vector<V3> v = {{-1, g, 0}, {1, g, 0}, {-1, -g, 0}, {1, -g, 0}, {0, -1, g}, {0, 1, g},
                         {0, -1, -g}, {0, 1, -g}, {g, 0, -1}, {g, 0, 1}, {-g, 0, -1}, {-g, 0, 1}};
    for (auto& x : v) x = unit(x);
    std::vector<std::array<int, 3>> F = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11},
                                         {1, 5, 9}, {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                                         {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8}, {3, 8, 9},
                                         {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    for (int l = 0; l < level; ++l) {
        std::unordered_map<std::uint64_t, int> edge_mid;
        edge_mid.reserve(F.size() * 2);
        auto midpoint = [&](int i, int j) {
            const std::uint64_t key = ((std::uint64_t)std::min(i, j) << 32) | (std::uint32_t)std::max(i, j);
            auto found = edge_mid.find(key);
            if (found != edge_mid.end()) return found->second;
            v.push_back(unit(v[i] + v[j]));
            const int id = (int)v.size() - 1;
            edge_mid.emplace(key, id);
            return id;
        };
        std::vector<std::array<int, 3>> next;
        next.reserve(F.size() * 4);
        for (const auto& f : F) {
            const int ab = midpoint(f[0], f[1]);
            const int bc = midpoint(f[1], f[2]);
            const int ca = midpoint(f[2], f[0]);
            next.push_back({f[0], ab, ca});
            next.push_back({f[1], bc, ab});
            next.push_back({f[2], ca, bc});
            next.push_back({ab, bc, ca});
        }
        F.swap(next);
    }
    double vol6 = 0;  // six times the polyhedron volume
    for (const auto& f : F) vol6 += dot(v[f[0]], cross(v[f[1]], v[f[2]]));
    const double s = std::cbrt(4 * PI / 3 / (std::fabs(vol6) / 6));
    Mesh m;
    m.nodes.reserve(v.size());
    for (const auto& x : v) m.nodes.push_back(center + (a * s) * x);
    m.tris = F;
    m.tags.assign(F.size(), tag);
    m.orient([center](V3 x) { return center - x; });
    return m;
}

}  // namespace bem
