// ref_dump.cpp -- golden-vector dumper compiled against the UNMODIFIED reference
// headers (squirmer-bem-3dtube, src/*.hpp).  Test infrastructure only: it is built
// by oracle/Makefile into oracle/_ref/ and run by tests/golden/make_golden.py to
// write the JSON fixtures under tests/golden/.  Nothing in the product links it.
//
// Each case prints one JSON object with every double at 17 significant digits.
//   ref_dump <case> [tmpdir]
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include "duct_flow.hpp"
#include "swimmer.hpp"
#include "trajectory.hpp"

using namespace bem;

namespace {

struct Json {
    std::string s;
    bool first = true;
    void sep() { if (!first) s += ","; first = false; }
    void open() { s += "{"; first = true; }
    void close() { s += "}"; first = false; }
    static std::string num(double v) {
        if (v != v) return "NaN";
        char b[40];
        std::snprintf(b, sizeof b, "%.17g", v);
        return b;
    }
    void key(const std::string& k) { sep(); s += "\"" + k + "\":"; }
    void kv(const std::string& k, double v) { key(k); s += num(v); }
    void kvs(const std::string& k, const std::string& v) { key(k); s += "\"" + v + "\""; }
    void kv(const std::string& k, const std::vector<double>& v) {
        key(k);
        s += "[";
        for (size_t i = 0; i < v.size(); ++i) s += (i ? "," : "") + num(v[i]);
        s += "]";
    }
    void kv(const std::string& k, const std::vector<V3>& v) {
        std::vector<double> f;
        for (auto& x : v) { f.push_back(x.x); f.push_back(x.y); f.push_back(x.z); }
        kv(k, f);
    }
    void kv(const std::string& k, V3 v) { kv(k, std::vector<double>{v.x, v.y, v.z}); }
    void obj(const std::string& k) { key(k); open(); }
};

void dump_mesh(Json& j, const std::string& k, const Mesh& m) {
    j.obj(k);
    std::vector<double> V, n, c, a, h, t;
    for (int p = 0; p < m.P(); ++p) {
        for (int q = 0; q < 3; ++q) { V.push_back(m.V[p][q].x); V.push_back(m.V[p][q].y); V.push_back(m.V[p][q].z); }
        n.push_back(m.normal[p].x); n.push_back(m.normal[p].y); n.push_back(m.normal[p].z);
        c.push_back(m.centroid[p].x); c.push_back(m.centroid[p].y); c.push_back(m.centroid[p].z);
        a.push_back(m.area[p]); h.push_back(m.h[p]); t.push_back(m.tags[p]);
    }
    j.kv("V", V); j.kv("normal", n); j.kv("centroid", c); j.kv("area", a); j.kv("h", h); j.kv("tags", t);
    j.close();
}

void dump_solution(Json& j, const std::string& k, const SwimmerSolution& s) {
    j.obj(k);
    j.kv("U", s.U); j.kv("Om", s.Om); j.kv("f_sphere", s.f_sphere); j.kv("f_tube", s.f_tube);
    j.close();
}

// panel_integrals over a grid of target points around panel p: covers the self
// panel, all four rules, and off-plane points.
void dump_panels(Json& j, const std::string& k, const Mesh& M, const std::vector<int>& ps) {
    j.obj(k);
    std::vector<double> P, X, S, SL, DL;
    double sl[9], dl[9];
    for (int p : ps) {
        V3 c = M.centroid[p], n = M.normal[p];
        double h = M.h[p];
        // self
        panel_integrals(M, p, c, true, sl, dl);
        P.push_back(p); X.push_back(c.x); X.push_back(c.y); X.push_back(c.z); S.push_back(1);
        for (int q = 0; q < 9; ++q) { SL.push_back(sl[q]); DL.push_back(dl[q]); }
        for (double d : {0.3, 0.6, 0.9, 1.2, 2.0, 2.9, 3.1, 5.0, 12.0}) {
            for (double tilt : {0.0, 0.7}) {
                V3 t = unit(cross(n, M.V[p][0] - c));
                V3 dir = unit((1 - tilt) * n + tilt * t);
                V3 x0 = c + (d * h) * dir;
                panel_integrals(M, p, x0, false, sl, dl);
                P.push_back(p); X.push_back(x0.x); X.push_back(x0.y); X.push_back(x0.z); S.push_back(0);
                for (int q = 0; q < 9; ++q) { SL.push_back(sl[q]); DL.push_back(dl[q]); }
            }
        }
    }
    j.kv("p", P); j.kv("x0", X); j.kv("self", S); j.kv("SL", SL); j.kv("DL", DL);
    j.close();
}

std::vector<V3> probe_points(double R, double b, double zext, int n) {
    std::vector<V3> pts;
    for (int i = 0; i < n; ++i) {
        double s = (i + 0.5) / n;
        V3 p{-0.8 * R + 1.6 * R * s, 0.3 * R * std::sin(7.0 * s), -zext + 2 * zext * s};
        if (norm(p - V3{b, 0, 0}) < 1.2) p.z += 2.5;
        pts.push_back(p);
    }
    return pts;
}

// one kinematics instance, as main.cpp run_kinematics does for one (a/R, beta)
void kin_case(Json& j, const std::string& k, double lam, double beta, int nth, int lev, double LoR,
              bool towed, V3 e, bool field) {
    const double a = 1.0;
    std::unique_ptr<Tube> tube;
    if (lam > 0) tube = std::make_unique<Tube>(a / lam, LoR * a / lam, a, nth);
    double b = lam > 0 ? beta * (a / lam - a) : 0.0;
    SwimmerSolver s(tube.get(), icosphere(a, lev, {b, 0, 0}), {b, 0, 0});
    auto sl1 = s.slip(e, 1, 0), sl2 = s.slip(e, 0, 1);
    auto m = s.solve_free({sl1, sl2});
    j.obj(k);
    j.kv("a_over_R", lam); j.kv("beta", beta); j.kv("n_theta", nth); j.kv("sphere_level", lev);
    j.kv("L_over_R", LoR); j.kv("e", e); j.kv("Ns", s.Ns); j.kv("Nt", s.Nt);
    dump_solution(j, "B1", m[0]);
    dump_solution(j, "B2", m[1]);
    if (towed) {
        auto tw = s.solve_prescribed({0, 0, 1}, {});
        dump_solution(j, "towed_z", tw);
        j.kv("drag_K", -s.force(tw).z / (6 * PI));
        auto tw2 = s.solve_prescribed({0.1, -0.2, 0.3}, {0.05, 0.1, -0.15});
        dump_solution(j, "towed_gen", tw2);
        j.kv("force_gen", s.force(tw2));
    }
    if (field) {
        double R = lam > 0 ? a / lam : 4.0;
        auto pts = probe_points(R, b, lam > 0 ? 0.45 * LoR * R : 3.0, 24);
        j.kv("points", pts);
        j.kv("vel_B1", s.velocity(m[0], sl1, pts));
        j.kv("vel_B2", s.velocity(m[1], sl2, pts));
    }
    j.close();
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: ref_dump <case> [tmpdir]\n"); return 1; }
    std::string c = argv[1];
    Json j;
    j.open();
    j.kvs("case", c);
    const V3 ez{0, 0, 1};
    if (c == "mesh") {
        dump_mesh(j, "swimmer_tube", swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 12, 4));
        dump_mesh(j, "swimmer_tube_24", swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 24, 4));
        dump_mesh(j, "duct", tube_mesh(1.0, uniform_z(0, 4, 6), 8, 3));
        dump_mesh(j, "ico2", icosphere(1.0, 2, {0.7, -0.1, 0.2}));
        Mesh m = icosphere(1.0, 1);
        m.translate({0.25, 0.5, -0.75});
        dump_mesh(j, "ico1_translated", m);
    } else if (c == "panel") {
        Mesh t = swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 12, 4);
        Mesh s = icosphere(1.0, 2, {0.7, 0, 0});
        dump_panels(j, "tube", t, {0, 7, 100, t.P() - 1, t.P() - 30});
        dump_panels(j, "sphere", s, {0, 33, 200, s.P() - 1});
        std::vector<double> g, w;
        gauss_legendre01(10, g, w);
        j.kv("gl10_x", g); j.kv("gl10_w", w);
    } else if (c == "swim_small") {
        kin_case(j, "offaxis", 0.3, 0.4, 8, 1, 4.0, true, ez, true);
        kin_case(j, "tilted", 0.35, 0.5, 10, 1, 4.0, true, unit(V3{0.3, 0.2, 1.0}), true);
        kin_case(j, "onaxis_l2", 0.3, 0.0, 12, 2, 4.0, true, ez, true);
        kin_case(j, "unbounded", 0.0, 0.0, 0, 2, 4.0, true, ez, true);
    } else if (c == "duct_small" || c == "duct_c1") {
        bool big = c == "duct_c1";
        DuctFlow d(1.0, 4.0, big ? 24 : 8, big ? 24 : 8, big ? 6 : 3, 1.0);
        j.kv("P", d.mesh.P());
        std::vector<double> dps = {0.5, 1, 2, 4}, Q;
        for (double dP : dps) Q.push_back(d.solve(dP, 0.0).Q);
        j.kv("dP", dps); j.kv("Q", Q);
        auto s = d.solve(2.5, 0.5);
        j.kv("Q_25_05", s.Q);
        if (!big) { j.kv("u", s.u); j.kv("f", s.f); }
        auto s1 = d.solve(1.0, 0.0);
        std::vector<V3> pts;
        for (double ang : {0.0, PI / 5, PI / 2})
            for (int k = 0; k < 20; ++k) {
                double r = 0.95 * k / 19;
                pts.push_back({r * std::cos(ang), r * std::sin(ang), 2.0});
            }
        j.kv("points", pts);
        j.kv("vel", d.velocity(s1, pts));
        if (big) { j.kv("u1", s1.u); j.kv("f1", s1.f); }
    } else if (c == "c2") {
        kin_case(j, "c2", 0.3, 0.0, 24, 3, 4.0, true, ez, false);
    } else if (c == "c2_l2") {
        kin_case(j, "l2_axis", 0.3, 0.0, 24, 2, 4.0, true, ez, true);
        kin_case(j, "l2_off", 0.45, 0.5, 24, 2, 4.0, false, ez, false);
        kin_case(j, "l2_tilt", 0.2, 0.7, 24, 2, 4.0, false, unit(V3{-0.2, 0.4, 1.0}), false);
    } else if (c == "traj") {
        std::string dir = argc > 2 ? argv[2] : ".";
        TrajectoryParams P;
        P.alpha = -1.5; P.a_over_R = 0.3; P.beta0 = 0.5; P.pitch0_deg = 5; P.yaw0_deg = 10;
        P.dt = 0.5; P.t_max = 3.0; P.n_theta = 12; P.sphere_level = 1;
        std::string st = run_trajectory(P, dir + "/traj_small", false);
        j.kvs("status", st);
        std::ifstream in(dir + "/traj_small.csv");
        std::stringstream ss; ss << in.rdbuf();
        std::string body = ss.str(), esc;
        for (char ch : body) { if (ch == '\n') esc += "\\n"; else if (ch == '"') esc += "\\\""; else esc += ch; }
        j.kvs("csv", esc);
    } else {
        std::fprintf(stderr, "unknown case %s\n", c.c_str());
        return 1;
    }
    j.close();
    std::printf("%s\n", j.s.c_str());
    return 0;
}
