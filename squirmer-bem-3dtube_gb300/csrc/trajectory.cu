// trajectory.cu -- swimmer trajectories in a tube (src/trajectory.hpp:42-151).
//
//   dX/dt = U(X, e),   de/dt = Omega(X, e) x e,   U = U[B1 = 1] + alpha U[B2 = 1]
//
// The tube moves with the swimmer (always centred at z = 0), so it is built and
// factored once; each evaluation translates the sphere to (x, y, 0), rebuilds
// only the swimmer couplings and solves the two squirming modes.  In mixed
// precision every evaluation of a time-stepping stage runs for all active
// swimmers of an ensemble at once (grouped assembly, Schur GEMMs and
// refinement), with the tube's inverse shared by all of them.
#include <cuda_runtime.h>

#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "bem/utils/io.hpp"
#include "bem/utils/mesh.hpp"
#include "common.cuh"
#include "solver.cuh"

using namespace sqbem;

namespace {

using State = std::array<double, 6>;  // x, y, z, ex, ey, ez

constexpr int TRAJ_GROUP = 48;

struct Modes {
    double U1[3], O1[3], U2[3], O2[3];
};

// U, Omega of the B1 = 1 and B2 = 1 modes for many swimmers around one tube.
class Evaluator {
public:
    Evaluator(const sqbem_traj_params& P, int precision) : prec_(precision) {
        a_ = 1.0;
        R_ = a_ / P.a_over_R;
        tube_ = std::make_unique<sqbem_tube>();
        tube_->build(R_, P.L_over_R * R_, a_, P.n_theta, 4, 1.0, precision);
        sph0_ = bem::icosphere(a_, P.sphere_level);
    }
    double R() const { return R_; }
    double a() const { return a_; }
    cudaStream_t stream() const { return tube_->st; }

    std::vector<Modes> modes(const std::vector<State>& ys) {
        std::vector<Modes> out(ys.size());
        for (size_t c0 = 0; c0 < ys.size(); c0 += TRAJ_GROUP) {
            const size_t G = std::min<size_t>(TRAJ_GROUP, ys.size() - c0);
            std::vector<std::unique_ptr<sqbem_swimmer>> sw(G);
            std::vector<std::vector<double>> slips(G);
            for (size_t g = 0; g < G; ++g) {
                const State& y = ys[c0 + g];
                const double c[3] = {y[0], y[1], 0.0};
                bem::Mesh S = sph0_;
                S.translate({c[0], c[1], c[2]});
                const auto V = mesh_vertices(S);
                sw[g] = std::make_unique<sqbem_swimmer>();
                sw[g]->st.borrow(tube_->st);
                const bem::V3 e = bem::unit(bem::V3{y[3], y[4], y[5]});
                const double ev[3] = {e.x, e.y, e.z};
                if (prec_ == SQBEM_MIXED) {
                    sw[g]->set_geometry(tube_.get(), S.P(), V.data(), c, 1.0, prec_);
                } else {
                    sw[g]->build(tube_.get(), S.P(), V.data(), c, 1.0, prec_);
                }
                slips[g] = squirmer_slip_host(sw[g]->host_panels, c, ev, 1, 0);
                const auto u2 = squirmer_slip_host(sw[g]->host_panels, c, ev, 0, 1);
                slips[g].insert(slips[g].end(), u2.begin(), u2.end());
            }
            if (prec_ == SQBEM_MIXED) {
                std::vector<sqbem_swimmer*> sp;
                for (auto& s : sw) sp.push_back(s.get());
                DevBuf<int> flags(2, tube_->st);
                flags.zero();
                MixedCtx cx{tube_->st, flags.get(), flags.get() + 1};
                mixed_build_swimmers(sp, cx);
                std::vector<DevBuf<double>> din(G), dx(G);
                std::vector<const double*> ip;
                std::vector<double*> xp;
                for (size_t g = 0; g < G; ++g) {
                    din[g].alloc(slips[g].size(), tube_->st);
                    din[g].upload(slips[g].data(), slips[g].size());
                    dx[g].alloc((size_t)(sp[g]->mx.nt + sp[g]->mx.nc) * 2, tube_->st);
                    ip.push_back(din[g].get());
                    xp.push_back(dx[g].get());
                }
                int it = 0;
                double res = 0;
                mixed_solve(sp, false, ip, 2, xp, cx, &it, &res);
                for (size_t g = 0; g < G; ++g) {
                    const MixedSwimmer& M = sp[g]->mx;
                    const size_t ld = (size_t)M.nt + M.nc;
                    std::vector<double> w(12);
                    for (int k = 0; k < 2; ++k)
                        CUDA_CHECK(cudaMemcpyAsync(w.data() + 6 * k, dx[g].get() + k * ld + M.nt + M.ns, 6 * sizeof(double),
                                                   cudaMemcpyDeviceToHost, tube_->st));
                    count_d2h(12 * sizeof(double));
                    CUDA_CHECK(cudaStreamSynchronize(tube_->st));
                    Modes& m = out[c0 + g];
                    for (int q = 0; q < 3; ++q) {
                        m.U1[q] = w[q]; m.O1[q] = w[3 + q]; m.U2[q] = w[6 + q]; m.O2[q] = w[9 + q];
                    }
                }
            } else {
                for (size_t g = 0; g < G; ++g) {
                    double U[6], Om[6];
                    sw[g]->solve_free(2, slips[g].data(), U, Om, nullptr, nullptr);
                    Modes& m = out[c0 + g];
                    for (int q = 0; q < 3; ++q) {
                        m.U1[q] = U[q]; m.O1[q] = Om[q]; m.U2[q] = U[3 + q]; m.O2[q] = Om[3 + q];
                    }
                }
            }
            evals_ += G;
        }
        return out;
    }
    long long evals() const { return evals_; }

private:
    int prec_;
    double a_ = 1, R_ = 1;
    std::unique_ptr<sqbem_tube> tube_;
    bem::Mesh sph0_;
    long long evals_ = 0;
};

// state derivative (trajectory.hpp:52-65): U = U1 + alpha U2, de/dt = Omega x e
State derivative(const State& y, const Modes& m, double alpha, double* U, double* Om) {
    const bem::V3 e = bem::unit(bem::V3{y[3], y[4], y[5]});
    const bem::V3 u{m.U1[0] + alpha * m.U2[0], m.U1[1] + alpha * m.U2[1], m.U1[2] + alpha * m.U2[2]};
    const bem::V3 w{m.O1[0] + alpha * m.O2[0], m.O1[1] + alpha * m.O2[1], m.O1[2] + alpha * m.O2[2]};
    const bem::V3 de = bem::cross(w, e);
    if (U) { U[0] = u.x; U[1] = u.y; U[2] = u.z; }
    if (Om) { Om[0] = w.x; Om[1] = w.y; Om[2] = w.z; }
    return {u.x, u.y, u.z, de.x, de.y, de.z};
}

State axpy(const State& s, double h, const State& d) {
    State o;
    for (int i = 0; i < 6; ++i) o[i] = s[i] + h * d[i];
    return o;
}

void normalise_e(State& y) {
    const double n = std::sqrt(y[3] * y[3] + y[4] * y[4] + y[5] * y[5]);
    for (int i = 3; i < 6; ++i) y[i] /= n;
}

void check_params(const sqbem_traj_params& P) {
    if (!(P.a_over_R > 0 && P.a_over_R < 1) || !(P.dt > 0) || !(P.L_over_R > 0) || P.n_theta < 3 ||
        P.sphere_level < 0 || P.sphere_level > 5 || !(P.beta0 >= 0))
        fail(SQBEM_ERR_ARG, "trajectory: bad parameters");
}

}  // namespace

extern "C" int sqbem_trajectory_defaults(sqbem_traj_params* p) {
    return guarded([&] {
        if (!p) fail(SQBEM_ERR_ARG, "trajectory_defaults: null");
        *p = sqbem_traj_params{};
        p->alpha = 0;
        p->a_over_R = 0.3;
        p->beta0 = 0.5;
        p->pitch0_deg = 0;
        p->yaw0_deg = 0;
        p->dt = 0.5;
        p->t_max = 100;
        p->L_over_R = 4;
        p->n_theta = 30;
        p->sphere_level = 2;
        p->beta_stop = 0.95;
        p->budget_s = 0;
    });
}

extern "C" int sqbem_run_trajectory(const sqbem_traj_params* pp, const char* out_prefix, int verbose, int precision,
                                    char* status_out, int status_cap) {
    return guarded([&] {
        if (!pp || !out_prefix || (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "run_trajectory: bad arguments");
        const sqbem_traj_params P = *pp;
        check_params(P);
        require_device();
        bem::Timer clock;
        Evaluator ev(P, precision);
        const double R = ev.R(), a = ev.a();
        auto beta_of = [&](const State& y) { return std::hypot(y[0], y[1]) / (R - a); };
        struct Eval {
            State d;
            double U[3], Om[3];
        };
        auto evaluate = [&](const State& y) {
            const Modes m = ev.modes({y})[0];
            Eval r;
            r.d = derivative(y, m, P.alpha, r.U, r.Om);
            return r;
        };
        // ---- initialise or restart (trajectory.hpp:69-104)
        const std::string ck = std::string(out_prefix) + ".ckpt", csvp = std::string(out_prefix) + ".csv";
        State y{};
        double t = 0;
        int step = 0;
        std::vector<State> hist;  // up to three previous derivatives, oldest first
        std::ifstream in(ck);
        const bool restart = (bool)in;
        if (restart) {
            size_t nh = 0;
            in >> t >> step >> nh;
            for (double& v : y) in >> v;
            hist.resize(nh);
            for (State& h : hist)
                for (double& v : h) in >> v;
            if (verbose) std::printf("restart at t = %.3f (step %d)\n", t, step);
        } else {
            const double b = P.beta0 * (R - a), xi = P.pitch0_deg * bem::PI / 180, chi = P.yaw0_deg * bem::PI / 180;
            y = {-b, 0, 0, std::cos(chi) * std::sin(xi), std::sin(chi), std::cos(chi) * std::cos(xi)};
        }
        char info[256];
        std::snprintf(info, sizeof info,
                      "alpha=%g a_over_R=%g beta0=%g pitch0_deg=%g yaw0_deg=%g dt=%g n_theta=%d sphere_level=%d",
                      P.alpha, P.a_over_R, P.beta0, P.pitch0_deg, P.yaw0_deg, P.dt, P.n_theta, P.sphere_level);
        bem::Csv out(csvp, "t,x,y,z,ex,ey,ez,Ux,Uy,Uz,Omx,Omy,Omz,beta", {info}, restart);
        auto save = [&]() {
            std::ofstream o(ck);
            o.precision(17);
            o << t << " " << step << " " << hist.size() << "\n";
            for (double v : y) o << v << " ";
            o << "\n";
            for (const State& h : hist) {
                for (double v : h) o << v << " ";
                o << "\n";
            }
        };
        // ---- time loop (trajectory.hpp:108-144)
        std::string status = "finished";
        while (t < P.t_max - 1e-9) {
            if (beta_of(y) > P.beta_stop) {
                status = "wall contact";
                break;
            }
            const double el = clock.seconds();
            const long long ne = ev.evals();
            if (P.budget_s > 0 && ne > 0 && el + 1.3 * el / ne * (hist.size() < 3 ? 4 : 1) > P.budget_s) {
                status = "paused";
                break;
            }
            const Eval f = evaluate(y);
            out.row({t, y[0], y[1], y[2], y[3], y[4], y[5], f.U[0], f.U[1], f.U[2], f.Om[0], f.Om[1], f.Om[2],
                     beta_of(y)});
            if (hist.size() < 3) {  // RK4 start-up
                const Eval k2 = evaluate(axpy(y, P.dt / 2, f.d));
                const Eval k3 = evaluate(axpy(y, P.dt / 2, k2.d));
                const Eval k4 = evaluate(axpy(y, P.dt, k3.d));
                for (int i = 0; i < 6; ++i) y[i] += P.dt / 6 * (f.d[i] + 2 * k2.d[i] + 2 * k3.d[i] + k4.d[i]);
            } else {  // Adams-Bashforth 4
                const State &f1 = hist[2], &f2 = hist[1], &f3 = hist[0];
                for (int i = 0; i < 6; ++i) y[i] += P.dt / 24 * (55 * f.d[i] - 59 * f1[i] + 37 * f2[i] - 9 * f3[i]);
            }
            normalise_e(y);
            hist.push_back(f.d);
            if (hist.size() > 3) hist.erase(hist.begin());
            t += P.dt;
            ++step;
            save();
        }
        if (verbose)
            std::printf("%s: t = %.2f, beta = %.3f, z = %.2f  (%lld solves, %.1f s, %.2f s/solve)\n", status.c_str(), t,
                        beta_of(y), y[2], ev.evals(), clock.seconds(),
                        ev.evals() ? clock.seconds() / ev.evals() : 0.0);
        if (status != "paused") std::remove(ck.c_str());
        if (status_out && status_cap > 0) {
            std::strncpy(status_out, status.c_str(), status_cap - 1);
            status_out[status_cap - 1] = 0;
        }
    });
}

extern "C" int sqbem_trajectory_ensemble(int n, const double* y0, const double* alpha, const sqbem_traj_params* pp,
                                         int steps, int scheme, int precision, double* states, double* U, double* Om,
                                         int* status, double* device_seconds) {
    return guarded([&] {
        if (n < 0 || !pp || steps < 0 || (n > 0 && (!y0 || !alpha || !states || !status)) ||
            (scheme != 0 && scheme != 1) || (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "trajectory_ensemble: bad arguments");
        const sqbem_traj_params P = *pp;
        check_params(P);
        if (n == 0) return;
        require_device();
        Evaluator ev(P, precision);
        const double R = ev.R(), a = ev.a();
        EventTimer clk;
        clk.start(ev.stream());
        std::vector<State> y(n);
        std::vector<std::vector<State>> hist(n);
        for (int k = 0; k < n; ++k) {
            for (int i = 0; i < 6; ++i) y[k][i] = y0[6 * k + i];
            status[k] = 0;
            std::memcpy(states + (size_t)k * (steps + 1) * 6, y[k].data(), 6 * sizeof(double));
        }
        auto eval_all = [&](const std::vector<int>& ids, const std::vector<State>& ys, std::vector<State>& d,
                            std::vector<std::array<double, 6>>* uo) {
            const std::vector<Modes> m = ev.modes(ys);
            d.resize(ids.size());
            if (uo) uo->resize(ids.size());
            for (size_t j = 0; j < ids.size(); ++j) {
                double u[3], w[3];
                d[j] = derivative(ys[j], m[j], alpha[ids[j]], u, w);
                if (uo) (*uo)[j] = {u[0], u[1], u[2], w[0], w[1], w[2]};
            }
        };
        for (int s = 0; s < steps; ++s) {
            std::vector<int> ids;
            for (int k = 0; k < n; ++k) {
                if (status[k] == 0 && std::hypot(y[k][0], y[k][1]) / (R - a) > P.beta_stop) status[k] = 1;
                if (status[k] == 0) ids.push_back(k);
            }
            std::vector<State> ys, f, k2, k3, k4;
            for (int k : ids) ys.push_back(y[k]);
            std::vector<std::array<double, 6>> uo;
            if (!ids.empty()) eval_all(ids, ys, f, &uo);
            // members needing RK4 this step (scheme 1, or the first three steps)
            std::vector<size_t> rk;
            for (size_t j = 0; j < ids.size(); ++j)
                if (scheme == 1 || hist[ids[j]].size() < 3) rk.push_back(j);
            if (!rk.empty()) {
                std::vector<int> rid;
                std::vector<State> y2, y3, y4;
                for (size_t j : rk) {
                    rid.push_back(ids[j]);
                    y2.push_back(axpy(ys[j], P.dt / 2, f[j]));
                }
                eval_all(rid, y2, k2, nullptr);
                for (size_t q = 0; q < rk.size(); ++q) y3.push_back(axpy(ys[rk[q]], P.dt / 2, k2[q]));
                eval_all(rid, y3, k3, nullptr);
                for (size_t q = 0; q < rk.size(); ++q) y4.push_back(axpy(ys[rk[q]], P.dt, k3[q]));
                eval_all(rid, y4, k4, nullptr);
                for (size_t q = 0; q < rk.size(); ++q) {
                    const size_t j = rk[q];
                    State& yy = y[ids[j]];
                    for (int i = 0; i < 6; ++i)
                        yy[i] += P.dt / 6 * (f[j][i] + 2 * k2[q][i] + 2 * k3[q][i] + k4[q][i]);
                }
            }
            for (size_t j = 0; j < ids.size(); ++j) {
                const int k = ids[j];
                if (!(scheme == 1 || hist[k].size() < 3)) {
                    const State &f1 = hist[k][2], &f2 = hist[k][1], &f3 = hist[k][0];
                    for (int i = 0; i < 6; ++i)
                        y[k][i] += P.dt / 24 * (55 * f[j][i] - 59 * f1[i] + 37 * f2[i] - 9 * f3[i]);
                }
                normalise_e(y[k]);
                hist[k].push_back(f[j]);
                if (hist[k].size() > 3) hist[k].erase(hist[k].begin());
            }
            for (int k = 0; k < n; ++k) {
                std::memcpy(states + ((size_t)k * (steps + 1) + s + 1) * 6, y[k].data(), 6 * sizeof(double));
                for (int i = 0; i < 3; ++i) {
                    if (U) U[((size_t)k * steps + s) * 3 + i] = NAN;
                    if (Om) Om[((size_t)k * steps + s) * 3 + i] = NAN;
                }
            }
            for (size_t j = 0; j < ids.size(); ++j)
                for (int i = 0; i < 3; ++i) {
                    if (U) U[((size_t)ids[j] * steps + s) * 3 + i] = uo[j][i];
                    if (Om) Om[((size_t)ids[j] * steps + s) * 3 + i] = uo[j][3 + i];
                }
        }
        clk.stop(ev.stream());
        const double secs = clk.seconds();
        if (device_seconds) *device_seconds = secs;
    });
}
