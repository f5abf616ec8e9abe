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

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "bem/utils/io.hpp"
#include "bem/utils/mesh.hpp"
#include "common.cuh"
#include "concurrent.cuh"
#include "solver.cuh"
#include "sphere_share.cuh"
#include "tube_cache.cuh"

using namespace sqbem;

namespace {

using State = std::array<double, 6>;  // x, y, z, ex, ey, ez

constexpr int TRAJ_GROUP = 48;

// Field grid of one swimmer (the y = 0 plane of the reference's field mode,
// main.cpp:109-131, extended to 3-D): x, y in [-0.97 R, 0.97 R], z in
// [-z_extent, z_extent] around the sphere (the tube frame is centred on the
// swimmer); points outside r = 0.97 R or within 1.03 a of the centre are masked.
struct GridSpec {
    int nx = 25, ny = 25, nz = 41;
    double z_extent = 7.0;
};

// out[i] = x[i] + alpha x[ld + i]: the B1 + alpha B2 combination of two solutions
__global__ void combine_modes_kernel(const double* __restrict__ x, long long ld, int n, double alpha,
                                     double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = x[i] + alpha * x[ld + i];
}

struct Modes {
    double U1[3], O1[3], U2[3], O2[3];
};

// U, Omega of the B1 = 1 and B2 = 1 modes for many swimmers around one tube.
class Evaluator {
public:
    // the tube comes from the cache of factored tubes (tube_cache.cu): a call
    // with the tube of an earlier call reuses its factor
    Evaluator(const sqbem_traj_params& P, int precision) : prec_(precision) {
        a_ = 1.0;
        R_ = a_ / P.a_over_R;
        tube_ = cached_tube(R_, P.L_over_R * R_, a_, P.n_theta, 4, 1.0, precision);
        sph0_ = bem::icosphere(a_, P.sphere_level);
        if (precision == SQBEM_MIXED) {  // every evaluation of this call shares the sphere-sphere blocks
            const auto V = mesh_vertices(sph0_);
            const double c0[3] = {0, 0, 0};
            share_ = build_sphere_blocks(make_panels(V.data(), sph0_.P()), c0, 1.0, st_);
        }
    }
    // work on st_ that reads the shared tube ends before the reference is dropped
    ~Evaluator() { cudaStreamSynchronize(st_); }
    double R() const { return R_; }
    double a() const { return a_; }
    cudaStream_t stream() const { return st_; }

    // One group of swimmers built and solved for the B1 and B2 slip modes.  With
    // keep, the full solutions stay available: mixed, x = [f_t; f_s; w] per mode
    // on the device (ld = nt + nc); FP64, f_t and f_s per mode on the host.
    struct Group {
        std::vector<std::unique_ptr<sqbem_swimmer>> sw;
        std::vector<std::vector<double>> slips;  // 2 x 3 Ns per swimmer
        std::vector<Modes> modes;
        std::vector<DevBuf<double>> dx;          // mixed
        std::vector<std::vector<double>> ft, fs; // FP64: 2 x 3 Nt, 2 x 3 Ns
        std::vector<std::array<double, 3>> centre, e;
    };

    void solve_group(const std::vector<State>& ys, size_t c0, size_t G, bool keep, Group& gr, cudaStream_t st) {
        // host time per phase on stderr when SQBEM_HOST_TIMING is set (profiling aid)
        static const bool timing = std::getenv("SQBEM_HOST_TIMING") != nullptr;
        auto tp = std::chrono::steady_clock::now();
        auto lap = [&](const char* what) {
            if (!timing) return;
            const auto now = std::chrono::steady_clock::now();
            std::fprintf(stderr, "ensemble group %zu (%zu swimmers) %-8s %.2f ms\n", c0, G, what,
                         std::chrono::duration<double, std::milli>(now - tp).count());
            tp = now;
        };
        gr.sw.resize(G);
        gr.slips.resize(G);
        gr.modes.resize(G);
        gr.centre.resize(G);
        gr.e.resize(G);
        for (size_t g = 0; g < G; ++g) {
            const State& y = ys[c0 + g];
            const double c[3] = {y[0], y[1], 0.0};
            gr.centre[g] = {c[0], c[1], c[2]};
            bem::Mesh S = sph0_;
            S.translate({c[0], c[1], c[2]});
            const auto V = mesh_vertices(S);
            gr.sw[g] = std::make_unique<sqbem_swimmer>();
            gr.sw[g]->st.borrow(st);
            const bem::V3 e = bem::unit(bem::V3{y[3], y[4], y[5]});
            const double ev[3] = {e.x, e.y, e.z};
            if (prec_ == SQBEM_MIXED) {
                gr.sw[g]->set_geometry(tube_.get(), S.P(), V.data(), c, 1.0, prec_);
            } else {
                gr.sw[g]->build(tube_.get(), S.P(), V.data(), c, 1.0, prec_);
            }
            gr.e[g] = {ev[0], ev[1], ev[2]};
            if (prec_ != SQBEM_MIXED || keep) {  // host copies: the FP64 API and the field's surface velocity
                gr.slips[g] = squirmer_slip_host(gr.sw[g]->host_panels, c, ev, 1, 0);
                const auto u2 = squirmer_slip_host(gr.sw[g]->host_panels, c, ev, 0, 1);
                gr.slips[g].insert(gr.slips[g].end(), u2.begin(), u2.end());
            }
        }
        lap("geometry");
        if (prec_ == SQBEM_MIXED) {
            std::vector<sqbem_swimmer*> sp;
            for (auto& s : gr.sw) sp.push_back(s.get());
            DevBuf<int> flags(2, st);
            flags.zero();
            MixedCtx cx{st, flags.get(), flags.get() + 1};
            mixed_build_swimmers(sp, cx, share_);
            lap("build");
            // the slip modes on the device (slip_modes_group), solved in place
            std::vector<DevBuf<double>> din(G);
            gr.dx.clear();
            gr.dx.resize(G);
            std::vector<const double*> ip;
            std::vector<double*> xp;
            std::vector<SlipJob> sj;
            for (size_t g = 0; g < G; ++g) {
                din[g].alloc((size_t)6 * sp[g]->Ns, st);
                SlipJob j;
                j.rec = sp[g]->panels.rec.get();
                j.Ns = sp[g]->Ns;
                for (int q = 0; q < 3; ++q) {
                    j.xc[q] = gr.centre[g][q];
                    j.e[q] = gr.e[g][q];
                }
                j.out = din[g].get();
                sj.push_back(j);
                gr.dx[g].alloc((size_t)(sp[g]->mx.nt + sp[g]->mx.nc) * 2, st);
                ip.push_back(din[g].get());
                xp.push_back(gr.dx[g].get());
            }
            slip_modes_group(sj, st);
            int it = 0;
            double res = 0;
            mixed_solve(sp, false, ip, 2, xp, cx, &it, &res);
            std::vector<double> w(12 * G);
            for (size_t g = 0; g < G; ++g) {
                const MixedSwimmer& M = sp[g]->mx;
                const size_t ld = (size_t)M.nt + M.nc;
                for (int k = 0; k < 2; ++k)
                    CUDA_CHECK(cudaMemcpyAsync(w.data() + 12 * g + 6 * k, gr.dx[g].get() + k * ld + M.nt + M.ns,
                                               6 * sizeof(double), cudaMemcpyDeviceToHost, st));
                count_d2h(12 * sizeof(double));
            }
            CUDA_CHECK(cudaStreamSynchronize(st));
            lap("solve");
            for (size_t g = 0; g < G; ++g) {
                const double* wg = w.data() + 12 * g;
                Modes& m = gr.modes[g];
                for (int q = 0; q < 3; ++q) {
                    m.U1[q] = wg[q]; m.O1[q] = wg[3 + q]; m.U2[q] = wg[6 + q]; m.O2[q] = wg[9 + q];
                }
            }
            if (!keep) gr.dx.clear();
        } else {
            if (keep) {
                gr.ft.resize(G);
                gr.fs.resize(G);
            }
            for (size_t g = 0; g < G; ++g) {
                double U[6], Om[6];
                sqbem_swimmer& s = *gr.sw[g];
                if (keep) {
                    gr.ft[g].resize((size_t)6 * s.Nt);
                    gr.fs[g].resize((size_t)6 * s.Ns);
                }
                s.solve_free(2, gr.slips[g].data(), U, Om, keep ? gr.fs[g].data() : nullptr,
                             keep ? gr.ft[g].data() : nullptr);
                Modes& m = gr.modes[g];
                for (int q = 0; q < 3; ++q) {
                    m.U1[q] = U[q]; m.O1[q] = Om[q]; m.U2[q] = U[3 + q]; m.O2[q] = Om[3 + q];
                }
            }
        }
        evals_.fetch_add((long long)G);
    }

    // per-group device bytes (swimmer blocks B, A_uBt, D, Y, E, A_uBs, G_s^{-1}), with a margin
    double group_bytes(size_t G) const {
        const double t = 3.0 * tube_->Nt, sph = 3.0 * sph0_.P();
        return 1.25 * G * 4.0 * (6.0 * t * sph + 5.0 * sph * sph + 2.0 * t);
    }

    // The groups of an evaluation are independent: they run concurrently
    // (concurrent.cuh), each on its own stream, sharing the tube's factors.
    std::vector<Modes> modes(const std::vector<State>& ys) {
        std::vector<Modes> out(ys.size());
        const size_t ntask = (ys.size() + TRAJ_GROUP - 1) / TRAJ_GROUP;
        std::vector<double> bytes;
        for (size_t k = 0; k < ntask; ++k) bytes.push_back(group_bytes(std::min<size_t>(TRAJ_GROUP, ys.size() - k * TRAJ_GROUP)));
        run_concurrent(ntask, bytes, st_, [&](size_t k, cudaStream_t st) {
            const size_t c0 = k * TRAJ_GROUP, G = std::min<size_t>(TRAJ_GROUP, ys.size() - c0);
            Group gr;
            solve_group(ys, c0, G, false, gr, st);
            for (size_t g = 0; g < G; ++g) out[c0 + g] = gr.modes[g];
        });
        return out;
    }

    // Lab-frame velocity (swimmer.hpp:163-173, field.hpp:18-34) of swimmer k
    // (B1 = 1, B2 = alpha[k]) at the unmasked points of its grid.
    void fields(const std::vector<State>& ys, const double* alpha, const GridSpec& gs, double* u_out);
    long long evals() const { return evals_.load(); }

private:
    int prec_;
    double a_ = 1, R_ = 1;
    std::shared_ptr<const sqbem_tube> tube_;
    Stream st_;  // this evaluation's own stream (the cached tube's is not used)
    std::shared_ptr<const SphereBlocks> share_;  // mixed: the sphere-sphere blocks of this call
    bem::Mesh sph0_;
    std::atomic<long long> evals_{0};
};

void Evaluator::fields(const std::vector<State>& ys, const double* alpha, const GridSpec& gs, double* u_out) {
    const int Nt = tube_->Nt;
    const size_t npg = (size_t)gs.nx * gs.ny * gs.nz;
    const double lim = 0.97 * R_;
    const size_t ntask = (ys.size() + TRAJ_GROUP - 1) / TRAJ_GROUP;
    std::vector<double> bytes;
    for (size_t k = 0; k < ntask; ++k) bytes.push_back(group_bytes(std::min<size_t>(TRAJ_GROUP, ys.size() - k * TRAJ_GROUP)));
    run_concurrent(ntask, bytes, st_, [&](size_t task, cudaStream_t st) {
        const size_t c0 = task * TRAJ_GROUP, G = std::min<size_t>(TRAJ_GROUP, ys.size() - c0);
        Group gr;
        solve_group(ys, c0, G, true, gr, st);
        for (size_t g = 0; g < G; ++g) {
            const size_t k = c0 + g;
            sqbem_swimmer& s = *gr.sw[g];
            const int Ns = s.Ns, P = Nt + Ns;
            const double al = alpha[k];
            const std::array<double, 3>& c = gr.centre[g];
            double* uk = u_out + k * npg * 3;
            std::vector<double> pts;
            std::vector<size_t> idx;
            for (int i = 0; i < gs.nx; ++i)
                for (int j = 0; j < gs.ny; ++j)
                    for (int l = 0; l < gs.nz; ++l) {
                        const size_t q = ((size_t)i * gs.ny + j) * gs.nz + l;
                        const double x = -lim + 2 * lim * i / (gs.nx - 1), y = -lim + 2 * lim * j / (gs.ny - 1);
                        const double z = -gs.z_extent + 2 * gs.z_extent * l / (gs.nz - 1);
                        const double dx = x - c[0], dy = y - c[1], dz = z - c[2];
                        uk[3 * q] = uk[3 * q + 1] = uk[3 * q + 2] = NAN;
                        if (x * x + y * y > lim * lim || std::sqrt(dx * dx + dy * dy + dz * dz) < 1.03 * a_) continue;
                        pts.insert(pts.end(), {x, y, z});
                        idx.push_back(q);
                    }
            if (idx.empty()) continue;
            const int npts = (int)idx.size();
            DevBuf<PanelRec> mp((size_t)P, st);
            CUDA_CHECK(cudaMemcpyAsync(mp.get(), tube_->panels.rec.get(), sizeof(PanelRec) * Nt,
                                       cudaMemcpyDeviceToDevice, st));
            CUDA_CHECK(cudaMemcpyAsync(mp.get() + Nt, s.panels.rec.get(), sizeof(PanelRec) * Ns,
                                       cudaMemcpyDeviceToDevice, st));
            // tractions f = f[B1] + alpha f[B2], tube panels first (the order of x)
            DevBuf<double> df(3 * (size_t)P, st);
            if (prec_ == SQBEM_MIXED) {
                const long long ld = (long long)s.mx.nt + s.mx.nc;
                LAUNCH(combine_modes_kernel, ceil_div(3LL * P, 256), 256, 0, st, gr.dx[g].get(), ld, 3 * P, al,
                       df.get());
            } else {
                std::vector<double> hf(3 * (size_t)P);
                for (int i = 0; i < 3 * Nt; ++i) hf[i] = gr.ft[g][i] + al * gr.ft[g][3 * (size_t)Nt + i];
                for (int i = 0; i < 3 * Ns; ++i) hf[3 * (size_t)Nt + i] = gr.fs[g][i] + al * gr.fs[g][3 * (size_t)Ns + i];
                df.upload(hf.data(), hf.size());
            }
            // surface velocity: 0 on the tube, U + Omega x r + slip on the sphere
            const Modes& m = gr.modes[g];
            double U[3], W[3];
            for (int q = 0; q < 3; ++q) {
                U[q] = m.U1[q] + al * m.U2[q];
                W[q] = m.O1[q] + al * m.O2[q];
            }
            std::vector<double> hu(3 * (size_t)P, 0.0);
            const std::vector<double>& sl = gr.slips[g];
            for (int p = 0; p < Ns; ++p) {
                const double rx = s.host_panels[p].c[0] - c[0], ry = s.host_panels[p].c[1] - c[1],
                             rz = s.host_panels[p].c[2] - c[2];
                double* o = hu.data() + 3 * ((size_t)Nt + p);
                const double* s1 = sl.data() + 3 * p;
                const double* s2 = sl.data() + 3 * ((size_t)Ns + p);
                o[0] = U[0] + (W[1] * rz - W[2] * ry) + (s1[0] + al * s2[0]);
                o[1] = U[1] + (W[2] * rx - W[0] * rz) + (s1[1] + al * s2[1]);
                o[2] = U[2] + (W[0] * ry - W[1] * rx) + (s1[2] + al * s2[2]);
            }
            DevBuf<double> du(hu.size(), st), dpts(pts.size(), st), dout(pts.size(), st);
            DevBuf<int> ovf(1, st);
            ovf.zero();
            du.upload(hu.data(), hu.size());
            dpts.upload(pts.data(), pts.size());
            FieldJob job;
            job.pts = dpts.get();
            job.npts = npts;
            job.panels = mp.get();
            job.P = P;
            job.u = du.get();
            job.f = df.get();
            job.sscale = 1.0 / EIGHT_PI;  // mu = 1
            job.dscale = -1.0 / EIGHT_PI;
            job.out = dout.get();
            job.overflow = ovf.get();
            job.mixed = prec_ == SQBEM_MIXED;
            field_eval(job, st);
            std::vector<double> ho(pts.size());
            int h_ovf = 0;
            dout.download(ho.data(), ho.size());
            ovf.download(&h_ovf, 1);
            CUDA_CHECK(cudaStreamSynchronize(st));
            if (h_ovf) fail(SQBEM_ERR_ARG, "ensemble_field: a grid point has more than 256 near panels");
            for (int q = 0; q < npts; ++q)
                for (int d = 0; d < 3; ++d) uk[3 * idx[q] + d] = ho[3 * (size_t)q + d];
        }
    });
}

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

extern "C" int sqbem_ensemble_field(int n, const double* states, const double* alpha, const sqbem_traj_params* pp,
                                    int nx, int ny, int nz, double z_extent, int precision, double* u,
                                    double* device_seconds) {
    return guarded([&] {
        if (n < 0 || !pp || nx < 2 || ny < 2 || nz < 2 || !(z_extent > 0) || (n > 0 && (!states || !alpha || !u)) ||
            (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "ensemble_field: bad arguments");
        const sqbem_traj_params P = *pp;
        check_params(P);
        if (device_seconds) *device_seconds = 0;
        if (n == 0) return;
        require_device();
        Evaluator ev(P, precision);
        std::vector<State> ys(n);
        for (int k = 0; k < n; ++k) {
            for (int i = 0; i < 6; ++i) ys[k][i] = states[6 * k + i];
            normalise_e(ys[k]);
        }
        GridSpec gs;
        gs.nx = nx;
        gs.ny = ny;
        gs.nz = nz;
        gs.z_extent = z_extent;
        EventTimer clk;
        clk.start(ev.stream());
        ev.fields(ys, alpha, gs, u);
        clk.stop(ev.stream());
        const double secs = clk.seconds();
        if (device_seconds) *device_seconds = secs;
    });
}
