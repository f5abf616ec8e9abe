// batch.cu -- batched kinematics (sqbem_kinematics_batch): many independent
// (a/R, beta, level, e) instances in one call, all on one stream.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <exception>
#include <map>
#include <mutex>
#include <thread>
#include <memory>
#include <tuple>
#include <vector>

#include "bem/utils/mesh.hpp"
#include "common.cuh"
#include "concurrent.cuh"
#include "solver.cuh"
#include "sphere_share.cuh"

using namespace sqbem;

// u_s = (B1 + B2 cos th)(cos th rhat - e), cos th = rhat . e (kernels.hpp:107-111)
std::vector<double> squirmer_slip_host(const std::vector<PanelRec>& S, const double* xc, const double* e, double B1,
                                       double B2) {
    std::vector<double> u(3 * S.size());
    const bem::V3 c{xc[0], xc[1], xc[2]}, ev{e[0], e[1], e[2]};
    for (size_t p = 0; p < S.size(); ++p) {
        const bem::V3 rh = bem::unit(bem::V3{S[p].c[0], S[p].c[1], S[p].c[2]} - c);
        const double ct = bem::dot(rh, ev);
        const bem::V3 v = (B1 + B2 * ct) * (ct * rh - ev);
        u[3 * p] = v.x;
        u[3 * p + 1] = v.y;
        u[3 * p + 2] = v.z;
    }
    return u;
}

namespace sqbem {
namespace {
constexpr int SLIP_MAXJ = 64;
struct SlipArgs {
    int n;
    SlipJob j[SLIP_MAXJ];
};

// One panel per thread; the operations of squirmer_slip_host in its order,
// rounded the same way (no contraction), so the two agree bit for bit.
__global__ void slip_modes_kernel(const __grid_constant__ SlipArgs args) {
    const SlipJob& J = args.j[blockIdx.y];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= J.Ns) return;
    const PanelRec& P = J.rec[p];
    const double rx = __dsub_rn(P.c[0], J.xc[0]), ry = __dsub_rn(P.c[1], J.xc[1]), rz = __dsub_rn(P.c[2], J.xc[2]);
    const double nn = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
    const double inv = __ddiv_rn(1.0, __dsqrt_rn(nn));
    const double hx = __dmul_rn(inv, rx), hy = __dmul_rn(inv, ry), hz = __dmul_rn(inv, rz);
    const double ct = __dadd_rn(__dadd_rn(__dmul_rn(hx, J.e[0]), __dmul_rn(hy, J.e[1])), __dmul_rn(hz, J.e[2]));
    const double vx = __dsub_rn(__dmul_rn(ct, hx), J.e[0]);
    const double vy = __dsub_rn(__dmul_rn(ct, hy), J.e[1]);
    const double vz = __dsub_rn(__dmul_rn(ct, hz), J.e[2]);
    const double s1 = __dadd_rn(1.0, __dmul_rn(0.0, ct));  // B1 = 1, B2 = 0
    const double s2 = __dadd_rn(0.0, __dmul_rn(1.0, ct));  // B1 = 0, B2 = 1
    double* o1 = J.out + 3 * (long long)p;
    double* o2 = J.out + 3 * ((long long)J.Ns + p);
    o1[0] = __dmul_rn(s1, vx); o1[1] = __dmul_rn(s1, vy); o1[2] = __dmul_rn(s1, vz);
    o2[0] = __dmul_rn(s2, vx); o2[1] = __dmul_rn(s2, vy); o2[2] = __dmul_rn(s2, vz);
}
}  // namespace

void slip_modes_group(const std::vector<SlipJob>& jobs, cudaStream_t st) {
    for (size_t i0 = 0; i0 < jobs.size(); i0 += SLIP_MAXJ) {
        SlipArgs a;
        a.n = (int)std::min<size_t>(SLIP_MAXJ, jobs.size() - i0);
        int mx = 0;
        for (int k = 0; k < a.n; ++k) {
            a.j[k] = jobs[i0 + k];
            mx = std::max(mx, a.j[k].Ns);
        }
        if (mx > 0) LAUNCH(slip_modes_kernel, dim3((unsigned)ceil_div(mx, 128), (unsigned)a.n), 128, 0, st, a);
    }
}
}  // namespace sqbem

namespace {

struct Prepared {
    bem::Mesh tube, sphere;
    std::vector<double> sphereV;
    double R = 0, L = 0, b = 0;
    bool bounded = true;
};

Prepared prepare(const sqbem_instance& in) {
    Prepared p;
    const double a = 1.0;
    p.bounded = in.a_over_R > 0;
    p.R = p.bounded ? a / in.a_over_R : 0.0;
    p.L = in.L_over_R * p.R;
    p.b = p.bounded ? in.beta * (p.R - a) : 0.0;
    if (p.bounded) p.tube = bem::swimmer_tube_mesh(p.R, p.L, a, in.n_theta, in.n_r);
    p.sphere = bem::icosphere(a, in.sphere_level, {p.b, 0, 0});
    p.sphereV = mesh_vertices(p.sphere);
    return p;
}

// prepare() of every instance, spread over up to 8 host threads (mesh
// generation is host work on the end-to-end path).
std::vector<Prepared> prepare_all(int n, const sqbem_instance* inst) {
    std::vector<Prepared> prep((size_t)n);
    const int W = std::max(1, std::min(8, n / 4));
    std::atomic<int> next{0};
    std::exception_ptr err;
    std::mutex emu;
    auto work = [&]() {
        try {
            for (int k; (k = next.fetch_add(1)) < n;) prep[k] = prepare(inst[k]);
        } catch (...) {
            std::lock_guard<std::mutex> lk(emu);
            if (!err) err = std::current_exception();
        }
    };
    if (W == 1) {
        work();
    } else {
        std::vector<std::thread> th;
        for (int w = 0; w < W; ++w) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
    if (err) std::rethrow_exception(err);
    return prep;
}

// Where the results of a batch go: the fixed-stride records and, optionally,
// the tractions of both slip modes per instance (host arrays, may be null).
struct Outputs {
    double* results = nullptr;
    double* const* f_sphere = nullptr;  // [k]: 2 x 3 Ns (mode B1 = 1, then B2 = 1)
    double* const* f_tube = nullptr;    // [k]: 2 x 3 Nt
    double* fs(int k) const { return f_sphere ? f_sphere[k] : nullptr; }
    double* ft(int k) const { return f_tube ? f_tube[k] : nullptr; }
};

void validate(const sqbem_instance& in) {
    if (!(in.a_over_R >= 0 && in.a_over_R < 1) || !(in.beta >= 0 && in.beta < 1) || !(in.L_over_R > 0) ||
        in.sphere_level < 0 || in.sphere_level > 5 || (in.a_over_R > 0 && (in.n_theta < 3 || in.n_r < 1)))
        fail(SQBEM_ERR_ARG, "kinematics_batch: bad instance parameters");
    const double en = std::sqrt(in.e[0] * in.e[0] + in.e[1] * in.e[1] + in.e[2] * in.e[2]);
    if (!(std::fabs(en - 1.0) < 1e-12)) fail(SQBEM_ERR_ARG, "kinematics_batch: e must be a unit vector");
}

// One instance through the same handles the single-instance API uses.
void run_one(const sqbem_instance& in, const Prepared& P, int precision, cudaStream_t bs, double* res,
             double* f_sphere, double* f_tube) {
    std::unique_ptr<sqbem_tube> t;
    if (P.bounded) {
        t = std::make_unique<sqbem_tube>();
        t->st.borrow(bs);
        t->R = P.R; t->L = P.L; t->a = 1.0; t->n_theta = in.n_theta; t->n_r = in.n_r; t->mu = 1.0;
        t->precision = precision;
        t->mesh = P.tube;
        t->build_device();
    }
    sqbem_swimmer s;
    s.st.borrow(bs);
    const double c[3] = {P.b, 0, 0};
    s.build(t.get(), P.sphere.P(), P.sphereV.data(), c, 1.0, precision);
    auto u1 = squirmer_slip_host(s.host_panels, c, in.e, 1, 0);
    auto u2 = squirmer_slip_host(s.host_panels, c, in.e, 0, 1);
    std::vector<double> slips(u1);
    slips.insert(slips.end(), u2.begin(), u2.end());
    double U[6], Om[6];
    s.solve_free(2, slips.data(), U, Om, f_sphere, P.bounded ? f_tube : nullptr);
    for (int k = 0; k < 3; ++k) {
        res[k] = U[k];
        res[3 + k] = Om[k];
        res[6 + k] = U[3 + k];
        res[9 + k] = Om[3 + k];
    }
    res[12] = NAN;
    if (in.towed && std::fabs(P.b) < 1e-12) {
        const double Uz[3] = {0, 0, 1}, O0[3] = {0, 0, 0};
        std::vector<double> fs(3 * (size_t)s.Ns);
        s.solve_prescribed(Uz, O0, fs.data(), nullptr);
        double Fz = 0;  // force ON the sphere, F = -sum f dA (swimmer.hpp:156-160)
        for (int p = 0; p < s.Ns; ++p) Fz = Fz - s.host_panels[p].area * fs[3 * p + 2];
        res[12] = -Fz / (6 * bem::PI);
    }
    res[13] = s.Nt;
    res[14] = s.Ns;
    res[15] = s.ir_iterations;
}

// Mixed precision: instances with equal padded tube size and equal sphere size
// form a group; each group (in chunks of GROUP_MAX) is assembled member by
// member and then factored, Schur-reduced and refined with grouped launches.
// Members per chunk: SQBEM_GROUP_MAX, default 48 (at most 48 problems per
// grouped GEMM launch).
int group_max() {
    const char* e = std::getenv("SQBEM_GROUP_MAX");
    const int v = e ? std::atoi(e) : 48;
    return std::max(1, std::min(v, 48));
}

// Host wall time per phase of the grouped mixed path, printed to stderr when
// SQBEM_HOST_TIMING is set (profiling aid).
// Each line: the phase's duration and the time since the batch call began.
struct PhaseClock {
    bool on = std::getenv("SQBEM_HOST_TIMING") != nullptr;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    std::chrono::steady_clock::time_point t0 = t;
    void lap(const char* what, size_t G, int ntp, int ns) {
        if (!on) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "host %-14s G=%zu ntp=%d Ns=%d %.2f ms (at %.2f ms)\n", what, G, ntp, ns,
                     std::chrono::duration<double, std::milli>(now - t).count(),
                     std::chrono::duration<double, std::milli>(now - t0).count());
        t = now;
    }
};

// One chunk of a group (members with equal padded tube size and sphere size),
// everything on stream bs.
void run_chunk(const std::vector<int>& ids, int ntp_k, int ns_k, const sqbem_instance* inst,
               const std::vector<Prepared>& prep, cudaStream_t bs, const Outputs& out, PhaseClock& pc,
               const std::shared_ptr<const SphereBlocks>& share) {
    double* const results = out.results;
    const size_t G = ids.size();
    DevBuf<int> flags(2, bs);
    flags.zero();
    MixedCtx cx{bs, flags.get(), flags.get() + 1};
    std::vector<std::unique_ptr<sqbem_tube>> tubes(G);
    std::vector<std::unique_ptr<sqbem_swimmer>> sws(G);
    std::vector<sqbem_tube*> tp;
    std::vector<sqbem_swimmer*> sp;
    for (size_t g = 0; g < G; ++g) {
        const Prepared& P = prep[ids[g]];
        const sqbem_instance& in = inst[ids[g]];
        if (P.bounded) {
            tubes[g] = std::make_unique<sqbem_tube>();
            sqbem_tube& t = *tubes[g];
            t.st.borrow(bs);
            t.R = P.R; t.L = P.L; t.a = 1.0; t.n_theta = in.n_theta; t.n_r = in.n_r; t.mu = 1.0;
            t.precision = SQBEM_MIXED;
            t.mesh = P.tube;
            t.set_panels();
            tp.push_back(&t);
        }
    }
    pc.lap("setup", G, ntp_k, ns_k);
    if (!tp.empty()) mixed_build_tubes(tp, cx, /*explicit_inverse=*/false);  // each tube serves one swimmer
    pc.lap("tubes", G, ntp_k, ns_k);
    for (size_t g = 0; g < G; ++g) {
        const Prepared& P = prep[ids[g]];
        sws[g] = std::make_unique<sqbem_swimmer>();
        sws[g]->st.borrow(bs);
        const double c[3] = {P.b, 0, 0};
        sws[g]->set_geometry(tubes[g].get(), P.sphere.P(), P.sphereV.data(), c, 1.0, SQBEM_MIXED);
        sp.push_back(sws[g].get());
    }
    mixed_build_swimmers(sp, cx, share);
    pc.lap("swimmers", G, ntp_k, ns_k);
    // the B1 = 1 and B2 = 1 slip modes of every member, on the device
    std::vector<DevBuf<double>> slip(G), xs(G);
    std::vector<const double*> in_ptr;
    std::vector<double*> x_ptr;
    std::vector<SlipJob> sj;
    for (size_t g = 0; g < G; ++g) {
        sqbem_swimmer& s = *sws[g];
        slip[g].alloc((size_t)6 * s.Ns, bs);
        SlipJob j;
        j.rec = s.panels.rec.get();
        j.Ns = s.Ns;
        j.xc[0] = prep[ids[g]].b;
        for (int q = 0; q < 3; ++q) j.e[q] = inst[ids[g]].e[q];
        j.out = slip[g].get();
        sj.push_back(j);
        xs[g].alloc((size_t)(s.mx.nt + s.mx.nc) * 2, bs);
        in_ptr.push_back(slip[g].get());
        x_ptr.push_back(xs[g].get());
    }
    slip_modes_group(sj, bs);
    int iters = 0;
    double resid = 0;
    mixed_solve(sp, false, in_ptr, 2, x_ptr, cx, &iters, &resid);
    pc.lap("solve", G, ntp_k, ns_k);
    std::vector<std::vector<double>> hx(G);
    for (size_t g = 0; g < G; ++g) {
        hx[g].resize((size_t)(sws[g]->mx.nt + sws[g]->mx.nc) * 2);
        xs[g].download(hx[g].data(), hx[g].size());
    }
    // towed drag of the members on the axis (main.cpp:90-91)
    std::vector<sqbem_swimmer*> towed;
    std::vector<size_t> towed_g;
    for (size_t g = 0; g < G; ++g)
        if (inst[ids[g]].towed && std::fabs(prep[ids[g]].b) < 1e-12) {
            towed.push_back(sws[g].get());
            towed_g.push_back(g);
        }
    std::vector<std::vector<double>> hf(towed.size());
    if (!towed.empty()) {
        const double w6[6] = {0, 0, 1, 0, 0, 0};
        DevBuf<double> dw(6, bs);
        dw.upload(w6, 6);
        std::vector<DevBuf<double>> xt(towed.size());
        std::vector<const double*> wi;
        std::vector<double*> xo;
        for (size_t t = 0; t < towed.size(); ++t) {
            xt[t].alloc((size_t)(towed[t]->mx.nt + towed[t]->mx.nc), bs);
            wi.push_back(dw.get());
            xo.push_back(xt[t].get());
        }
        int it2 = 0;
        double r2 = 0;
        mixed_solve(towed, true, wi, 1, xo, cx, &it2, &r2);
        for (size_t t = 0; t < towed.size(); ++t) {
            hf[t].resize(xt[t].n);
            xt[t].download(hf[t].data(), hf[t].size());
        }
    }
    CUDA_CHECK(cudaStreamSynchronize(bs));
    for (size_t g = 0; g < G; ++g) {
        sqbem_swimmer& s = *sws[g];
        const int nt = s.mx.nt, ns = s.mx.ns, ldx = nt + s.mx.nc;
        double* res = results + (size_t)ids[g] * SQBEM_RESULT_STRIDE;
        for (int c = 0; c < 3; ++c) {
            res[c] = hx[g][nt + ns + c];
            res[3 + c] = hx[g][nt + ns + 3 + c];
            res[6 + c] = hx[g][ldx + nt + ns + c];
            res[9 + c] = hx[g][ldx + nt + ns + 3 + c];
        }
        res[12] = NAN;
        res[13] = s.Nt;
        res[14] = s.Ns;
        res[15] = iters;
        // x = [f_t; f_s; w] per mode
        for (int m = 0; m < 2; ++m) {
            if (double* fs = out.fs(ids[g]))
                std::memcpy(fs + (size_t)m * ns, hx[g].data() + (size_t)m * ldx + nt, sizeof(double) * ns);
            if (double* ft = out.ft(ids[g]); ft && nt)
                std::memcpy(ft + (size_t)m * nt, hx[g].data() + (size_t)m * ldx, sizeof(double) * nt);
        }
    }
    for (size_t t = 0; t < towed.size(); ++t) {
        sqbem_swimmer& s = *towed[t];
        double Fz = 0;
        for (int p = 0; p < s.Ns; ++p) Fz = Fz - s.host_panels[p].area * hf[t][s.mx.nt + 3 * p + 2];
        results[(size_t)ids[towed_g[t]] * SQBEM_RESULT_STRIDE + 12] = -Fz / (6 * bem::PI);
    }
}

// Device bytes a chunk holds at its peak, estimated from its sizes (FP32 tube
// block, inverse and split copies; swimmer blocks B, A_uBt, D, E, A_uBs, Y,
// G_s^{-1}; the LU working set), with a margin.
double chunk_bytes(size_t G, int ntp, int ns) {
    const double t = ntp, s = pad128(3 * ns);
    return 1.25 * G * 4.0 * (6.0 * t * t + 6.0 * t * s + 5.0 * s * s);
}

void run_mixed(int n, const sqbem_instance* inst, const std::vector<Prepared>& prep, cudaStream_t bs,
               const Outputs& out) {
    std::map<std::tuple<int, int, int>, std::vector<int>> groups;
    for (int k = 0; k < n; ++k) {
        const int ntp = prep[k].bounded ? pad128(3 * prep[k].tube.P()) : 0;
        groups[{prep[k].bounded ? 1 : 0, ntp, prep[k].sphere.P()}].push_back(k);
    }
    struct Chunk {
        std::vector<int> ids;
        int ntp, ns;
    };
    std::vector<Chunk> chunks;
    for (auto& kv : groups) {
        const std::vector<int>& all = kv.second;
        const size_t gm = (size_t)group_max();
        for (size_t c0 = 0; c0 < all.size(); c0 += gm)
            chunks.push_back({std::vector<int>(all.begin() + c0, all.begin() + std::min(all.size(), c0 + gm)),
                              std::get<1>(kv.first), std::get<2>(kv.first)});
    }
    // the larger spheres first: the longest tasks start early
    std::stable_sort(chunks.begin(), chunks.end(), [](const Chunk& a, const Chunk& b) {
        return a.ns != b.ns ? a.ns > b.ns : a.ids.size() > b.ids.size();
    });
    std::vector<double> bytes;
    for (const Chunk& c : chunks) bytes.push_back(chunk_bytes(c.ids.size(), c.ntp, c.ns));
    // the sphere-sphere blocks, translation invariant: assembled once per sphere
    // size for this call from its first instance, and shared by every chunk
    std::map<int, std::shared_ptr<const SphereBlocks>> shares;
    for (const Chunk& c : chunks) {
        if (shares.count(c.ns)) continue;
        const Prepared& P = prep[c.ids[0]];
        const double xc[3] = {P.b, 0, 0};
        shares[c.ns] = build_sphere_blocks(make_panels(P.sphereV.data(), P.sphere.P()), xc, 1.0, bs);
    }
    const auto call_start = std::chrono::steady_clock::now();
    run_concurrent(chunks.size(), bytes, bs, [&](size_t k, cudaStream_t st) {
        PhaseClock pc;
        pc.t0 = call_start;
        run_chunk(chunks[k].ids, chunks[k].ntp, chunks[k].ns, inst, prep, st, out, pc, shares[chunks[k].ns]);
    });
}

// FP64: one instance per task, the same concurrency as the mixed path.
void run_fp64(int n, const sqbem_instance* inst, const std::vector<Prepared>& prep, cudaStream_t bs,
              const Outputs& out) {
    std::vector<int> order(n);
    for (int k = 0; k < n; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return prep[a].sphere.P() > prep[b].sphere.P(); });
    std::vector<double> bytes;
    for (int k : order) {
        const double t = 3.0 * (prep[k].bounded ? prep[k].tube.P() : 0), s = 3.0 * prep[k].sphere.P();
        bytes.push_back(1.25 * 8.0 * (3.0 * t * t + 6.0 * t * s + 6.0 * s * s));
    }
    run_concurrent((size_t)n, bytes, bs, [&](size_t j, cudaStream_t st) {
        const int k = order[j];
        run_one(inst[k], prep[k], SQBEM_FP64, st, out.results + (size_t)k * SQBEM_RESULT_STRIDE, out.fs(k), out.ft(k));
    });
}

}  // namespace

namespace {
void kinematics_batch(int n, const sqbem_instance* inst, int precision, const Outputs& out, double* device_seconds) {
    if (n < 0 || (n > 0 && (!inst || !out.results)) || (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
        fail(SQBEM_ERR_ARG, "kinematics_batch: bad arguments");
    for (int k = 0; k < n; ++k) validate(inst[k]);
    if (device_seconds) *device_seconds = 0;
    if (n == 0) return;
    require_device();
    const std::vector<Prepared> prep = prepare_all(n, inst);
    Stream bs;
    EventTimer clk;
    clk.start(bs);
    if (precision == SQBEM_MIXED) run_mixed(n, inst, prep, bs, out);
    else run_fp64(n, inst, prep, bs, out);
    clk.stop(bs);
    const double secs = clk.seconds();
    if (device_seconds) *device_seconds = secs;
}
}  // namespace

extern "C" int sqbem_kinematics_batch(int n, const sqbem_instance* inst, int precision, double* results,
                                      double* device_seconds) {
    return guarded([&] {
        Outputs o;
        o.results = results;
        kinematics_batch(n, inst, precision, o, device_seconds);
    });
}

extern "C" int sqbem_kinematics_batch_tractions(int n, const sqbem_instance* inst, int precision, double* results,
                                                double* const* f_sphere, double* const* f_tube,
                                                double* device_seconds) {
    return guarded([&] {
        Outputs o;
        o.results = results;
        o.f_sphere = f_sphere;
        o.f_tube = f_tube;
        kinematics_batch(n, inst, precision, o, device_seconds);
    });
}

// Adjoint sensitivities per instance: build (FP64), both slip modes, and the
// translation derivatives of (U, Omega) for each (adjoint.cu).
extern "C" int sqbem_adjoint_batch(int n, const sqbem_instance* inst, int precision, double* results,
                                   double* device_seconds) {
    return guarded([&] {
        if (n < 0 || (n > 0 && (!inst || !results)) || precision != SQBEM_FP64)
            fail(SQBEM_ERR_ARG, "adjoint_batch: bad arguments (FP64 only)");
        for (int k = 0; k < n; ++k) validate(inst[k]);
        if (device_seconds) *device_seconds = 0;
        if (n == 0) return;
        require_device();
        Stream bs;
        EventTimer clk;
        clk.start(bs);
        const std::vector<Prepared> prep = prepare_all(n, inst);
        std::vector<double> bytes;
        for (int k = 0; k < n; ++k) {
            const double t = 3.0 * (prep[k].bounded ? prep[k].tube.P() : 0), sp = 3.0 * prep[k].sphere.P();
            bytes.push_back(1.25 * 8.0 * (3.0 * t * t + 7.0 * t * sp + 6.0 * sp * sp));
        }
        run_concurrent((size_t)n, bytes, bs, [&](size_t kk, cudaStream_t st) {
            const int k = (int)kk;
            const Prepared& P = prep[k];
            std::unique_ptr<sqbem_tube> t;
            if (P.bounded) {
                t = std::make_unique<sqbem_tube>();
                t->st.borrow(st);
                t->R = P.R; t->L = P.L; t->a = 1.0; t->n_theta = inst[k].n_theta; t->n_r = inst[k].n_r; t->mu = 1.0;
                t->precision = SQBEM_FP64;
                t->mesh = P.tube;
                t->build_device();
            }
            sqbem_swimmer s;
            s.st.borrow(st);
            const double c[3] = {P.b, 0, 0};
            s.build(t.get(), P.sphere.P(), P.sphereV.data(), c, 1.0, SQBEM_FP64);
            auto slips = squirmer_slip_host(s.host_panels, c, inst[k].e, 1, 0);
            const auto u2 = squirmer_slip_host(s.host_panels, c, inst[k].e, 0, 1);
            slips.insert(slips.end(), u2.begin(), u2.end());
            double U[6], Om[6], dU[18], dOm[18];
            s.adjoint(2, slips.data(), U, Om, dU, dOm);
            double* r = results + (size_t)k * SQBEM_ADJOINT_STRIDE;
            for (int m = 0; m < 2; ++m) {
                double* o = r + 24 * m;
                for (int a = 0; a < 3; ++a) {
                    o[a] = U[3 * m + a];
                    o[3 + a] = Om[3 * m + a];
                }
                for (int e = 0; e < 9; ++e) {
                    o[6 + e] = dU[9 * m + e];
                    o[15 + e] = dOm[9 * m + e];
                }
            }
        });
        clk.stop(bs);
        const double secs = clk.seconds();
        if (device_seconds) *device_seconds = secs;
    });
}
