// api.cu -- the C ABI (include/sqbem.h): host-side orchestration of the BEM
// solves on one GPU.  Geometry is produced on the host (bit-identical to the
// reference's mesh.hpp); every O(N^2) and O(N^3) step runs in CUDA kernels of
// this library.  There is no CPU fallback.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "assemble.cuh"
#include "bem/utils/mesh.hpp"
#include "common.cuh"
#include "dense.cuh"
#include "solver.cuh"

namespace sqbem {

std::atomic<long long> g_launches{0};
static thread_local std::string g_last_error;

void require_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        (void)cudaGetLastError();
        fail(SQBEM_ERR_NO_DEVICE, "no CUDA device available (%s)", e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
    }
}

void set_last_error(const char* msg) { g_last_error = msg; }

static std::atomic<long long> g_wait_cycles{DEFAULT_WAIT_CYCLES};
static std::atomic<int> g_refine_max_it{DEFAULT_REFINE_MAX_IT};
long long gemm_wait_cycles() { return g_wait_cycles.load(std::memory_order_relaxed); }
int refine_max_iterations() { return g_refine_max_it.load(std::memory_order_relaxed); }

// Per-panel geometry exactly as Mesh::geometry (mesh.hpp:61-72).
std::vector<PanelRec> make_panels(const double* V, int P) {
    std::vector<PanelRec> out((size_t)P);
    for (int p = 0; p < P; ++p) {
        const double* v = V + 9 * (size_t)p;
        const bem::V3 a{v[0], v[1], v[2]}, b{v[3], v[4], v[5]}, c{v[6], v[7], v[8]};
        const bem::V3 cr = bem::cross(b - a, c - a);
        const double area = 0.5 * bem::norm(cr);
        const bem::V3 n = (1.0 / (2 * area)) * cr;
        const bem::V3 ce = (1.0 / 3) * (a + b + c);
        PanelRec& r = out[p];
        std::memcpy(r.v, v, 9 * sizeof(double));
        r.n[0] = n.x; r.n[1] = n.y; r.n[2] = n.z;
        r.c[0] = ce.x; r.c[1] = ce.y; r.c[2] = ce.z;
        r.area = area;
        r.h = std::sqrt(2 * area);
        r.pad = 0;
    }
    return out;
}

std::vector<double> mesh_vertices(const bem::Mesh& m) {
    std::vector<double> V((size_t)m.P() * 9);
    for (int p = 0; p < m.P(); ++p)
        for (int k = 0; k < 3; ++k) {
            V[9 * p + 3 * k] = m.V[p][k].x;
            V[9 * p + 3 * k + 1] = m.V[p][k].y;
            V[9 * p + 3 * k + 2] = m.V[p][k].z;
        }
    return V;
}

void DevPanels::set(const std::vector<PanelRec>& host, cudaStream_t st) {
    P = (int)host.size();
    rec.alloc(host.size(), st);
    rec.upload(host.data(), host.size());
    std::vector<double> c((size_t)P * 3);
    for (int p = 0; p < P; ++p) {
        c[3 * p] = host[p].c[0];
        c[3 * p + 1] = host[p].c[1];
        c[3 * p + 2] = host[p].c[2];
    }
    cent.alloc(c.size(), st);
    cent.upload(c.data(), c.size());
    area_total = 0;
    for (int p = 0; p < P; ++p) area_total += host[p].area;
    area_max = 0;
    for (int p = 0; p < P; ++p) area_max = std::max(area_max, 5.0 * host[p].area);
}

cudaStream_t Stream::get() const {
    if (owned) std::call_once(once, [this] { CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); });
    return s;
}
Stream::~Stream() {
    if (s && owned) cudaStreamDestroy(s);
}
void Stream::borrow(cudaStream_t other) {
    if (s && owned) cudaStreamDestroy(s);
    s = other;
    owned = false;
}

// ---------------------------------------------------------------- deflation
// A(off + 3i + a, off + 3p + b) += sc m_i[a] m_p[b] A_p  (swimmer.hpp:64-74)
template <class T>
__global__ void deflate_kernel(T* A, long long rs, long long cs, const PanelRec* __restrict__ P, int np, double sc) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = 3LL * np;
    if (t >= n * n) return;
    const int r = (int)(t % n), c = (int)(t / n);
    const int i = r / 3, a = r % 3, p = c / 3, b = c % 3;
    const double v = sc * P[i].n[a] * P[p].n[b] * P[p].area;
    A[r * rs + c * cs] = (T)((double)A[r * rs + c * cs] + v);
}

template <class T>
void deflate(T* A, long long rs, long long cs, const DevPanels& P, double mu, cudaStream_t st) {
    const double sc = 1.0 / (EIGHT_PI * mu * std::sqrt(P.area_total));
    const long long n = 3LL * P.P;
    if (n == 0) return;
    LAUNCH(deflate_kernel<T>, ceil_div(n * n, 256), 256, 0, st, A, rs, cs, P.rec.get(), P.P, sc);
}
template void deflate<double>(double*, long long, long long, const DevPanels&, double, cudaStream_t);
template void deflate<float>(float*, long long, long long, const DevPanels&, double, cudaStream_t);

// rigid-body map K (3Ns x 6, column-major): u = U + Omega x r  (swimmer.hpp:224-231)
std::vector<double> rigid_map(const std::vector<PanelRec>& S, const double* xc) {
    const int Ns = (int)S.size(), ns = 3 * Ns;
    std::vector<double> K((size_t)ns * 6, 0.0);
    for (int p = 0; p < Ns; ++p) {
        const double rx = S[p].c[0] - xc[0], ry = S[p].c[1] - xc[1], rz = S[p].c[2] - xc[2];
        for (int a = 0; a < 3; ++a) K[(3 * p + a) + (size_t)a * ns] = 1;
        K[(3 * p + 0) + 4 * (size_t)ns] = rz;  K[(3 * p + 0) + 5 * (size_t)ns] = -ry;
        K[(3 * p + 1) + 3 * (size_t)ns] = -rz; K[(3 * p + 1) + 5 * (size_t)ns] = rx;
        K[(3 * p + 2) + 3 * (size_t)ns] = ry;  K[(3 * p + 2) + 4 * (size_t)ns] = -rx;
    }
    return K;
}

// scaled force-free / torque-free rows (6 x 3Ns, column-major ld 6), swimmer.hpp:114-125
std::vector<double> constraint_rows(const std::vector<PanelRec>& S, const double* xc, double sc) {
    const int Ns = (int)S.size(), ns = 3 * Ns;
    std::vector<double> F((size_t)6 * ns, 0.0);
    auto at = [&](int r, int c) -> double& { return F[r + 6 * (size_t)c]; };
    for (int p = 0; p < Ns; ++p) {
        const double rx = S[p].c[0] - xc[0], ry = S[p].c[1] - xc[1], rz = S[p].c[2] - xc[2];
        const double A = S[p].area * sc;
        for (int a = 0; a < 3; ++a) at(a, 3 * p + a) = A;
        at(3, 3 * p + 1) = -A * rz; at(3, 3 * p + 2) = A * ry;
        at(4, 3 * p + 0) = A * rz;  at(4, 3 * p + 2) = -A * rx;
        at(5, 3 * p + 0) = -A * ry; at(5, 3 * p + 1) = A * rx;
    }
    return F;
}

}  // namespace sqbem

using namespace sqbem;

// ---------------------------------------------------------------- C ABI: misc
extern "C" const char* sqbem_last_error(void) { return g_last_error.c_str(); }
extern "C" const char* sqbem_version(void) { return "sqbem 0.1 (sm_103a)"; }
extern "C" long long sqbem_launch_count(void) { return g_launches.load(); }

extern "C" int sqbem_set_limits(long long gemm_wait_cycles, int refine_max_iterations) {
    return guarded([&] {
        if (refine_max_iterations > 1000) fail(SQBEM_ERR_ARG, "set_limits: at most 1000 refinement steps");
        g_wait_cycles.store(gemm_wait_cycles < 0 ? DEFAULT_WAIT_CYCLES : gemm_wait_cycles);
        g_refine_max_it.store(refine_max_iterations < 0 ? DEFAULT_REFINE_MAX_IT : refine_max_iterations);
    });
}

// ---------------------------------------------------------------- geometry
static int put_mesh(const bem::Mesh& m, double* V, int* tags, int cap, int* P) {
    if (P) *P = m.P();
    if (V && cap >= m.P()) {
        auto v = mesh_vertices(m);
        std::memcpy(V, v.data(), v.size() * sizeof(double));
    }
    if (tags && cap >= m.P())
        for (int p = 0; p < m.P(); ++p) tags[p] = m.tags[p];
    return SQBEM_OK;
}

extern "C" int sqbem_tube_mesh(double R, const double* z, int nz1, int n_theta, int n_r, double* V, int* tags,
                               int cap, int* P) {
    return guarded([&] {
        if (!z || nz1 < 2 || n_theta < 3 || n_r < 1) fail(SQBEM_ERR_ARG, "tube_mesh: bad arguments");
        put_mesh(bem::tube_mesh(R, std::vector<double>(z, z + nz1), n_theta, n_r), V, tags, cap, P);
    });
}

extern "C" int sqbem_swimmer_tube_mesh(double R, double L, double a, int n_theta, int n_r, double* V, int* tags,
                                       int cap, int* P) {
    return guarded([&] {
        if (n_theta < 3 || n_r < 1 || !(R > 0) || !(L > 0)) fail(SQBEM_ERR_ARG, "swimmer_tube_mesh: bad arguments");
        put_mesh(bem::swimmer_tube_mesh(R, L, a, n_theta, n_r), V, tags, cap, P);
    });
}

extern "C" int sqbem_uniform_z(double z0, double z1, int nz, double* z) {
    return guarded([&] {
        if (nz < 1 || !z) fail(SQBEM_ERR_ARG, "uniform_z: bad arguments");
        auto v = bem::uniform_z(z0, z1, nz);
        std::memcpy(z, v.data(), v.size() * sizeof(double));
    });
}

extern "C" int sqbem_icosphere(double a, int level, const double* center, int tag, double* V, int* tags, int cap,
                               int* P) {
    return guarded([&] {
        if (level < 0 || level > 7 || !(a > 0)) fail(SQBEM_ERR_ARG, "icosphere: bad arguments");
        bem::V3 c{};
        if (center) c = {center[0], center[1], center[2]};
        put_mesh(bem::icosphere(a, level, c, tag), V, tags, cap, P);
    });
}

extern "C" int sqbem_geometry(int P, const double* V, double* normal, double* centroid, double* area, double* h) {
    return guarded([&] {
        if (P < 0 || (P > 0 && !V)) fail(SQBEM_ERR_ARG, "geometry: bad arguments");
        auto pr = make_panels(V, P);
        for (int p = 0; p < P; ++p) {
            if (normal) std::memcpy(normal + 3 * p, pr[p].n, 3 * sizeof(double));
            if (centroid) std::memcpy(centroid + 3 * p, pr[p].c, 3 * sizeof(double));
            if (area) area[p] = pr[p].area;
            if (h) h[p] = pr[p].h;
        }
    });
}

// ---------------------------------------------------------------- panel integrals
extern "C" int sqbem_panel_integrals(int n, const double* V9, const double* x0, const int* self, double* SL,
                                     double* DL) {
    return guarded([&] {
        if (n < 0 || (n > 0 && (!V9 || !x0 || !self || !SL || !DL))) fail(SQBEM_ERR_ARG, "panel_integrals: bad arguments");
        if (n == 0) return;
        require_device();
        Stream s;
        auto pr = make_panels(V9, n);
        DevBuf<PanelRec> dP(n, s);
        dP.upload(pr.data(), n);
        DevBuf<double> dx(3 * (size_t)n, s), dsl(9 * (size_t)n, s), ddl(9 * (size_t)n, s);
        DevBuf<int> dself(n, s);
        dx.upload(x0, 3 * (size_t)n);
        dself.upload(self, n);
        panel_pairs(n, dP.get(), dx.get(), dself.get(), dsl.get(), ddl.get(), s);
        dsl.download(SL, 9 * (size_t)n);
        ddl.download(DL, 9 * (size_t)n);
        CUDA_CHECK(cudaStreamSynchronize(s));
    });
}

// Test hook, not part of the public ABI: the mixed path's FP64 reciprocal
// square root on n host values (its error bound is checked by the GPU tests).
extern "C" int sqbem_test_rsqrt_nr(int n, const double* x, double* y) {
    return guarded([&] {
        if (n < 0 || (n > 0 && (!x || !y))) fail(SQBEM_ERR_ARG, "test_rsqrt_nr: bad arguments");
        if (n == 0) return;
        require_device();
        Stream s;
        DevBuf<double> dx(n, s), dy(n, s);
        dx.upload(x, n);
        rsqrt_nr_eval(n, dx.get(), dy.get(), s);
        dy.download(y, n);
        CUDA_CHECK(cudaStreamSynchronize(s));
    });
}

// ---------------------------------------------------------------- dense
extern "C" int sqbem_solve_dense(int n, int nrhs, const double* A, double* B, int* pivoted) {
    return guarded([&] {
        if (n <= 0 || nrhs < 0 || !A || (nrhs > 0 && !B)) fail(SQBEM_ERR_ARG, "solve_dense: bad arguments");
        require_device();
        Stream s;
        DevBuf<double> dA((size_t)n * n, s), dB((size_t)n * std::max(nrhs, 1), s);
        dA.upload(A, (size_t)n * n);
        if (nrhs) dB.upload(B, (size_t)n * nrhs);
        LU64 lu;
        lu.factor_inplace(std::move(dA), n, s, "dgesv failed");
        lu.solve(dB.get(), n, nrhs, s);
        if (nrhs) dB.download(B, (size_t)n * nrhs);
        CUDA_CHECK(cudaStreamSynchronize(s));
        if (pivoted) *pivoted = lu.pivoted ? 1 : 0;
    });
}

// ---------------------------------------------------------------- field
extern "C" int sqbem_velocity_at(int P, const double* V, const double* u, const double* f, double mu, int npts,
                                 const double* pts, double* out, int precision) {
    return guarded([&] {
        if (P < 0 || npts < 0 || (P > 0 && (!V || !u || !f)) || (npts > 0 && (!pts || !out)))
            fail(SQBEM_ERR_ARG, "velocity_at: bad arguments");
        if (npts == 0) return;
        require_device();
        Stream s;
        DevPanels dp;
        dp.set(make_panels(V, P), s);
        DevBuf<double> du(3 * (size_t)P, s), df(3 * (size_t)P, s), dpts(3 * (size_t)npts, s), dout(3 * (size_t)npts, s);
        DevBuf<int> ovf(1, s);
        ovf.zero();
        du.upload(u, 3 * (size_t)P);
        df.upload(f, 3 * (size_t)P);
        dpts.upload(pts, 3 * (size_t)npts);
        FieldJob job;
        job.pts = dpts.get();
        job.npts = npts;
        job.panels = dp.rec.get();
        job.P = P;
        job.u = du.get();
        job.f = df.get();
        job.sscale = 1.0 / (EIGHT_PI * mu);
        job.dscale = -1.0 / EIGHT_PI;
        job.out = dout.get();
        job.overflow = ovf.get();
        job.mixed = precision == SQBEM_MIXED;
        field_eval(job, s);
        int h_ovf = 0;
        dout.download(out, 3 * (size_t)npts);
        ovf.download(&h_ovf, 1);
        CUDA_CHECK(cudaStreamSynchronize(s));
        if (h_ovf) fail(SQBEM_ERR_ARG, "velocity_at: a point has more than 256 near panels");
    });
}

// ---------------------------------------------------------------- tube
extern "C" int sqbem_tube_create(double R, double L, double a, int n_theta, int n_r, double mu, int precision,
                                 sqbem_tube** out) {
    return guarded([&] {
        if (!out || !(R > 0) || !(L > 0) || n_theta < 3 || n_r < 1 || !(mu > 0) ||
            (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "Tube: bad arguments");
        require_device();
        auto t = std::make_unique<sqbem_tube>();
        t->build(R, L, a, n_theta, n_r, mu, precision);
        *out = t.release();
    });
}

extern "C" int sqbem_tube_panels(const sqbem_tube* t, int* Nt) {
    return guarded([&] {
        if (!t || !Nt) fail(SQBEM_ERR_ARG, "tube_panels: null argument");
        *Nt = t->Nt;
    });
}

extern "C" int sqbem_tube_mesh_get(const sqbem_tube* t, double* V, int* tags) {
    return guarded([&] {
        if (!t) fail(SQBEM_ERR_ARG, "tube_mesh_get: null tube");
        put_mesh(t->mesh, V, tags, t->Nt, nullptr);
    });
}

extern "C" void sqbem_tube_destroy(sqbem_tube* t) { delete t; }

// ---------------------------------------------------------------- swimmer
extern "C" int sqbem_swimmer_create(const sqbem_tube* tube, int Ns, const double* V, const int* tags,
                                    const double* center, double mu, int precision, sqbem_swimmer** out) {
    return guarded([&] {
        (void)tags;
        if (!out || Ns <= 0 || !V || !center || !(mu > 0) ||
            (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "SwimmerSolver: bad arguments");
        require_device();
        auto s = std::make_unique<sqbem_swimmer>();
        s->build(tube, Ns, V, center, mu, precision);
        *out = s.release();
    });
}

extern "C" int sqbem_swimmer_solve_free(sqbem_swimmer* s, int nrhs, const double* slips, double* U, double* Om,
                                        double* f_sphere, double* f_tube) {
    return guarded([&] {
        if (!s || nrhs <= 0 || !slips || !U || !Om) fail(SQBEM_ERR_ARG, "solve_free: bad arguments");
        s->solve_free(nrhs, slips, U, Om, f_sphere, f_tube);
    });
}

extern "C" int sqbem_swimmer_solve_prescribed(sqbem_swimmer* s, const double* U, const double* Om, double* f_sphere,
                                              double* f_tube) {
    return guarded([&] {
        if (!s || !U || !Om) fail(SQBEM_ERR_ARG, "solve_prescribed: bad arguments");
        s->solve_prescribed(U, Om, f_sphere, f_tube);
    });
}

extern "C" int sqbem_swimmer_adjoint(sqbem_swimmer* s, int nrhs, const double* slips, double* U, double* Om,
                                     double* dU_dc, double* dOm_dc) {
    return guarded([&] {
        if (!s || nrhs <= 0 || !slips || !U || !Om || !dU_dc || !dOm_dc) fail(SQBEM_ERR_ARG, "adjoint: bad arguments");
        s->adjoint(nrhs, slips, U, Om, dU_dc, dOm_dc);
    });
}

extern "C" int sqbem_swimmer_timings(const sqbem_swimmer* s, double* ta, double* ts) {
    return guarded([&] {
        if (!s) fail(SQBEM_ERR_ARG, "timings: null swimmer");
        if (ta) *ta = s->t_assembly;
        if (ts) *ts = s->t_schur;
    });
}

extern "C" int sqbem_swimmer_refinement(const sqbem_swimmer* s, int* it, double* res) {
    return guarded([&] {
        if (!s) fail(SQBEM_ERR_ARG, "refinement: null swimmer");
        if (it) *it = s->ir_iterations;
        if (res) *res = s->ir_residual;
    });
}

extern "C" void sqbem_swimmer_destroy(sqbem_swimmer* s) { delete s; }

// ---------------------------------------------------------------- duct
extern "C" int sqbem_duct_create(double R, double L, int n_theta, int n_z, int n_r, double mu, int precision,
                                 sqbem_duct** out) {
    return guarded([&] {
        if (!out || !(R > 0) || !(L > 0) || n_theta < 3 || n_z < 1 || n_r < 1 || !(mu > 0) ||
            (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "DuctFlow: bad arguments");
        require_device();
        auto d = std::make_unique<sqbem_duct>();
        d->build(R, L, n_theta, n_z, n_r, mu, precision);
        *out = d.release();
    });
}

extern "C" int sqbem_duct_panels(const sqbem_duct* d, int* P) {
    return guarded([&] {
        if (!d || !P) fail(SQBEM_ERR_ARG, "duct_panels: null argument");
        *P = d->P;
    });
}

extern "C" int sqbem_duct_mesh_get(const sqbem_duct* d, double* V, int* tags) {
    return guarded([&] {
        if (!d) fail(SQBEM_ERR_ARG, "duct_mesh_get: null duct");
        put_mesh(d->mesh, V, tags, d->P, nullptr);
    });
}

extern "C" int sqbem_duct_solve(sqbem_duct* d, double p_in, double p_out, double* u, double* f, double* Q) {
    return guarded([&] {
        if (!d || !Q) fail(SQBEM_ERR_ARG, "duct_solve: bad arguments");
        d->solve(p_in, p_out, u, f, Q);
    });
}

extern "C" void sqbem_duct_destroy(sqbem_duct* d) { delete d; }
