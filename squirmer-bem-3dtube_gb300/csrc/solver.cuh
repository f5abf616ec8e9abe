// solver.cuh -- device-resident state behind the C ABI handles.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "assemble.cuh"
#include "bem/utils/mesh.hpp"
#include "common.cuh"
#include "dense.cuh"
#include "mixed.cuh"
#include "mixed_solver.cuh"

namespace sqbem {

// A CUDA stream owned by a handle, or borrowed from the caller (batched calls
// run every handle on the batch stream).
// A stream of its own, created at first use, or one borrowed from the caller
// (batched paths hand every member the group's stream, and creating a stream
// per member only to drop it cost tens of microseconds each).
struct Stream {
    mutable cudaStream_t s = nullptr;
    mutable std::once_flag once;
    bool owned = true;
    Stream() = default;
    ~Stream();
    Stream(const Stream&) = delete;
    Stream& operator=(const Stream&) = delete;
    void borrow(cudaStream_t other);
    cudaStream_t get() const;
    operator cudaStream_t() const { return get(); }
};

// Panels of one mesh on the device: records + centroids (targets).
struct DevPanels {
    int P = 0;
    DevBuf<PanelRec> rec;
    DevBuf<double> cent;
    double area_total = 0;  // sum of areas in panel order (swimmer.hpp:66)
    double area_max = 0;    // max of 5 * area (swimmer.hpp:116)
    void set(const std::vector<PanelRec>& host, cudaStream_t st);
};

std::vector<PanelRec> make_panels(const double* V, int P);
std::vector<double> mesh_vertices(const bem::Mesh& m);
std::vector<double> rigid_map(const std::vector<PanelRec>& S, const double* xc);
std::vector<double> constraint_rows(const std::vector<PanelRec>& S, const double* xc, double sc);
template <class T>
void deflate(T* A, long long rs, long long cs, const DevPanels& P, double mu, cudaStream_t st);

// Device timer on a stream.
struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer() {
        CUDA_CHECK(cudaEventCreate(&a));
        CUDA_CHECK(cudaEventCreate(&b));
    }
    ~EventTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    void start(cudaStream_t s) { CUDA_CHECK(cudaEventRecord(a, s)); }
    void stop(cudaStream_t s) { CUDA_CHECK(cudaEventRecord(b, s)); }
    double seconds() {
        CUDA_CHECK(cudaEventSynchronize(b));
        float ms = 0;
        CUDA_CHECK(cudaEventElapsedTime(&ms, a, b));
        return ms * 1e-3;
    }
};

}  // namespace sqbem

// Tube, src/swimmer.hpp:33-75
struct sqbem_tube {
    sqbem::Stream st;
    int precision = SQBEM_FP64;
    double R = 1, L = 4, a = 1, mu = 1;
    int n_theta = 0, n_r = 4;
    bem::Mesh mesh;
    int Nt = 0;
    std::vector<sqbem::PanelRec> host_panels;
    sqbem::DevPanels panels;
    sqbem::LU64 lu;           // FP64 factor of the deflated T
    sqbem::MixedTube mt;      // mixed: FP32 T (for residuals) and its split-BF16 factor
    void build(double R, double L, double a, int n_theta, int n_r, double mu, int precision);
    void build_device();  // from `mesh` and the parameters already set
    void set_panels();    // panel records only (the grouped mixed build factors later)
};

// host slip field (kernels.hpp:107-111) at the panel centroids, packed xyz
std::vector<double> squirmer_slip_host(const std::vector<sqbem::PanelRec>& S, const double* xc, const double* e,
                                       double B1, double B2);

namespace sqbem {
// The same slip field on the device, bit-identical to squirmer_slip_host: for
// every job, out[0 .. 3 Ns) = the B1 = 1 mode and out[3 Ns .. 6 Ns) = the B2 = 1
// mode at the centroids of the Ns panel records (one grouped launch).
struct SlipJob {
    const PanelRec* rec = nullptr;
    int Ns = 0;
    double xc[3] = {0, 0, 0};
    double e[3] = {0, 0, 1};
    double* out = nullptr;
};
void slip_modes_group(const std::vector<SlipJob>& jobs, cudaStream_t st);
}  // namespace sqbem

// SwimmerSolver, src/swimmer.hpp:83-289
struct sqbem_swimmer {
    sqbem::Stream st;
    const sqbem_tube* tube = nullptr;
    int precision = SQBEM_FP64;
    double mu = 1;
    double xc[3] = {0, 0, 0};
    int Ns = 0, Nt = 0;
    std::vector<sqbem::PanelRec> host_panels;
    sqbem::DevPanels panels;
    // FP64 path (column-major)
    sqbem::DevBuf<double> Gs, Gc, AuBt, AuBs, D, Y;
    sqbem::LU64 luM, luGs;
    bool haveM = false, haveGs = false;
    // mixed path
    sqbem::MixedSwimmer mx;
    double t_assembly = 0, t_schur = 0;
    int ir_iterations = 0;
    double ir_residual = 0;
    void build(const sqbem_tube* tube, int Ns, const double* V, const double* center, double mu, int precision);
    void set_geometry(const sqbem_tube* tube, int Ns, const double* V, const double* center, double mu,
                      int precision);
    void build_fp64();
    void factor_M();  // LU of M = [Gs Gc; F 0] (FP64 path), once
    void solve_free(int nrhs, const double* slips, double* U, double* Om, double* f_sphere, double* f_tube);
    void solve_prescribed(const double* U, const double* Om, double* f_sphere, double* f_tube);
    void solve_mixed(bool prescribed, int nrhs, const double* in, double* U, double* Om, double* f_sphere,
                     double* f_tube);
    // free-swimming solutions and their derivatives with respect to a rigid
    // translation of the sphere (adjoint.cu); per right-hand side 3 + 3 + 9 + 9
    void adjoint(int nrhs, const double* slips, double* U, double* Om, double* dU_dc, double* dOm_dc);
};

// DuctFlow, src/duct_flow.hpp:22-109
struct sqbem_duct {
    sqbem::Stream st;
    int precision = SQBEM_FP64;
    double R = 1, L = 4, mu = 1;
    bem::Mesh mesh;
    int P = 0;
    std::vector<int> cap;  // cap panel indices (columns of Fk)
    sqbem::DevPanels panels;
    sqbem::LU64 lu;
    sqbem::DevBuf<double> Fk;
    void build(double R, double L, int n_theta, int n_z, int n_r, double mu, int precision);
    void solve(double p_in, double p_out, double* u, double* f, double* Q);
};
