// assemble.cuh -- device-side panel records and assembly / field job descriptors.
#pragma once
#include <cuda_runtime.h>

namespace sqbem {

// One source panel as the kernels read it (144 bytes): vertices, unit normal
// (out of the fluid), centroid, area and h = sqrt(2 area) -- the fields of
// Mesh::geometry (src/utils/mesh.hpp:55-72).
// Algorithmic flops of one quadrature-node evaluation (accum in assemble.cu,
// FMA = 2): r from the vertex vectors 15, |r|^2 5, 1/|r| 1, powers 2, s 1,
// r.m 5, d 3, diagonal 2, s r 3, SL 12, d r 3, DL 12.
constexpr double FLOPS_PER_EVAL = 64.0;
// The self integral's evaluations form SL only: without r.m 5, d 3, d r 3, DL 12.
constexpr double FLOPS_PER_EVAL_SL = 41.0;

struct PanelRec {
    double v[9];
    double n[3];
    double c[3];
    double area, h, pad;
};
static_assert(sizeof(PanelRec) == 144, "PanelRec layout");

// One coupling block: targets are points (panel centroids), sources are panels.
// S receives SL * sscale, D receives DL * dscale, at element
// (row, col) -> row * rs + col * cs with row = 3i + a, col = 3p + b.
template <class TO>
struct BlockJob {
    const double* tgt = nullptr;  // 3 per target
    int nT = 0;
    const PanelRec* src = nullptr;
    int nS = 0;
    int same_mesh = 0;  // target i is the centroid of source panel i -> self integral
    // same_mesh == 0: target i is the centroid of source panel self_of[i] (self
    // integral there; a negative entry: none); null: no target is a centroid
    const int* self_of = nullptr;
    TO* S = nullptr;
    long long s_rs = 1, s_cs = 0;
    TO* D = nullptr;
    long long d_rs = 1, d_cs = 0;
    double sscale = 0, dscale = 0;
    int2* near_list = nullptr;
    int* near_count = nullptr;  // [heavy, light, work counter] (assemble.cu)
    int near_cap = 0;
    int* rule_count = nullptr;  // [5]: near pairs per rule, counted only for kernel statistics
};

struct FieldJob {
    const double* pts = nullptr;  // 3 per point
    int npts = 0;
    const PanelRec* panels = nullptr;
    int P = 0;
    const double* u = nullptr;  // 3 per panel
    const double* f = nullptr;  // 3 per panel
    double sscale = 0, dscale = 0;
    double* out = nullptr;  // 3 per point
    int* overflow = nullptr;
    int mixed = 0;
};

void init_tables();
template <class TO>
void assemble_block(const BlockJob<TO>& job, int near_cap, cudaStream_t st, bool mixed);
template <class T>
void add_rowsums(const T* D, long long rs, long long cs, int nrows, int ncolpanels, double* out, cudaStream_t st);
template <class T>
void diag_complete(T* A, long long rs, long long cs, int n, const double* rsum, double ext,
                   const unsigned char* mask, cudaStream_t st);
void panel_pairs(int n, const PanelRec* P, const double* x0, const int* self, double* SL, double* DL,
                 cudaStream_t st);
void field_eval(const FieldJob& job, cudaStream_t st);

}  // namespace sqbem

namespace sqbem {

// One sphere-tube coupling term of the adjoint contraction (adjoint.cu).  For a
// rigid translation c of the sphere, every target x (3 per target) and every
// source panel s contribute, per adjoint vector o < 6 and solution j < nm,
//   gs * sum_q w_q grad_r [lam_o . G(r) f_j] + ts * sum_q w_q grad_r [lam_o . T(r).m_s v_j],
// r = x_q - x, with the quadrature of the assembly (same rule choice).
// lam[3t + a + o*lam_ld] belongs to target t; f[3s + a + j*f_ld] to source s;
// v[3i + a + j*v_ld] to the sphere panel i, which is the source when v_src = 1
// and the target otherwise.
struct AdjTerm {
    const double* tgt = nullptr;
    int nT = 0;
    const double* lam = nullptr;
    long long lam_ld = 0;
    const PanelRec* src = nullptr;
    int nS = 0;
    const double* f = nullptr;
    long long f_ld = 0;
    const double* v = nullptr;
    long long v_ld = 0;
    int v_src = 0;
    double gs = 0, ts = 0;
};
constexpr int ADJ_MAX_MODES = 2;
// out[o*6 + j*3 + k] (6 x ADJ_MAX_MODES x 3) <- sum over the terms; nm <= ADJ_MAX_MODES.
// Deterministic: per-CTA partials reduced in a fixed order.
void adjoint_pairs(const AdjTerm* terms, int nterms, int nm, double* out, cudaStream_t st);

// y = rsqrt_nr(x) elementwise on device arrays: the FP64 reciprocal square root of
// the mixed path's near-singular and self integrals (for its accuracy test).
void rsqrt_nr_eval(int n, const double* x, double* y, cudaStream_t st);

}  // namespace sqbem
