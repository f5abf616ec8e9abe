// assemble.cu -- panel-quadrature assembly of the BEM blocks, panel integrals
// and the field (representation formula) on the GPU.
//
// Physics, as in the reference (src/utils/kernels.hpp:8-21, 29-82):
//   SL_ij = int_p G_ij dS,  G_ij(r) = d_ij/|r| + r_i r_j/|r|^3,
//   DL_ij = int_p T_ijk m_k dS,  T_ijk(r) = -6 r_i r_j r_k/|r|^5,  r = x - x0,
// with the rule chosen by d = |c_p - x0| / h_p: d >= 3 -> 7 points, >= 1.5 ->
// 28, >= 0.75 -> 112, else 448 (Dunavant-7 on 1/4/16/64 sub-triangles), and the
// self panel by a Duffy transform over three sub-triangles with 10 x 10
// Gauss-Legendre points (DL = 0 there, since r.m = 0 on a flat panel).
//
// GPU structure (one block = a set of target centroids x sources panels):
//   far_kernel   one thread per (target, source) pair, 64 targets x 16 sources
//                per CTA; source panels staged in shared memory; pairs with
//                d >= 3 use the 7-point rule in registers and write their 3x3
//                blocks (coalesced: consecutive threads own consecutive rows of
//                a column-major block); pairs with d < 3 and the self pair are
//                appended to a near list.
//   near_kernel  one warp per near pair: the lanes split the 28/112/448 rule
//                points (or the 300 Duffy points), reduce with warp shuffles,
//                and lanes 0..8 write the entries.  Entries have fixed positions,
//                so the result does not depend on the list order.
//   rowsum / completion kernels: the completed double layer adds -sum_p D_ip to
//                the diagonal 3x3 blocks (duct_flow.hpp:103-105,
//                swimmer.hpp:218-220), computed by a fixed-order reduction over
//                the stored D block (deterministic).
// Precision: FP64 everywhere in SQBEM_FP64 mode.  In SQBEM_MIXED mode the
// relative vectors (vertex and centroid offsets) and the rule choice are FP64,
// rounded once; the far (7) and near (28/112) rules are evaluated in FP32 from
// them, while the 448-point near-singular rule and the Duffy self integrals stay
// FP64, with a reciprocal square root refined from an FP32 seed (rsqrt_nr).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "assemble.cuh"
#include "bem/utils/quadrature.hpp"
#include "common.cuh"

namespace sqbem {

// ---------------------------------------------------------------- tables
struct QPoint {
    double l0, l1, l2, w;
};
struct QPointF {
    float l0, l1, l2, w;
};
__host__ __device__ constexpr int rule_off(int r) { return r <= 0 ? 0 : r == 1 ? 7 : r == 2 ? 35 : r == 3 ? 147 : 595; }
__device__ QPoint d_rule[595];
__device__ QPointF d_rulef[595];
__constant__ QPoint c_rule7[7];
__constant__ QPointF c_rule7f[7];
__device__ double d_gl_x[10], d_gl_w[10];
__device__ QPoint d_duffy[100];  // (x_a, x_b, w_a * w_b) for the 10 x 10 GL grid

static std::once_flag g_table_once[64];

void init_tables() {
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) fail(SQBEM_ERR_ARG, "device ordinal %d out of range", dev);
    std::call_once(g_table_once[dev], [] {
        std::vector<QPoint> h;
        std::vector<QPointF> hf;
        for (const auto& R : bem::rules())
            for (size_t q = 0; q < R.W.size(); ++q) {
                h.push_back({R.L[q][0], R.L[q][1], R.L[q][2], R.W[q]});
                hf.push_back({(float)R.L[q][0], (float)R.L[q][1], (float)R.L[q][2], (float)R.W[q]});
            }
        if (h.size() != 595) fail(SQBEM_ERR_ARG, "quadrature table has %zu points", h.size());
        CUDA_CHECK(cudaMemcpyToSymbol(d_rule, h.data(), sizeof(QPoint) * 595));
        CUDA_CHECK(cudaMemcpyToSymbol(d_rulef, hf.data(), sizeof(QPointF) * 595));
        CUDA_CHECK(cudaMemcpyToSymbol(c_rule7, h.data(), sizeof(QPoint) * 7));
        CUDA_CHECK(cudaMemcpyToSymbol(c_rule7f, hf.data(), sizeof(QPointF) * 7));
        std::vector<double> gx, gw;
        bem::gauss_legendre01(10, gx, gw);
        CUDA_CHECK(cudaMemcpyToSymbol(d_gl_x, gx.data(), sizeof(double) * 10));
        CUDA_CHECK(cudaMemcpyToSymbol(d_gl_w, gw.data(), sizeof(double) * 10));
        std::vector<QPoint> duf;
        for (int a = 0; a < 10; ++a)
            for (int b = 0; b < 10; ++b) duf.push_back({gx[a], gx[b], 0.0, gw[a] * gw[b]});
        CUDA_CHECK(cudaMemcpyToSymbol(d_duffy, duf.data(), sizeof(QPoint) * 100));
        CUDA_CHECK(cudaDeviceSynchronize());
    });
}

// ---------------------------------------------------------------- kernel sums
// Unique entries of the two symmetric 3x3 results plus the 1/|r| diagonal term.
template <class T>
struct Acc {
    T dg, sxx, sxy, sxz, syy, syz, szz, dxx, dxy, dxz, dyy, dyz, dzz;
    __device__ void zero() { dg = sxx = sxy = sxz = syy = syz = szz = dxx = dxy = dxz = dyy = dyz = dzz = T(0); }
};

// 1/sqrt(x) in FP64 for the mixed path's near-singular and self integrals: the
// FP32 seed y0 = rsqrtf(x) (relative error e0 below ~2^-21.5, including the
// rounding of x to FP32) refined by one Newton step for f(y) = 1/y^2 - x,
// y1 = y0 (3 - x y0^2) / 2, whose relative error is 1.5 e0^2 + O(e0^3) < 1e-13.
// Four FP64 operations instead of a full-precision FP64 reciprocal square root.
// x is a squared distance between quadrature point and target, far inside the
// FP32 range (and never 0: the Duffy and Gauss points are interior).
__device__ __forceinline__ double rsqrt_nr(double x) {
    const double y = (double)rsqrtf((float)x);
    return y * fma(-0.5 * x * y, y, 1.5);
}

template <bool NR>
__device__ __forceinline__ double rsqrt_t(double x) {
    if constexpr (NR) return rsqrt_nr(x);
    else return rsqrt(x);
}
template <bool NR>
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }

// One quadrature node: accumulate w G(r) and w T(r).m (kernels.hpp:29-40).
// NR: FP64 with rsqrt_nr (the mixed path's FP64 integrals).
template <class T, bool WITH_DL, bool NR = false>
__device__ __forceinline__ void accum(Acc<T>& A, T rx, T ry, T rz, T w, T mx, T my, T mz) {
    const T r2 = rx * rx + ry * ry + rz * rz;
    const T ir = rsqrt_t<NR>(r2);
    const T ir2 = ir * ir;
    const T ir3 = ir * ir2;
    const T s = w * ir3;
    A.dg += w * ir;
    const T sx = s * rx, sy = s * ry, sz = s * rz;
    A.sxx += sx * rx; A.sxy += sx * ry; A.sxz += sx * rz;
    A.syy += sy * ry; A.syz += sy * rz; A.szz += sz * rz;
    if (WITH_DL) {
        const T d = T(-6) * w * (rx * mx + ry * my + rz * mz) * ir3 * ir2;
        const T dx = d * rx, dy = d * ry, dz = d * rz;
        A.dxx += dx * rx; A.dxy += dx * ry; A.dxz += dx * rz;
        A.dyy += dy * ry; A.dyz += dy * rz; A.dzz += dz * rz;
    }
}

template <class T>
__device__ __forceinline__ void warp_reduce(Acc<T>& A) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        A.dg += __shfl_xor_sync(0xffffffffu, A.dg, o);
        A.sxx += __shfl_xor_sync(0xffffffffu, A.sxx, o);
        A.sxy += __shfl_xor_sync(0xffffffffu, A.sxy, o);
        A.sxz += __shfl_xor_sync(0xffffffffu, A.sxz, o);
        A.syy += __shfl_xor_sync(0xffffffffu, A.syy, o);
        A.syz += __shfl_xor_sync(0xffffffffu, A.syz, o);
        A.szz += __shfl_xor_sync(0xffffffffu, A.szz, o);
        A.dxx += __shfl_xor_sync(0xffffffffu, A.dxx, o);
        A.dxy += __shfl_xor_sync(0xffffffffu, A.dxy, o);
        A.dxz += __shfl_xor_sync(0xffffffffu, A.dxz, o);
        A.dyy += __shfl_xor_sync(0xffffffffu, A.dyy, o);
        A.dyz += __shfl_xor_sync(0xffffffffu, A.dyz, o);
        A.dzz += __shfl_xor_sync(0xffffffffu, A.dzz, o);
    }
}

// entry (a, b) of SL or DL from the accumulator
template <class T>
__device__ __forceinline__ T sl_entry(const Acc<T>& A, int a, int b) {
    const int k = a * 3 + b;
    T v = k == 0 ? A.sxx : k == 1 || k == 3 ? A.sxy : k == 2 || k == 6 ? A.sxz
        : k == 4 ? A.syy : k == 5 || k == 7 ? A.syz : A.szz;
    return a == b ? v + A.dg : v;
}
template <class T>
__device__ __forceinline__ T dl_entry(const Acc<T>& A, int a, int b) {
    const int k = a * 3 + b;
    return k == 0 ? A.dxx : k == 1 || k == 3 ? A.dxy : k == 2 || k == 6 ? A.dxz
         : k == 4 ? A.dyy : k == 5 || k == 7 ? A.dyz : A.dzz;
}

// Rule index of kernels.hpp:74-75 evaluated exactly as the reference does:
// d = |c - x0| / h with round-to-nearest products and sums in the reference's
// order (no FMA contraction), IEEE sqrt and division -- so a pair sitting on a
// threshold picks the same rule.
__device__ __forceinline__ int rule_of(const PanelRec& P, double x, double y, double z) {
    const double dx = P.c[0] - x, dy = P.c[1] - y, dz = P.c[2] - z;
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double d = __ddiv_rn(__dsqrt_rn(d2), P.h);
    return d < 0.75 ? 3 : (d < 1.5 ? 2 : (d < 3.0 ? 1 : 0));
}

// ---------------------------------------------------------------- whole-pair integrals
// Sum over one rule's points split across the 32 lanes of a warp (after the
// call every lane holds the complete sums).  FP64 or FP32 evaluation from the
// FP64 relative vertex vectors e_k = V_k - x0.
template <class T, bool NR = false>
__device__ void warp_rule(Acc<T>& A, const PanelRec& P, double x, double y, double z, int rule, int lane) {
    A.zero();
    const T e0x = (T)(P.v[0] - x), e0y = (T)(P.v[1] - y), e0z = (T)(P.v[2] - z);
    const T e1x = (T)(P.v[3] - x), e1y = (T)(P.v[4] - y), e1z = (T)(P.v[5] - z);
    const T e2x = (T)(P.v[6] - x), e2y = (T)(P.v[7] - y), e2z = (T)(P.v[8] - z);
    const T mx = (T)P.n[0], my = (T)P.n[1], mz = (T)P.n[2];
    const T area = (T)P.area;
    const int q0 = rule_off(rule), q1 = rule_off(rule + 1);
    for (int q = q0 + lane; q < q1; q += 32) {
        T l0, l1, l2, w;
        if constexpr (sizeof(T) == 8) {
            const QPoint Q = d_rule[q];
            l0 = Q.l0; l1 = Q.l1; l2 = Q.l2; w = Q.w;
        } else {
            const QPointF Q = d_rulef[q];
            l0 = Q.l0; l1 = Q.l1; l2 = Q.l2; w = Q.w;
        }
        const T rx = l0 * e0x + l1 * e1x + l2 * e2x;
        const T ry = l0 * e0y + l1 * e1y + l2 * e2y;
        const T rz = l0 * e0z + l1 * e1z + l2 * e2z;
        accum<T, true, NR>(A, rx, ry, rz, w * area, mx, my, mz);
    }
    warp_reduce(A);
}

// FP32 evaluation of a 7/28/112-point rule from centroid-relative offsets:
// r = (c - x0) + sum_k l_k (V_k - c).  The FP64 differences and their FP32
// roundings are spread over lanes 0..15 (one value each) and broadcast by
// shuffles, so a pair costs a few FP64 warp instructions instead of a dozen
// per lane (GB300's FP64 pipe runs at about 1/64 of the FP32 rate).
__device__ void warp_rule_f32(Acc<float>& A, const PanelRec* Pg, double x, double y, double z, int rule, int lane) {
    A.zero();
    float val = 0.f;
    if (lane < 9) val = (float)(Pg->v[lane] - Pg->c[lane % 3]);
    else if (lane < 12) val = (float)(Pg->c[lane - 9] - (lane == 9 ? x : lane == 10 ? y : z));
    else if (lane < 15) val = (float)Pg->n[lane - 12];
    else if (lane == 15) val = (float)Pg->area;
    float d[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) d[k] = __shfl_sync(0xffffffffu, val, k);
    const float bx = __shfl_sync(0xffffffffu, val, 9), by = __shfl_sync(0xffffffffu, val, 10),
                bz = __shfl_sync(0xffffffffu, val, 11);
    const float mx = __shfl_sync(0xffffffffu, val, 12), my = __shfl_sync(0xffffffffu, val, 13),
                mz = __shfl_sync(0xffffffffu, val, 14), area = __shfl_sync(0xffffffffu, val, 15);
    const int q0 = rule_off(rule), q1 = rule_off(rule + 1);
    for (int q = q0 + lane; q < q1; q += 32) {
        const QPointF Q = d_rulef[q];
        const float rx = bx + (Q.l0 * d[0] + Q.l1 * d[3] + Q.l2 * d[6]);
        const float ry = by + (Q.l0 * d[1] + Q.l1 * d[4] + Q.l2 * d[7]);
        const float rz = bz + (Q.l0 * d[2] + Q.l1 * d[5] + Q.l2 * d[8]);
        accum<float, true>(A, rx, ry, rz, Q.w * area, mx, my, mz);
    }
    warp_reduce(A);
}

// Duffy self integral (kernels.hpp:50-65): x0 inside the panel; three
// sub-triangles (x0, V_e, V_e+1), x = x0 + u[(1 - v) e1 + v e2], Jacobian u J.
// The edge vectors and J are formed once per sub-triangle; the lanes split its
// 10 x 10 points.
template <bool NR = false>
__device__ void warp_self(Acc<double>& A, const PanelRec& P, double x, double y, double z, int lane) {
    A.zero();
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int f = e == 2 ? 0 : e + 1;
        const double e1x = P.v[3 * e] - x, e1y = P.v[3 * e + 1] - y, e1z = P.v[3 * e + 2] - z;
        const double e2x = P.v[3 * f] - x, e2y = P.v[3 * f + 1] - y, e2z = P.v[3 * f + 2] - z;
        const double cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
        const double J = sqrt(cx * cx + cy * cy + cz * cz);
        for (int g = lane; g < 100; g += 32) {
            const QPoint Q = d_duffy[g];
            const double u = Q.l0, v = Q.l1;
            const double rx = u * ((1 - v) * e1x + v * e2x);
            const double ry = u * ((1 - v) * e1y + v * e2y);
            const double rz = u * ((1 - v) * e1z + v * e2z);
            accum<double, false, NR>(A, rx, ry, rz, Q.w * u * J, 0.0, 0.0, 0.0);
        }
    }
    warp_reduce(A);
}

// ---------------------------------------------------------------- near-pair list
// One list of capacity near_cap: the heavy pairs (448-point rule, self
// integral) fill it from the front, the light ones (28/112 points) from the back,
// so the near kernel can take the heavy ones first.  near_count[0], [1]: the
// heavy and light counts; [2]: the near kernel's work counter.  A slot is
// written only while it is inside the list; counts whose sum exceeds the
// capacity mean overflow (the near kernel then does nothing and the host
// fails the call).
template <class TO>
__device__ __forceinline__ void near_append(const BlockJob<TO>& job, int i, int p, int rule) {
    const bool heavy = rule >= 3;
    const int slot = atomicAdd(job.near_count + (heavy ? 0 : 1), 1);
    if (slot < job.near_cap) job.near_list[heavy ? slot : job.near_cap - 1 - slot] = make_int2(i, p | (rule << 28));
}

// ---------------------------------------------------------------- far kernel
constexpr int FAR_TGT = 64;   // targets per CTA (threads)
constexpr int FAR_SRC = 16;   // source panels per CTA

// FP64 mode: one thread per target, the CTA's source panels staged in shared
// memory; the exact rule test per pair, then the 7-point rule in FP64.
template <class TO>
__global__ void __launch_bounds__(FAR_TGT) far_kernel(BlockJob<TO> job) {
    __shared__ PanelRec sp[FAR_SRC];
    const int p0 = blockIdx.y * FAR_SRC;
    const int ns = min(FAR_SRC, job.nS - p0);
    {
        const double* src = reinterpret_cast<const double*>(job.src + p0);
        double* dst = reinterpret_cast<double*>(sp);
        const int nd = ns * (int)(sizeof(PanelRec) / sizeof(double));
        for (int k = threadIdx.x; k < nd; k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    const int i = blockIdx.x * FAR_TGT + threadIdx.x;
    if (i >= job.nT) return;
    const int self_p = job.same_mesh ? i : (job.self_of ? job.self_of[i] : -1);
    const double x = job.tgt[3 * i], y = job.tgt[3 * i + 1], z = job.tgt[3 * i + 2];
    for (int s = 0; s < ns; ++s) {
        const PanelRec& P = sp[s];
        const int p = p0 + s;
        const int rule = p == self_p ? 4 : rule_of(P, x, y, z);
        if (rule != 0) {
            near_append(job, i, p, rule);
            if (job.rule_count) atomicAdd(job.rule_count + rule, 1);
            continue;
        }
        Acc<double> A;
        A.zero();
        const double e0x = P.v[0] - x, e0y = P.v[1] - y, e0z = P.v[2] - z;
        const double e1x = P.v[3] - x, e1y = P.v[4] - y, e1z = P.v[5] - z;
        const double e2x = P.v[6] - x, e2y = P.v[7] - y, e2z = P.v[8] - z;
        const double mx = P.n[0], my = P.n[1], mz = P.n[2], area = P.area;
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const double l0 = c_rule7[q].l0, l1 = c_rule7[q].l1, l2 = c_rule7[q].l2, w = c_rule7[q].w;
            accum<double, true>(A, l0 * e0x + l1 * e1x + l2 * e2x, l0 * e0y + l1 * e1y + l2 * e2y,
                                l0 * e0z + l1 * e1z + l2 * e2z, w * area, mx, my, mz);
        }
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const long long r = 3LL * i + a, c = 3LL * p + b;
                if (job.S) job.S[r * job.s_rs + c * job.s_cs] = (TO)(sl_entry(A, a, b) * job.sscale);
                if (job.D) job.D[r * job.d_rs + c * job.d_cs] = (TO)(dl_entry(A, a, b) * job.dscale);
            }
    }
}

// FP32 view of a source panel for the mixed far field, formed once per block by
// far_prep_kernel: the offsets of the 7 quadrature nodes from the centroid
// (sum_k l_k (V_k - c), formed in FP64 and rounded once), the node weights of
// the single layer (w area) and of the double layer (-6 w area), the normal,
// the centroid as an unevaluated sum hi + lo of two floats, and the squared rule
// thresholds (0.75 h)^2, (1.5 h)^2, (3 h)^2 lowered (thlo) and raised (thhi) by
// 1e-5.  Everything here depends on the source panel only, so the pair loop
// forms a node as (c - x0) + o_q.
struct __align__(16) FarF {
    float o[21];
    float ws[7], wd[7];
    float n[3];
    float chi[3], clo[3];
    float thlo[3], thhi[3];
    float pad[2];
};
static_assert(sizeof(FarF) % 16 == 0, "FarF is copied as float4");

// v = hi + lo with hi = fl32(v) and lo = fl32(v - hi): the pair carries v to
// about 2^-48 relative, so a difference of two such pairs formed in FP32,
// (a_hi - b_hi) + (a_lo - b_lo), is within ~2.5 FP32 ulps of the exact one.
__device__ __forceinline__ void split2(double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// FarF of every source panel and the hi + lo split (x, y, z hi; x, y, z lo) of
// every target: the only FP64 work of the mixed far field.
__global__ void far_prep_kernel(const PanelRec* __restrict__ src, int nS, const double* __restrict__ tgt, int nT,
                                FarF* __restrict__ srcf, float* __restrict__ tgtf) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nS) {
        const PanelRec& P = src[k];
        FarF F;
        double d[9];
        for (int q = 0; q < 9; ++q) d[q] = P.v[q] - P.c[q % 3];
        for (int q = 0; q < 7; ++q) {
            const QPoint& R = c_rule7[q];
            for (int x = 0; x < 3; ++x) F.o[3 * q + x] = (float)(R.l0 * d[x] + R.l1 * d[3 + x] + R.l2 * d[6 + x]);
            F.ws[q] = (float)(R.w * P.area);
            F.wd[q] = (float)(-6.0 * R.w * P.area);
        }
        for (int q = 0; q < 3; ++q) {
            F.n[q] = (float)P.n[q];
            split2(P.c[q], F.chi[q], F.clo[q]);
        }
        const double h2 = P.h * P.h;
        const double t[3] = {0.5625 * h2, 2.25 * h2, 9.0 * h2};
        for (int q = 0; q < 3; ++q) {
            F.thlo[q] = (float)(t[q] * (1.0 - 1e-5));
            F.thhi[q] = (float)(t[q] * (1.0 + 1e-5));
        }
        F.pad[0] = F.pad[1] = 0.f;
        srcf[k] = F;
    }
    if (k < nT)
        for (int q = 0; q < 3; ++q) split2(tgt[3 * k + q], tgtf[6 * k + q], tgtf[6 * k + 3 + q]);
}

// Mixed mode: as far_kernel, all in FP32.  c - x0 comes from the hi + lo pairs
// (relative error <= ~2.5 ulp per component, so d2 is within ~5e-7 of the exact
// value), and the rule from comparing d2 with the thresholds' 1e-5 bands: a
// pair clear of every band has the rule the reference's FP64 test gives; a
// pair inside a band (rare) takes the reference's exact test (rule_of).  The
// near kernel takes the rule from the list.  Near pairs are gathered in a
// shared-memory list first (heavy from the front, light from the back) and
// appended to the global list with one atomic per class at the end of the CTA,
// so no thread waits on a global atomic inside the pair loop.
// SRC: source panels per CTA (FAR_SRC, or fewer for blocks with few targets,
// such as the tube's sector-0 rows, so that the grid still fills the GPU).
template <class TO, int SRC>
__global__ void __launch_bounds__(FAR_TGT, 8) far_kernel_f32(BlockJob<TO> job, const FarF* __restrict__ srcf,
                                                          const float* __restrict__ tgtf) {
    constexpr int FAR_PAIRS = FAR_TGT * SRC;
    __shared__ FarF sf[SRC];
    __shared__ int2 nl[FAR_PAIRS];
    __shared__ int ncount[2], nbase[2], rcount[5];
    const int p0 = blockIdx.y * SRC;
    const int ns = min(SRC, job.nS - p0);
    {
        const float4* s4 = reinterpret_cast<const float4*>(srcf + p0);
        float4* d4 = reinterpret_cast<float4*>(sf);
        const int n4 = ns * (int)(sizeof(FarF) / sizeof(float4));
        for (int k = threadIdx.x; k < n4; k += blockDim.x) d4[k] = s4[k];
    }
    if (threadIdx.x < 2) ncount[threadIdx.x] = 0;
    if (threadIdx.x < 5) rcount[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * FAR_TGT + threadIdx.x;
    const int nsi = i < job.nT ? ns : 0;  // targets past the end take part in the barriers only
    float xh = 0.f, yh = 0.f, zh = 0.f, xl = 0.f, yl = 0.f, zl = 0.f;
    int self_p = -1;
    if (nsi > 0) {
        xh = tgtf[6 * i]; yh = tgtf[6 * i + 1]; zh = tgtf[6 * i + 2];
        xl = tgtf[6 * i + 3]; yl = tgtf[6 * i + 4]; zl = tgtf[6 * i + 5];
        self_p = job.same_mesh ? i : (job.self_of ? job.self_of[i] : -1);
    }
    const float ss = (float)job.sscale, ds = (float)job.dscale;
    // column-major outputs (row stride 1, every block of the mixed path): per
    // target row 3 i the row bases, per pair one column offset
    const bool colmajor = (!job.S || job.s_rs == 1) && (!job.D || job.d_rs == 1);
    const long long scs = job.s_cs, dcs = job.d_cs;
    TO* const Sr = job.S ? job.S + 3LL * i : nullptr;
    TO* const Dr = job.D ? job.D + 3LL * i : nullptr;
    for (int s = 0; s < nsi; ++s) {
        const FarF& F = sf[s];
        const int p = p0 + s;
        const float bx = (F.chi[0] - xh) + (F.clo[0] - xl);
        const float by = (F.chi[1] - yh) + (F.clo[1] - yl);
        const float bz = (F.chi[2] - zh) + (F.clo[2] - zl);
        const float d2 = bx * bx + by * by + bz * bz;
        int rule;
        if (p == self_p) rule = 4;
        else if (d2 > F.thhi[2]) rule = 0;
        else if (d2 < F.thlo[2] && d2 > F.thhi[1]) rule = 1;
        else if (d2 < F.thlo[1] && d2 > F.thhi[0]) rule = 2;
        else if (d2 < F.thlo[0]) rule = 3;
        else rule = rule_of(job.src[p], job.tgt[3 * i], job.tgt[3 * i + 1], job.tgt[3 * i + 2]);
        if (rule != 0) {
            const bool heavy = rule >= 3;
            const int slot = atomicAdd(&ncount[heavy ? 0 : 1], 1);  // at most FAR_PAIRS in total
            nl[heavy ? slot : FAR_PAIRS - 1 - slot] = make_int2(i, p | (rule << 28));
            if (job.rule_count) atomicAdd(&rcount[rule], 1);
            continue;
        }
        Acc<float> A;
        A.zero();
        // r = (c - x0) + o_q; the accumulation of accum<float, true> with the
        // node weights precomputed
        const float mx = F.n[0], my = F.n[1], mz = F.n[2];
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const float rx = bx + F.o[3 * q], ry = by + F.o[3 * q + 1], rz = bz + F.o[3 * q + 2];
            const float r2 = rx * rx + ry * ry + rz * rz;
            const float ir = rsqrtf(r2);
            const float ir2 = ir * ir;
            const float ir3 = ir * ir2;
            const float sw = F.ws[q] * ir3;
            A.dg += F.ws[q] * ir;
            const float sx = sw * rx, sy = sw * ry, sz = sw * rz;
            A.sxx += sx * rx; A.sxy += sx * ry; A.sxz += sx * rz;
            A.syy += sy * ry; A.syz += sy * rz; A.szz += sz * rz;
            const float dd = (F.wd[q] * ir3) * ((rx * mx + ry * my + rz * mz) * ir2);
            const float dx = dd * rx, dy = dd * ry, dz = dd * rz;
            A.dxx += dx * rx; A.dxy += dx * ry; A.dxz += dx * rz;
            A.dyy += dy * ry; A.dyz += dy * rz; A.dzz += dz * rz;
        }
        if (colmajor) {
            // the 3x3 block at base + 3 p ld + a + b ld: one base per pair, the
            // columns b = 1, 2 at the hoisted strides, rows a as immediates
            if (Sr) {
                TO* sp = Sr + 3LL * p * scs;
#pragma unroll
                for (int b = 0; b < 3; ++b)
#pragma unroll
                    for (int a = 0; a < 3; ++a) sp[a + b * scs] = (TO)(sl_entry(A, a, b) * ss);
            }
            if (Dr) {
                TO* dp = Dr + 3LL * p * dcs;
#pragma unroll
                for (int b = 0; b < 3; ++b)
#pragma unroll
                    for (int a = 0; a < 3; ++a) dp[a + b * dcs] = (TO)(dl_entry(A, a, b) * ds);
            }
            continue;
        }
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const long long r = 3LL * i + a, c = 3LL * p + b;
                if (job.S) job.S[r * job.s_rs + c * job.s_cs] = (TO)(sl_entry(A, a, b) * ss);
                if (job.D) job.D[r * job.d_rs + c * job.d_cs] = (TO)(dl_entry(A, a, b) * ds);
            }
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        const int n = ncount[threadIdx.x];
        nbase[threadIdx.x] = n > 0 ? atomicAdd(job.near_count + threadIdx.x, n) : 0;
    }
    if (job.rule_count && threadIdx.x >= 1 && threadIdx.x < 5 && rcount[threadIdx.x] > 0)
        atomicAdd(job.rule_count + threadIdx.x, rcount[threadIdx.x]);
    __syncthreads();
    const int nh = ncount[0], nlt = ncount[1], cap = job.near_cap;
    for (int e = threadIdx.x; e < nh; e += FAR_TGT) {
        const int slot = nbase[0] + e;
        if (slot < cap) job.near_list[slot] = nl[e];
    }
    for (int e = threadIdx.x; e < nlt; e += FAR_TGT) {
        const int slot = nbase[1] + e;
        if (slot < cap) job.near_list[cap - 1 - slot] = nl[FAR_PAIRS - 1 - e];
    }
}

// ---------------------------------------------------------------- near kernel
// Warps take pairs from a shared counter, heavy pairs first (a heavy pair costs
// up to 16x a light one; static striding left SMs idle for a third of the run).
// Each pair is computed whole by one warp, so the result does not depend on the
// order.
template <class TO, bool MIXED>
__global__ void __launch_bounds__(32, 24) near_kernel(BlockJob<TO> job) {
    const int lane = threadIdx.x & 31;
    const int nh = job.near_count[0], nl = job.near_count[1];
    if (nh + nl > job.near_cap) return;  // overflow: reported by the host
    // heavy pairs (448-point rule, self integrals) by warp index: warp g takes
    // g, g + W, ...; one-warp CTAs are dispatched round-robin over the SMs, so
    // consecutive heavy pairs run on different SMs' FP64 pipes (a shared counter
    // hands consecutive tickets to the warps of one SM).  Then the light pairs
    // from the counter.
    const int W = gridDim.x * (blockDim.x >> 5);
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int kh = gw;
    for (;;) {
        int k;
        if (kh < nh) {
            k = kh;
            kh += W;
        } else {
            int t = 0;
            if (lane == 0) t = atomicAdd(job.near_count + 2, 1);
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t >= nl) break;
            k = nh + t;
        }
        const int2 e = job.near_list[k < nh ? k : job.near_cap - 1 - (k - nh)];
        const int i = e.x, p = e.y & 0x0fffffff;
        const PanelRec P = job.src[p];
        const double x = job.tgt[3 * i], y = job.tgt[3 * i + 1], z = job.tgt[3 * i + 2];
        const int rule = e.y >> 28;  // exact rule (4 = self), decided by the far kernel
        double sl = 0, dl = 0;
        const int a = lane / 3, b = lane % 3;
        if (rule == 4) {
            Acc<double> A;
            warp_self<MIXED>(A, P, x, y, z, lane);
            if (lane < 9) { sl = sl_entry(A, a, b); dl = 0.0; }
        } else if (MIXED && rule < 3) {
            Acc<float> A;
            warp_rule_f32(A, job.src + p, x, y, z, rule, lane);
            if (lane < 9) { sl = sl_entry(A, a, b); dl = dl_entry(A, a, b); }
        } else {
            Acc<double> A;
            warp_rule<double, MIXED>(A, P, x, y, z, rule, lane);
            if (lane < 9) { sl = sl_entry(A, a, b); dl = dl_entry(A, a, b); }
        }
        if (lane < 9) {
            const long long r = 3LL * i + a, c = 3LL * p + b;
            if (job.S) job.S[r * job.s_rs + c * job.s_cs] = (TO)(sl * job.sscale);
            if (job.D) job.D[r * job.d_rs + c * job.d_cs] = (TO)(dl * job.dscale);
        }
    }
}

template <class TO>
void assemble_block(const BlockJob<TO>& job0, int near_cap, cudaStream_t st, bool mixed) {
    if (job0.nT <= 0 || job0.nS <= 0) return;
    init_tables();
    BlockJob<TO> job = job0;
    DevBuf<int2> list((size_t)near_cap, st);
    DevBuf<int> count(3, st);
    count.zero();
    job.near_list = list.get();
    job.near_count = count.get();
    job.near_cap = near_cap;
    DevBuf<int> rc;
    if (kstats_on()) {
        rc.alloc(5, st);
        rc.zero();
        job.rule_count = rc.get();
    }
    dim3 grid(ceil_div(job.nT, FAR_TGT), ceil_div(job.nS, FAR_SRC));
    // few target blocks (the tube's sector-0 rows): 4 sources per CTA, 4x the CTAs
    const bool narrow = mixed && (long long)grid.x * grid.y < 2LL * 152 * 4;
    const dim3 grid4(grid.x, ceil_div(job.nS, 4));
    // credited work: every pair considered, at the 7-point rule; bytes written
    const double pairs = (double)job.nT * job.nS;
    const double fl = pairs * 7.0 * FLOPS_PER_EVAL;
    const double by = pairs * 9.0 * sizeof(TO) * ((job.S ? 1 : 0) + (job.D ? 1 : 0));
    if (mixed) {
        DevBuf<FarF> srcf((size_t)job.nS, st);
        DevBuf<float> tgtf((size_t)job.nT * 6, st);
        LAUNCH(far_prep_kernel, ceil_div(std::max(job.nS, job.nT), 128), 128, 0, st, job.src, job.nS, job.tgt, job.nT,
               srcf.get(), tgtf.get());
        if (narrow)
            TIMED_LAUNCH("assemble_far", fl, by, (far_kernel_f32<TO, 4>), grid4, FAR_TGT, 0, st, job, srcf.get(), tgtf.get());
        else
            TIMED_LAUNCH("assemble_far", fl, by, (far_kernel_f32<TO, FAR_SRC>), grid, FAR_TGT, 0, st, job, srcf.get(),
                         tgtf.get());
    } else {
        TIMED_LAUNCH("assemble_far", fl, by, far_kernel<TO>, grid, FAR_TGT, 0, st, job);
    }
    static int sms = 0;
    static std::once_flag sms_once;
    std::call_once(sms_once, [] {
        int dev = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    });
    // 24 one-warp CTAs per SM (80 registers per thread): consecutive pairs of the
    // list -- the heavy 448-point and self pairs come first -- go to warps of
    // different SMs, so they do not queue on a few SMs' FP64 pipes
    const int warps = sms * 24;
    // credited FP64-pipe work of the near kernel (kernel statistics only, which
    // count the pairs per rule on the device): the 448-point rule and the self
    // integral, plus in FP64 mode the 28- and 112-point rules (FP32 in mixed mode)
    if (kstats_on()) {
        int* counts = kstat_pinned_ints(5);
        CUDA_CHECK(cudaMemcpyAsync(counts, rc.get(), 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
        const double w[5] = {0.0, mixed ? 0.0 : 28.0 * FLOPS_PER_EVAL, mixed ? 0.0 : 112.0 * FLOPS_PER_EVAL,
                             448.0 * FLOPS_PER_EVAL, 300.0 * FLOPS_PER_EVAL_SL};
        char note[96];
        std::snprintf(note, sizeof note, "nT=%d nS=%d same=%d mixed=%d", job.nT, job.nS, job.same_mesh, (int)mixed);
        kstat_note(note);
        const int ks = kstat_begin(st);
        if (mixed) LAUNCH((near_kernel<TO, true>), warps, 32, 0, st, job);
        else LAUNCH((near_kernel<TO, false>), warps, 32, 0, st, job);
        kstat_end_counted(ks, "assemble_near", st, counts, w, 5, 0.0);
    } else if (mixed) {
        LAUNCH((near_kernel<TO, true>), warps, 32, 0, st, job);
    } else {
        LAUNCH((near_kernel<TO, false>), warps, 32, 0, st, job);
    }
    if ((long long)job.nT * job.nS > near_cap) {
        // the list could overflow only for blocks larger than its capacity
        int h[3] = {};
        count.download(h, 3);
        CUDA_CHECK(cudaStreamSynchronize(st));
        if ((long long)h[0] + h[1] > near_cap)
            fail(SQBEM_ERR_ARG, "near-pair list overflow (%lld > %d)", (long long)h[0] + h[1], near_cap);
    }
}

template void assemble_block<double>(const BlockJob<double>&, int, cudaStream_t, bool);
template void assemble_block<float>(const BlockJob<float>&, int, cudaStream_t, bool);

// ---------------------------------------------------------------- row sums
// partial[chunk][row][b] = sum over source panels p in the chunk of D(row, 3p + b).
// FP64 blocks are summed in FP64.  FP32 blocks are summed in FP32 pairs: each
// entry enters through an error-free TwoSum (the rounding error of every
// addition kept in a second FP32 sum), so the chunk's (double)s + (double)c is
// accurate to about 2^-48 of the sum of magnitudes -- what an FP64 sum of the
// FP32 entries gives -- at 6 FP32 operations per entry instead of an FP64 add
// (1/64 of the FP32 rate on GB300, which made this kernel FP64-bound).
__device__ __forceinline__ void two_sum_f(float& s, float& c, float x) {
    const float t = __fadd_rn(s, x);
    const float z = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z)));
    s = t;
}

template <class T>
__global__ void rowsum_kernel(const T* __restrict__ D, long long rs, long long cs, int nrows, int ncolpanels,
                              int chunk, double* __restrict__ partial) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    const int c = blockIdx.y;
    const int p0 = c * chunk, p1 = min(ncolpanels, p0 + chunk);
    double* o = partial + ((long long)c * nrows + row) * 3;
    if constexpr (sizeof(T) == sizeof(float)) {
        float s[3] = {0.f, 0.f, 0.f}, e[3] = {0.f, 0.f, 0.f};
#pragma unroll 4
        for (int p = p0; p < p1; ++p) {
            const long long base = row * rs + 3LL * p * cs;
            const float d0 = __ldg(D + base), d1 = __ldg(D + base + cs), d2 = __ldg(D + base + 2 * cs);
            two_sum_f(s[0], e[0], d0);
            two_sum_f(s[1], e[1], d1);
            two_sum_f(s[2], e[2], d2);
        }
        for (int b = 0; b < 3; ++b) o[b] = (double)s[b] + (double)e[b];
    } else {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int p = p0; p < p1; ++p) {
            const long long base = row * rs + 3LL * p * cs;
            s0 += (double)D[base];
            s1 += (double)D[base + cs];
            s2 += (double)D[base + 2 * cs];
        }
        o[0] = s0; o[1] = s1; o[2] = s2;
    }
}

// Add the chunked row sums (fixed order) to out[row * 3 + b]
__global__ void rowsum_finish(const double* __restrict__ partial, int nchunk, int nrows, double* __restrict__ out) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrows) return;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int c = 0; c < nchunk; ++c) {
        const double* o = partial + ((long long)c * nrows + row) * 3;
        s0 += o[0]; s1 += o[1]; s2 += o[2];
    }
    out[row * 3] += s0;
    out[row * 3 + 1] += s1;
    out[row * 3 + 2] += s2;
}

template <class T>
void add_rowsums(const T* D, long long rs, long long cs, int nrows, int ncolpanels, double* out, cudaStream_t st) {
    if (nrows <= 0 || ncolpanels <= 0) return;
    const int chunk = 32;  // panels per CTA column: many CTAs, so the loads overlap
    const int nchunk = ceil_div(ncolpanels, chunk);
    DevBuf<double> part((size_t)nchunk * nrows * 3, st);
    LAUNCH(rowsum_kernel<T>, dim3(ceil_div(nrows, 128), nchunk), 128, 0, st, D, rs, cs, nrows, ncolpanels, chunk,
           part.get());
    LAUNCH(rowsum_finish, ceil_div(nrows, 128), 128, 0, st, part.get(), nchunk, nrows, out);
}
template void add_rowsums<double>(const double*, long long, long long, int, int, double*, cudaStream_t);
template void add_rowsums<float>(const float*, long long, long long, int, int, double*, cudaStream_t);

// A(3i+a, 3i+b) -= rsum[(3i+a)*3 + b] (+ ext * delta_ab) for columns b with
// colmask bit b of mask[i] set (all three when mask == nullptr).
template <class T>
__global__ void diag_complete_kernel(T* A, long long rs, long long cs, int n, const double* __restrict__ rsum,
                                     double ext, const unsigned char* __restrict__ mask) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 9 * n) return;
    const int i = t / 9, a = (t % 9) / 3, b = t % 3;
    if (mask && !((mask[i] >> b) & 1)) return;
    const long long r = 3LL * i + a, c = 3LL * i + b;
    const double v = (double)A[r * rs + c * cs] - rsum[r * 3 + b] - (a == b ? ext : 0.0);
    A[r * rs + c * cs] = (T)v;
}

template <class T>
void diag_complete(T* A, long long rs, long long cs, int n, const double* rsum, double ext,
                   const unsigned char* mask, cudaStream_t st) {
    if (n <= 0) return;
    LAUNCH(diag_complete_kernel<T>, ceil_div(9LL * n, 256), 256, 0, st, A, rs, cs, n, rsum, ext, mask);
}
template void diag_complete<double>(double*, long long, long long, int, const double*, double,
                                    const unsigned char*, cudaStream_t);
template void diag_complete<float>(float*, long long, long long, int, const double*, double,
                                   const unsigned char*, cudaStream_t);

// ---------------------------------------------------------------- panel integrals (API)
__global__ void pairs_kernel(int n, const PanelRec* __restrict__ P, const double* __restrict__ x0,
                             const int* __restrict__ self, double* SL, double* DL) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp >= n) return;
    const PanelRec R = P[warp];
    const double x = x0[3 * warp], y = x0[3 * warp + 1], z = x0[3 * warp + 2];
    Acc<double> A;
    const bool is_self = self[warp] != 0;
    if (is_self) warp_self(A, R, x, y, z, lane);
    else warp_rule<double>(A, R, x, y, z, rule_of(R, x, y, z), lane);
    if (lane < 9) {
        const int a = lane / 3, b = lane % 3;
        SL[9 * warp + lane] = sl_entry(A, a, b);
        DL[9 * warp + lane] = is_self ? 0.0 : dl_entry(A, a, b);
    }
}

void panel_pairs(int n, const PanelRec* P, const double* x0, const int* self, double* SL, double* DL,
                 cudaStream_t st) {
    if (n <= 0) return;
    init_tables();
    LAUNCH(pairs_kernel, ceil_div(32LL * n, 256), 256, 0, st, n, P, x0, self, SL, DL);
}

// ---------------------------------------------------------------- field
// u_j(x0) = sum_p [SL_p,ij f_p,i / (8 pi mu) - DL_p,ij u_p,i / (8 pi)]  (field.hpp:18-34)
// One warp per point: pass 1, the lanes take the panels round-robin and apply the
// 7-point rule to far panels while near panels (d < 3) are collected in shared
// memory; pass 2, the whole warp integrates each near panel (lanes split the
// rule points).  Fixed order, hence deterministic.
constexpr int FIELD_WARPS = 4;
constexpr int FIELD_NEAR_CAP = 256;

template <class TC>
__global__ void __launch_bounds__(FIELD_WARPS * 32) field_kernel(FieldJob job) {
    __shared__ int near_p[FIELD_WARPS][FIELD_NEAR_CAP];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int pt = blockIdx.x * FIELD_WARPS + wl;
    if (pt >= job.npts) return;
    const double x = job.pts[3 * pt], y = job.pts[3 * pt + 1], z = job.pts[3 * pt + 2];
    double ux = 0, uy = 0, uz = 0;
    int nnear = 0;
    int overflow = 0;
    for (int base = 0; base < job.P; base += 32) {
        const int p = base + lane;
        int rule = -1;
        PanelRec P;
        if (p < job.P) {
            P = job.panels[p];
            rule = rule_of(P, x, y, z);
        }
        const unsigned nearmask = __ballot_sync(0xffffffffu, rule > 0);
        if (rule > 0) {
            const int slot = nnear + __popc(nearmask & ((1u << lane) - 1));
            if (slot < FIELD_NEAR_CAP) near_p[wl][slot] = p;
        }
        nnear += __popc(nearmask);
        if (rule == 0) {
            Acc<TC> A;
            A.zero();
            const TC e0x = (TC)(P.v[0] - x), e0y = (TC)(P.v[1] - y), e0z = (TC)(P.v[2] - z);
            const TC e1x = (TC)(P.v[3] - x), e1y = (TC)(P.v[4] - y), e1z = (TC)(P.v[5] - z);
            const TC e2x = (TC)(P.v[6] - x), e2y = (TC)(P.v[7] - y), e2z = (TC)(P.v[8] - z);
            const TC mx = (TC)P.n[0], my = (TC)P.n[1], mz = (TC)P.n[2], area = (TC)P.area;
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                TC l0, l1, l2, w;
                if constexpr (sizeof(TC) == 8) {
                    l0 = c_rule7[q].l0; l1 = c_rule7[q].l1; l2 = c_rule7[q].l2; w = c_rule7[q].w;
                } else {
                    l0 = c_rule7f[q].l0; l1 = c_rule7f[q].l1; l2 = c_rule7f[q].l2; w = c_rule7f[q].w;
                }
                accum<TC, true>(A, l0 * e0x + l1 * e1x + l2 * e2x, l0 * e0y + l1 * e1y + l2 * e2y,
                                l0 * e0z + l1 * e1z + l2 * e2z, w * area, mx, my, mz);
            }
            const double* f = job.f + 3 * p;
            const double* u = job.u + 3 * p;
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int i = 0; i < 3; ++i)
                    s += (double)sl_entry(A, i, j) * f[i] * job.sscale + (double)dl_entry(A, i, j) * u[i] * job.dscale;
                (j == 0 ? ux : j == 1 ? uy : uz) += s;
            }
        }
    }
    if (nnear > FIELD_NEAR_CAP) overflow = 1;
    __syncwarp();
    // warp-reduce the far part (fixed butterfly order)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ux += __shfl_xor_sync(0xffffffffu, ux, o);
        uy += __shfl_xor_sync(0xffffffffu, uy, o);
        uz += __shfl_xor_sync(0xffffffffu, uz, o);
    }
    const int nn = min(nnear, FIELD_NEAR_CAP);
    for (int k = 0; k < nn; ++k) {
        const int p = near_p[wl][k];
        const PanelRec P = job.panels[p];
        const int rule = rule_of(P, x, y, z);
        double sl[9], dl[9];
        if (job.mixed && rule < 3) {
            Acc<float> A;
            warp_rule_f32(A, job.panels + p, x, y, z, rule, lane);
            for (int q = 0; q < 9; ++q) { sl[q] = sl_entry(A, q / 3, q % 3); dl[q] = dl_entry(A, q / 3, q % 3); }
        } else {
            Acc<double> A;
            if (job.mixed) warp_rule<double, true>(A, P, x, y, z, rule, lane);
            else warp_rule<double, false>(A, P, x, y, z, rule, lane);
            for (int q = 0; q < 9; ++q) { sl[q] = sl_entry(A, q / 3, q % 3); dl[q] = dl_entry(A, q / 3, q % 3); }
        }
        const double* f = job.f + 3 * p;
        const double* u = job.u + 3 * p;
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int i = 0; i < 3; ++i) s += sl[3 * i + j] * f[i] * job.sscale + dl[3 * i + j] * u[i] * job.dscale;
            (j == 0 ? ux : j == 1 ? uy : uz) += s;
        }
    }
    if (lane == 0) {
        job.out[3 * pt] = ux;
        job.out[3 * pt + 1] = uy;
        job.out[3 * pt + 2] = uz;
        if (overflow) atomicExch(job.overflow, 1);
    }
}

__global__ void rsqrt_nr_kernel(int n, const double* __restrict__ x, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = rsqrt_nr(x[i]);
}

void rsqrt_nr_eval(int n, const double* x, double* y, cudaStream_t st) {
    if (n > 0) LAUNCH(rsqrt_nr_kernel, ceil_div(n, 256), 256, 0, st, n, x, y);
}

void field_eval(const FieldJob& job, cudaStream_t st) {
    if (job.npts <= 0) return;
    init_tables();
    if (job.mixed) LAUNCH(field_kernel<float>, ceil_div(job.npts, FIELD_WARPS), FIELD_WARPS * 32, 0, st, job);
    else LAUNCH(field_kernel<double>, ceil_div(job.npts, FIELD_WARPS), FIELD_WARPS * 32, 0, st, job);
}

}  // namespace sqbem

// ---------------------------------------------------------------- adjoint contraction
namespace sqbem {

constexpr int ADJ_TT = 32;   // targets per CTA (one per lane)
constexpr int ADJ_ST = 32;   // source panels per CTA (staged in shared memory)
constexpr int ADJ_OUT = 6 * ADJ_MAX_MODES * 3;

// Gradients with respect to r of  phi_G = lam.G(r).f = (lam.f)/|r| + (lam.r)(f.r)/|r|^3
//   grad phi_G = [lam (f.r) + f (lam.r) - (lam.f) r] / |r|^3 - 3 (lam.r)(f.r) r / |r|^5
// and of phi_T = lam.(T(r).m).v = -6 (r.m)(lam.r)(v.r) / |r|^5
//   grad phi_T = -6 [m (lam.r)(v.r) + lam (r.m)(v.r) + v (r.m)(lam.r)] / |r|^5
//                + 30 (r.m)(lam.r)(v.r) r / |r|^7
// (kernels.hpp:8-9 differentiated), accumulated with the weights gs w, ts w.
__global__ void __launch_bounds__(6 * ADJ_TT) adjoint_pairs_kernel(AdjTerm J, int nm, double* partial) {
    __shared__ PanelRec sp[ADJ_ST];
    __shared__ double sf[ADJ_ST][ADJ_MAX_MODES][3];
    __shared__ double sv[ADJ_ST][ADJ_MAX_MODES][3];
    const int tid = threadIdx.x, o = tid / ADJ_TT, lt = tid % ADJ_TT;
    const int t = blockIdx.x * ADJ_TT + lt;
    const int s0 = blockIdx.y * ADJ_ST, ns = min(ADJ_ST, J.nS - s0);
    {
        const double* srcd = reinterpret_cast<const double*>(J.src + s0);
        double* dstd = reinterpret_cast<double*>(sp);
        for (int e = tid; e < ns * 18; e += blockDim.x) dstd[e] = srcd[e];
        for (int e = tid; e < ns * ADJ_MAX_MODES * 3; e += blockDim.x) {
            const int s = e / (ADJ_MAX_MODES * 3), j = (e / 3) % ADJ_MAX_MODES, a = e % 3;
            sf[s][j][a] = j < nm ? J.f[3 * (long long)(s0 + s) + a + j * J.f_ld] : 0.0;
            sv[s][j][a] = (J.v_src && j < nm) ? J.v[3 * (long long)(s0 + s) + a + j * J.v_ld] : 0.0;
        }
    }
    __syncthreads();
    double acc[ADJ_MAX_MODES][3];
#pragma unroll
    for (int j = 0; j < ADJ_MAX_MODES; ++j) acc[j][0] = acc[j][1] = acc[j][2] = 0.0;
    if (t < J.nT) {
        const double x = J.tgt[3 * t], y = J.tgt[3 * t + 1], z = J.tgt[3 * t + 2];
        const double* lp = J.lam + 3 * (long long)t + o * J.lam_ld;
        const double lx = lp[0], ly = lp[1], lz = lp[2];
        double tv[ADJ_MAX_MODES][3];
#pragma unroll
        for (int j = 0; j < ADJ_MAX_MODES; ++j)
#pragma unroll
            for (int a = 0; a < 3; ++a) tv[j][a] = (!J.v_src && j < nm) ? J.v[3 * (long long)t + a + j * J.v_ld] : 0.0;
        for (int s = 0; s < ns; ++s) {
            const PanelRec& P = sp[s];
            const int rule = rule_of(P, x, y, z);
            const double e0x = P.v[0] - x, e0y = P.v[1] - y, e0z = P.v[2] - z;
            const double e1x = P.v[3] - x, e1y = P.v[4] - y, e1z = P.v[5] - z;
            const double e2x = P.v[6] - x, e2y = P.v[7] - y, e2z = P.v[8] - z;
            const double mx = P.n[0], my = P.n[1], mz = P.n[2];
            double fv[ADJ_MAX_MODES][3], vv[ADJ_MAX_MODES][3], lf[ADJ_MAX_MODES];
#pragma unroll
            for (int j = 0; j < ADJ_MAX_MODES; ++j) {
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    fv[j][a] = sf[s][j][a];
                    vv[j][a] = J.v_src ? sv[s][j][a] : tv[j][a];
                }
                lf[j] = lx * fv[j][0] + ly * fv[j][1] + lz * fv[j][2];
            }
            const int q0 = rule_off(rule), q1 = rule_off(rule + 1);
            for (int q = q0; q < q1; ++q) {
                const QPoint Q = d_rule[q];
                const double rx = Q.l0 * e0x + Q.l1 * e1x + Q.l2 * e2x;
                const double ry = Q.l0 * e0y + Q.l1 * e1y + Q.l2 * e2y;
                const double rz = Q.l0 * e0z + Q.l1 * e1z + Q.l2 * e2z;
                const double w = Q.w * P.area;
                const double r2 = rx * rx + ry * ry + rz * rz;
                const double ir = rsqrt(r2), ir2 = ir * ir, ir3 = ir * ir2, ir5 = ir3 * ir2, ir7 = ir5 * ir2;
                const double sm = rx * mx + ry * my + rz * mz;
                const double sl = rx * lx + ry * ly + rz * lz;
                const double wg = w * J.gs, wt = w * J.ts;
#pragma unroll
                for (int j = 0; j < ADJ_MAX_MODES; ++j) {
                    if (j >= nm) break;
                    const double sfj = rx * fv[j][0] + ry * fv[j][1] + rz * fv[j][2];
                    const double svj = rx * vv[j][0] + ry * vv[j][1] + rz * vv[j][2];
                    // grad phi_G = (lam sf + f sl - lf r) ir3 + cg r
                    const double cg = -3.0 * sl * sfj * ir5;
                    // grad phi_T = -6 ir5 (m sl sv + lam sm sv + v sm sl) + ct r
                    const double a1 = sl * svj, a2 = sm * svj, a3 = sm * sl;
                    const double ct = 30.0 * a3 * svj * ir7, m6 = -6.0 * ir5;
                    const double gx = (lx * sfj + fv[j][0] * sl - lf[j] * rx) * ir3 + cg * rx;
                    const double gy = (ly * sfj + fv[j][1] * sl - lf[j] * ry) * ir3 + cg * ry;
                    const double gz = (lz * sfj + fv[j][2] * sl - lf[j] * rz) * ir3 + cg * rz;
                    const double tx = m6 * (mx * a1 + lx * a2 + vv[j][0] * a3) + ct * rx;
                    const double ty = m6 * (my * a1 + ly * a2 + vv[j][1] * a3) + ct * ry;
                    const double tz = m6 * (mz * a1 + lz * a2 + vv[j][2] * a3) + ct * rz;
                    acc[j][0] += wg * gx + wt * tx;
                    acc[j][1] += wg * gy + wt * ty;
                    acc[j][2] += wg * gz + wt * tz;
                }
            }
        }
    }
    // the 32 lanes of a warp share o: reduce over targets, lane 0 writes
#pragma unroll
    for (int j = 0; j < ADJ_MAX_MODES; ++j)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            double v = acc[j][a];
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
            acc[j][a] = v;
        }
    if (lt == 0) {
        const long long cta = blockIdx.x + (long long)gridDim.x * blockIdx.y;
        double* out = partial + cta * ADJ_OUT + o * ADJ_MAX_MODES * 3;
#pragma unroll
        for (int j = 0; j < ADJ_MAX_MODES; ++j)
#pragma unroll
            for (int a = 0; a < 3; ++a) out[j * 3 + a] = acc[j][a];
    }
}

// out[k] = sum over the ncta partial records, in order
__global__ void adjoint_reduce_kernel(const double* __restrict__ partial, long long ncta, double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= ADJ_OUT) return;
    double s = 0.0;
    for (long long c = 0; c < ncta; ++c) s += partial[c * ADJ_OUT + k];
    out[k] = s;
}

void adjoint_pairs(const AdjTerm* terms, int nterms, int nm, double* out, cudaStream_t st) {
    if (nm < 1 || nm > ADJ_MAX_MODES) fail(SQBEM_ERR_ARG, "adjoint_pairs: %d solutions (at most %d)", nm, ADJ_MAX_MODES);
    init_tables();
    long long total = 0;
    for (int k = 0; k < nterms; ++k)
        total += (long long)ceil_div(terms[k].nT, ADJ_TT) * ceil_div(terms[k].nS, ADJ_ST);
    DevBuf<double> partial((size_t)std::max<long long>(total, 1) * ADJ_OUT, st);
    partial.zero();
    long long off = 0;
    for (int k = 0; k < nterms; ++k) {
        const AdjTerm& J = terms[k];
        if (J.nT <= 0 || J.nS <= 0) continue;
        const dim3 grid(ceil_div(J.nT, ADJ_TT), ceil_div(J.nS, ADJ_ST));
        // far-rule estimate: per node and adjoint vector 54 + 81 nm flops
        const double fl = (double)J.nT * J.nS * 7.0 * 6.0 * (54.0 + 81.0 * nm);
        const double by = (double)J.nS * sizeof(PanelRec) * grid.x + (double)J.nT * 8.0 * 3.0 * 7.0;
        TIMED_LAUNCH("adjoint_pairs", fl, by, adjoint_pairs_kernel, grid, 6 * ADJ_TT, 0, st, J, nm,
                     partial.get() + off * ADJ_OUT);
        off += (long long)grid.x * grid.y;
    }
    LAUNCH(adjoint_reduce_kernel, 1, 64, 0, st, partial.get(), total, out);
}

}  // namespace sqbem
