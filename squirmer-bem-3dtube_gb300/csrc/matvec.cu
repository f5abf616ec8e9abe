// matvec.cu -- grouped FP64-accumulated matrix-vector products and helpers.
//
// matvec: one thread per row, columns split into chunks of MV_CHUNK across
// blockIdx.y (coalesced column-major reads, the vector chunk staged in shared
// memory); chunk partial sums land in a scratch array and are added in chunk
// order by a second kernel, so the result does not depend on scheduling.
//
// FP32 matrices: GB300's FP64 pipe (about 1/64 of the FP32 rate) would bound an
// FP64 multiply-add per element far below HBM speed, so the FP32 x FP64 products
// are accumulated in FP32 pairs instead: x = xh + xl (two FP32 parts), and per
// element the compensated dot product of Ogita, Rump and Oishi ("Dot2", SIAM J.
// Sci. Comput. 26, 2005): TwoProduct by FMA, TwoSum of the running sum, the
// errors and a * xl gathered in a second FP32 accumulator.  The chunk result
// (double)s + (double)c is as accurate as a sum formed in twice the FP32
// precision, close to FP64 for the residuals of the refinement.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "common.cuh"
#include "matvec.cuh"

namespace sqbem {

namespace {

constexpr int MV_ROWS = 128;
#ifndef SQBEM_MV_CHUNK
#define SQBEM_MV_CHUNK 128
#endif
#ifndef SQBEM_MV_BATCH
#define SQBEM_MV_BATCH 8
#endif
constexpr int MV_CHUNK = SQBEM_MV_CHUNK;
constexpr int MV_BATCH = SQBEM_MV_BATCH;  // matrix loads issued together before their products
constexpr int MV_RMAX = 8;

constexpr int MAXJOBS = 48;
struct MvDev {
    MvJob j;
    long long part_off;  // offset of this job's partials in the scratch
    int nchunk;
    int rstride;         // partials per row (= r)
};
struct MvArgs {
    int n;
    MvDev j[MAXJOBS];
};
struct CopyArgs {
    int n;
    CopyJob j[MAXJOBS];
};
struct NormArgs {
    int n;
    NormJob j[MAXJOBS];
};

// compensated FP32 multiply-accumulate: (s, c) += a * (xh + xl).  The error-free
// transformations use the _rn intrinsics, which the compiler never fuses into
// multiply-adds (a fused s + a * xh would break TwoSum's exactness).
__device__ __forceinline__ void dot2_step(float& s, float& c, float a, float xh, float xl) {
    const float p = __fmul_rn(a, xh);
    const float e = __fmaf_rn(a, xh, -p);  // exact: a * xh = p + e
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));  // exact: s + p = t + err
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
    c = __fmaf_rn(a, xl, c);
}

// PLAIN: one FP32 multiply-add per element and column (x rounded to FP32),
// accumulated in FP32 within the chunk; for products whose error only enters a
// correction: preconditioner applications and residual updates r -= A d with a
// small d.  Without the compensation the kernel is HBM-bound, so it keeps
// twice as many loads in flight.
template <int R, bool PLAIN>
__global__ void __launch_bounds__(MV_ROWS) mv_partial32(const __grid_constant__ MvArgs args,
                                                        double* __restrict__ part) {
    constexpr int NB = PLAIN ? 2 * MV_BATCH : MV_BATCH;
    static_assert(MV_CHUNK % NB == 0 && NB % 4 == 0, "matvec chunk must be a multiple of the load batch");
    // the staged vector: xh by column, then (compensated) xl; PLAIN reads four
    // columns per shared-memory load
    __shared__ __align__(16) float xs[R][(PLAIN ? 1 : 2) * MV_CHUNK];
    const int jb = blockIdx.z, c = blockIdx.y;
    const int nchunk = args.j[jb].nchunk;
    if (c >= nchunk) return;
    const float* __restrict__ A = args.j[jb].j.A32;
    const double* __restrict__ X = args.j[jb].j.x;
    const long long lda = args.j[jb].j.lda, ldx = args.j[jb].j.ldx;
    const int m = args.j[jb].j.m, n = args.j[jb].j.n, r = args.j[jb].j.r;
    const long long poff = args.j[jb].part_off;
    const int rstride = args.j[jb].rstride;
    const int j0 = c * MV_CHUNK, nj = min(n, j0 + MV_CHUNK) - j0;
    for (int e = threadIdx.x; e < R * MV_CHUNK; e += MV_ROWS) {
        const int k = e / MV_CHUNK, j = e % MV_CHUNK;
        const double v = (k < r && j < nj) ? X[j0 + j + (long long)k * ldx] : 0.0;
        const float h = (float)v;
        xs[k][j] = h;
        if (!PLAIN) xs[k][MV_CHUNK + j] = (float)(v - (double)h);
    }
    __syncthreads();
    const int row = blockIdx.x * MV_ROWS + threadIdx.x;
    if (row >= m) return;
    float s[R], cc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) s[k] = cc[k] = 0.f;
    const float* a = A + row + (long long)j0 * lda;
    // NB independent loads in flight per thread; entries past the chunk read as
    // 0 (and the staged vector is 0 there), adding nothing.
    for (int j = 0; j < nj; j += NB) {
        float av[NB];
#pragma unroll
        for (int u = 0; u < NB; ++u) av[u] = j + u < nj ? __ldg(a + (long long)(j + u) * lda) : 0.f;
        if (PLAIN) {
#pragma unroll
            for (int u = 0; u < NB; u += 4)
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const float4 q = *reinterpret_cast<const float4*>(&xs[k][j + u]);
                    s[k] = fmaf(av[u], q.x, s[k]);
                    s[k] = fmaf(av[u + 1], q.y, s[k]);
                    s[k] = fmaf(av[u + 2], q.z, s[k]);
                    s[k] = fmaf(av[u + 3], q.w, s[k]);
                }
        } else {
#pragma unroll
            for (int u = 0; u < NB; ++u)
#pragma unroll
                for (int k = 0; k < R; ++k) dot2_step(s[k], cc[k], av[u], xs[k][j + u], xs[k][MV_CHUNK + j + u]);
        }
    }
    double* o = part + poff + ((long long)c * m + row) * rstride;
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (k < r) o[k] = (double)s[k] + (double)cc[k];
}

// PLAIN with two rows per thread: one 8-byte load gives a thread rows 2t and
// 2t + 1 of a column, so a warp reads 256 contiguous bytes per load and the
// load count halves.  Used when every job's base address and leading
// dimension keep those loads 8-byte aligned (checked on the host).
template <int R>
__global__ void __launch_bounds__(MV_ROWS) mv_plain2(const __grid_constant__ MvArgs args, double* __restrict__ part) {
    constexpr int NB = 2 * MV_BATCH;
    static_assert(MV_CHUNK % NB == 0 && NB % 4 == 0, "matvec chunk must be a multiple of the load batch");
    __shared__ __align__(16) float xs[R][MV_CHUNK];
    const int jb = blockIdx.z, c = blockIdx.y;
    const int nchunk = args.j[jb].nchunk;
    if (c >= nchunk) return;
    const float* __restrict__ A = args.j[jb].j.A32;
    const double* __restrict__ X = args.j[jb].j.x;
    const long long lda = args.j[jb].j.lda, ldx = args.j[jb].j.ldx;
    const int m = args.j[jb].j.m, n = args.j[jb].j.n, r = args.j[jb].j.r;
    const long long poff = args.j[jb].part_off;
    const int rstride = args.j[jb].rstride;
    const int j0 = c * MV_CHUNK, nj = min(n, j0 + MV_CHUNK) - j0;
    for (int e = threadIdx.x; e < R * MV_CHUNK; e += MV_ROWS) {
        const int k = e / MV_CHUNK, j = e % MV_CHUNK;
        xs[k][j] = (k < r && j < nj) ? (float)X[j0 + j + (long long)k * ldx] : 0.f;
    }
    __syncthreads();
    const int row = 2 * (blockIdx.x * MV_ROWS + threadIdx.x);
    if (row >= m) return;
    const bool two = row + 1 < m;
    float s0[R], s1[R];
#pragma unroll
    for (int k = 0; k < R; ++k) s0[k] = s1[k] = 0.f;
    const float* a = A + row + (long long)j0 * lda;
    for (int j = 0; j < nj; j += NB) {
        float2 av[NB];
#pragma unroll
        for (int u = 0; u < NB; ++u) {
            const float* p = a + (long long)(j + u) * lda;
            av[u] = j + u < nj ? (two ? __ldg(reinterpret_cast<const float2*>(p)) : make_float2(__ldg(p), 0.f))
                               : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < NB; u += 4)
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const float4 q = *reinterpret_cast<const float4*>(&xs[k][j + u]);
                s0[k] = fmaf(av[u].x, q.x, s0[k]);     s1[k] = fmaf(av[u].y, q.x, s1[k]);
                s0[k] = fmaf(av[u + 1].x, q.y, s0[k]); s1[k] = fmaf(av[u + 1].y, q.y, s1[k]);
                s0[k] = fmaf(av[u + 2].x, q.z, s0[k]); s1[k] = fmaf(av[u + 2].y, q.z, s1[k]);
                s0[k] = fmaf(av[u + 3].x, q.w, s0[k]); s1[k] = fmaf(av[u + 3].y, q.w, s1[k]);
            }
    }
    double* o = part + poff + ((long long)c * m + row) * rstride;
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (k < r) {
            o[k] = (double)s0[k];
            if (two) o[rstride + k] = (double)s1[k];
        }
}

template <int R>
__global__ void __launch_bounds__(MV_ROWS) mv_partial(const __grid_constant__ MvArgs args, double* __restrict__ part) {
    const MvDev& D = args.j[blockIdx.z];
    const MvJob& J = D.j;
    const int row = blockIdx.x * MV_ROWS + threadIdx.x;
    const int c = blockIdx.y;
    if (c >= D.nchunk || row >= J.m) return;
    const int j0 = c * MV_CHUNK, j1 = min(J.n, j0 + MV_CHUNK);
    double s[R];
#pragma unroll
    for (int k = 0; k < R; ++k) s[k] = 0.0;
    const int r = J.r;
    if (J.A32) {
        const float* a = J.A32 + row + (long long)j0 * J.lda;
#pragma unroll 8
        for (int j = j0; j < j1; ++j, a += J.lda) {
            const double v = (double)__ldg(a);
#pragma unroll
            for (int k = 0; k < R; ++k)
                if (k < r) s[k] = fma(v, __ldg(J.x + j + (long long)k * J.ldx), s[k]);
        }
    } else {
        const double* a = J.A64 + row + (long long)j0 * J.lda;
#pragma unroll 4
        for (int j = j0; j < j1; ++j, a += J.lda) {
            const double v = __ldg(a);
#pragma unroll
            for (int k = 0; k < R; ++k)
                if (k < r) s[k] = fma(v, __ldg(J.x + j + (long long)k * J.ldx), s[k]);
        }
    }
    double* o = part + D.part_off + ((long long)c * J.m + row) * D.rstride;
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (k < r) o[k] = s[k];
}

// Jobs with few rows (the six constraint rows F against the sphere unknowns):
// one thread per row would leave each CTA a handful of threads walking MV_CHUNK
// dependent loads.  Here a warp takes a row and MV_WIDE columns, its lanes
// interleaved over the columns, and a shuffle tree adds the lanes' sums (a
// fixed order, so the result does not depend on scheduling).  FP64 products
// and sums whatever the matrix's precision: the work is a few kilobytes.
constexpr int MV_FEW = 32;    // rows at most
constexpr int MV_WIDE = 256;  // columns per CTA: 8 per lane, loaded together
constexpr int MV_FEW_WARPS = 8;
template <int R>
__global__ void __launch_bounds__(32 * MV_FEW_WARPS) mv_few(const __grid_constant__ MvArgs args,
                                                           double* __restrict__ part) {
    const MvDev& D = args.j[blockIdx.z];
    const MvJob& J = D.j;
    const int c = blockIdx.y;
    if (c >= D.nchunk) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int j0 = c * MV_WIDE, j1 = min(J.n, j0 + MV_WIDE);
    const int r = J.r;
    for (int row = w; row < J.m; row += MV_FEW_WARPS) {  // warp-uniform
        double s[R];
#pragma unroll
        for (int k = 0; k < R; ++k) s[k] = 0.0;
        constexpr int PER = MV_WIDE / 32;
        double v[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int j = j0 + lane + 32 * u;
            const long long o = row + (long long)j * J.lda;
            v[u] = j < j1 ? (J.A32 ? (double)__ldg(J.A32 + o) : __ldg(J.A64 + o)) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < R; ++k) {
            if (k >= r) break;
            double xv[PER];
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int j = j0 + lane + 32 * u;
                xv[u] = j < j1 ? __ldg(J.x + j + (long long)k * J.ldx) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < PER; ++u) s[k] = fma(v[u], xv[u], s[k]);
        }
#pragma unroll
        for (int k = 0; k < R; ++k)
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], d);
        if (lane == 0) {
            double* o = part + D.part_off + ((long long)c * J.m + row) * D.rstride;
#pragma unroll
            for (int k = 0; k < R; ++k)
                if (k < r) o[k] = s[k];
        }
    }
}

__global__ void mv_finish(const __grid_constant__ MvArgs args, const double* __restrict__ part) {
    const MvDev& D = args.j[blockIdx.y];
    const MvJob& J = D.j;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= J.m) return;
    for (int k = 0; k < J.r; ++k) {
        double s = 0.0;
        for (int c = 0; c < D.nchunk; ++c) s += part[D.part_off + ((long long)c * J.m + row) * D.rstride + k];
        double* y = J.y + row + (long long)k * J.ldy;
        *y = J.beta == 0.0 ? J.alpha * s : fma(J.alpha, s, J.beta * *y);
    }
}

// ---------------------------------------------------------------- rigid-body columns
// y = A K chunk by chunk (RG_PANELS panels = 3 RG_PANELS columns per CTA column
// block), partial sums per chunk, added in chunk order by rigid_finish.
constexpr int RG_PANELS = 32;
struct RigidDev {
    RigidJob j;
    long long part_off;
    int nchunk;
};
struct RigidArgs {
    int n;
    RigidDev j[MAXJOBS];
};

// error-free s + a -> (s, c): the compensated sum of the translation columns
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float a) {
    const float t = __fadd_rn(s, a);
    const float z = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(a, z)));
    s = t;
}

__global__ void __launch_bounds__(MV_ROWS) rigid_partial(const __grid_constant__ RigidArgs args,
                                                         double* __restrict__ part) {
    // per panel of the chunk: r (hi, lo) for the rotation entries
    __shared__ float rh[RG_PANELS][3], rl[RG_PANELS][3];
    const RigidDev& D = args.j[blockIdx.z];
    const int c = blockIdx.y;
    if (c >= D.nchunk) return;
    const int p0 = c * RG_PANELS, np = min(D.j.np, p0 + RG_PANELS) - p0;
    for (int e = threadIdx.x; e < 3 * RG_PANELS; e += blockDim.x) {
        const int q = e / 3, k = e - 3 * q;
        const double v = q < np ? D.j.rc[3 * (p0 + q) + k] : 0.0;
        const float h = (float)v;
        rh[q][k] = h;
        rl[q][k] = (float)(v - (double)h);
    }
    __syncthreads();
    const int row = blockIdx.x * MV_ROWS + threadIdx.x;
    if (row >= D.j.m) return;
    float s[6], cc[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k] = cc[k] = 0.f;
    const float* a = D.j.A + row + (long long)(3 * p0) * D.j.lda;
    const long long lda = D.j.lda;
    for (int q0 = 0; q0 < np; q0 += 4) {
        float av[12];
#pragma unroll
        for (int u = 0; u < 12; ++u) av[u] = q0 + u / 3 < np ? __ldg(a + (long long)(3 * q0 + u) * lda) : 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u;
            if (q >= np) break;
            const float x = av[3 * u], y = av[3 * u + 1], z = av[3 * u + 2];
            two_sum_acc(s[0], cc[0], x);
            two_sum_acc(s[1], cc[1], y);
            two_sum_acc(s[2], cc[2], z);
            // column 3 (e_x x r): -rz a_y + ry a_z; 4 (e_y x r): rz a_x - rx a_z;
            // 5 (e_z x r): -ry a_x + rx a_y
            dot2_step(s[3], cc[3], y, -rh[q][2], -rl[q][2]);
            dot2_step(s[3], cc[3], z, rh[q][1], rl[q][1]);
            dot2_step(s[4], cc[4], x, rh[q][2], rl[q][2]);
            dot2_step(s[4], cc[4], z, -rh[q][0], -rl[q][0]);
            dot2_step(s[5], cc[5], x, -rh[q][1], -rl[q][1]);
            dot2_step(s[5], cc[5], y, rh[q][0], rl[q][0]);
        }
    }
    double* o = part + D.part_off + ((long long)c * D.j.m + row) * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = (double)s[k] + (double)cc[k];
}

__global__ void rigid_finish(const __grid_constant__ RigidArgs args, const double* __restrict__ part) {
    const RigidDev& D = args.j[blockIdx.y];
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= D.j.m) return;
    for (int k = 0; k < 6; ++k) {
        double t = 0.0;
        for (int c = 0; c < D.nchunk; ++c) t += part[D.part_off + ((long long)c * D.j.m + row) * 6 + k];
        D.j.y[row + (long long)k * D.j.ldy] = t;
    }
}

// blockIdx.x: 256 rows, blockIdx.y: job, blockIdx.z: every gridDim.z-th column
// (no per-element division; consecutive threads walk a column)
__global__ void copy_kernel_g(const __grid_constant__ CopyArgs args) {
    const CopyJob& J = args.j[blockIdx.y];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= J.rows) return;
    const double* s64 = J.s64;
    const float* s32 = J.s32;
    double* d64 = J.d64;
    float* d32 = J.d32;
    const long long lds = J.lds, ldd = J.ldd;
    const double alpha = J.alpha, beta = J.beta;
    if (alpha == 1.0 && beta == 0.0) {  // plain copy / conversion: no FP64 arithmetic
        for (int c = blockIdx.z; c < J.cols; c += gridDim.z) {
            if (s32 && d32) d32[r + c * ldd] = s32[r + c * lds];
            else if (s32) d64[r + c * ldd] = (double)s32[r + c * lds];
            else if (d32) d32[r + c * ldd] = (float)s64[r + c * lds];
            else d64[r + c * ldd] = s64[r + c * lds];
        }
        return;
    }
    for (int c = blockIdx.z; c < J.cols; c += gridDim.z) {
        const double s = s64 ? s64[r + c * lds] : (double)s32[r + c * lds];
        if (d64) {
            double* d = d64 + r + c * ldd;
            *d = beta == 0.0 ? alpha * s : fma(alpha, s, beta * *d);
        } else {
            float* d = d32 + r + c * ldd;
            *d = (float)(beta == 0.0 ? alpha * s : fma(alpha, s, beta * (double)*d));
        }
    }
}

// one block per (job, column): fixed-order tree reduction
__global__ void sumsq_kernel(const __grid_constant__ NormArgs args) {
    __shared__ double red[256];
    const NormJob& J = args.j[blockIdx.y];
    const int c = blockIdx.x;
    if (c >= J.cols) return;
    double s = 0.0;
    for (int r = threadIdx.x; r < J.rows; r += blockDim.x) {
        const double v = J.x[r + (long long)c * J.ldx];
        s = fma(v, v, s);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) J.out[c] = red[0];
}

}  // namespace

static void matvec_launches(const std::vector<MvJob>& jobs, cudaStream_t st);

// Compensated FP32, plain FP32 and FP64 jobs go to separate launches: one job
// of another kind would move the whole launch onto its kernel.
void matvec_group(const std::vector<MvJob>& jobs_in, cudaStream_t st) {
    std::vector<MvJob> j32, j32p, j64;
    for (const MvJob& j : jobs_in)
        if (j.m > 0 && j.r > 0) {
            if (j.r > MV_RMAX) fail(SQBEM_ERR_ARG, "matvec: at most %d right-hand sides", MV_RMAX);
            (j.A32 ? (j.plain ? j32p : j32) : j64).push_back(j);
        }
    matvec_launches(j32, st);
    matvec_launches(j32p, st);
    matvec_launches(j64, st);
}

static void matvec_launches(const std::vector<MvJob>& jobs, cudaStream_t st) {
    for (size_t i0 = 0; i0 < jobs.size(); i0 += MAXJOBS) {
        MvArgs a;
        a.n = (int)std::min<size_t>(MAXJOBS, jobs.size() - i0);
        long long off = 0;
        int maxm = 0, maxc = 0, maxr = 0;
        double bytes = 0;
        bool few = true;
        for (int k = 0; k < a.n; ++k) few = few && jobs[i0 + k].m <= MV_FEW;
        for (int k = 0; k < a.n; ++k) {
            const MvJob& j = jobs[i0 + k];
            a.j[k].j = j;
            a.j[k].nchunk = std::max(1, ceil_div(j.n, few ? MV_WIDE : MV_CHUNK));
            a.j[k].part_off = off;
            a.j[k].rstride = j.r;
            off += (long long)a.j[k].nchunk * j.m * j.r;
            maxr = std::max(maxr, j.r);
            maxm = std::max(maxm, j.m);
            maxc = std::max(maxc, a.j[k].nchunk);
            bytes += (double)j.m * j.n * (j.A32 ? 4 : 8);
        }
        DevBuf<double> part((size_t)off, st);
        const dim3 grid(ceil_div(maxm, MV_ROWS), maxc, (unsigned)a.n);
        bool all32 = true;
        for (int k = 0; k < a.n; ++k) all32 = all32 && a.j[k].j.A32 != nullptr;
        if (kstats_on()) {
            char note[96];
            std::snprintf(note, sizeof note, "jobs=%d m=%d chunks=%d r=%d fp32=%d plain=%d few=%d", a.n, maxm, maxc,
                          maxr, (int)all32, (int)(all32 && a.j[0].j.plain), (int)few);
            kstat_note(note);
        }
        const bool plain = all32 && a.j[0].j.plain;
        // two rows per thread: every base and leading dimension keeps 8-byte loads aligned
        bool pairs_ok = true;
        for (int k = 0; k < a.n && pairs_ok; ++k)
            pairs_ok = a.j[k].j.A32 && ((uintptr_t)a.j[k].j.A32 % 8 == 0) && a.j[k].j.lda % 2 == 0;
        if (few) {
            const dim3 g(1, maxc, (unsigned)a.n);
            if (maxr <= 2) TIMED_LAUNCH("matvec", 0.0, bytes, mv_few<2>, g, 32 * MV_FEW_WARPS, 0, st, a, part.get());
            else TIMED_LAUNCH("matvec", 0.0, bytes, mv_few<MV_RMAX>, g, 32 * MV_FEW_WARPS, 0, st, a, part.get());
        } else if (plain && pairs_ok && maxr <= 2) {
            const dim3 g2(ceil_div(maxm, 2 * MV_ROWS), maxc, (unsigned)a.n);
            TIMED_LAUNCH("matvec", 0.0, bytes, mv_plain2<2>, g2, MV_ROWS, 0, st, a, part.get());
        } else if (plain) {
            if (maxr <= 2) TIMED_LAUNCH("matvec", 0.0, bytes, (mv_partial32<2, true>), grid, MV_ROWS, 0, st, a, part.get());
            else TIMED_LAUNCH("matvec", 0.0, bytes, (mv_partial32<MV_RMAX, true>), grid, MV_ROWS, 0, st, a, part.get());
        } else if (all32) {
            // the compensated sums are FP32-issue-bound, so the column count is a
            // template parameter (2: refinement; 6: the rigid-body columns A_u K)
            if (maxr <= 2) TIMED_LAUNCH("matvec", 0.0, bytes, (mv_partial32<2, false>), grid, MV_ROWS, 0, st, a, part.get());
            else if (maxr <= 6) TIMED_LAUNCH("matvec", 0.0, bytes, (mv_partial32<6, false>), grid, MV_ROWS, 0, st, a, part.get());
            else TIMED_LAUNCH("matvec", 0.0, bytes, (mv_partial32<MV_RMAX, false>), grid, MV_ROWS, 0, st, a, part.get());
        } else if (maxr <= 2) {
            TIMED_LAUNCH("matvec", 0.0, bytes, mv_partial<2>, grid, MV_ROWS, 0, st, a, part.get());
        } else {
            TIMED_LAUNCH("matvec", 0.0, bytes, mv_partial<MV_RMAX>, grid, MV_ROWS, 0, st, a, part.get());
        }
        LAUNCH(mv_finish, dim3(ceil_div(maxm, 128), (unsigned)a.n), 128, 0, st, a, part.get());
    }
}

void rigid_product_group(const std::vector<RigidJob>& jobs_in, cudaStream_t st) {
    std::vector<RigidJob> jobs;
    for (const RigidJob& j : jobs_in)
        if (j.m > 0 && j.np > 0) jobs.push_back(j);
    for (size_t i0 = 0; i0 < jobs.size(); i0 += MAXJOBS) {
        RigidArgs a;
        a.n = (int)std::min<size_t>(MAXJOBS, jobs.size() - i0);
        long long off = 0;
        int maxm = 0, maxc = 0;
        double bytes = 0;
        for (int k = 0; k < a.n; ++k) {
            const RigidJob& j = jobs[i0 + k];
            a.j[k].j = j;
            a.j[k].nchunk = ceil_div(j.np, RG_PANELS);
            a.j[k].part_off = off;
            off += (long long)a.j[k].nchunk * j.m * 6;
            maxm = std::max(maxm, j.m);
            maxc = std::max(maxc, a.j[k].nchunk);
            bytes += 4.0 * j.m * 3.0 * j.np;
        }
        DevBuf<double> part((size_t)off, st);
        TIMED_LAUNCH("matvec", 0.0, bytes, rigid_partial, dim3(ceil_div(maxm, MV_ROWS), maxc, (unsigned)a.n), MV_ROWS, 0,
                     st, a, part.get());
        LAUNCH(rigid_finish, dim3(ceil_div(maxm, 128), (unsigned)a.n), 128, 0, st, a, part.get());
    }
}

void copy_group(const std::vector<CopyJob>& jobs_in, cudaStream_t st) {
    std::vector<CopyJob> jobs;
    for (const CopyJob& j : jobs_in)
        if (j.rows > 0 && j.cols > 0) jobs.push_back(j);
    for (size_t i0 = 0; i0 < jobs.size(); i0 += MAXJOBS) {
        CopyArgs a;
        a.n = (int)std::min<size_t>(MAXJOBS, jobs.size() - i0);
        int mr = 0, mc = 0;
        double bytes = 0;
        for (int k = 0; k < a.n; ++k) {
            a.j[k] = jobs[i0 + k];
            mr = std::max(mr, a.j[k].rows);
            mc = std::max(mc, a.j[k].cols);
            bytes += (double)a.j[k].rows * a.j[k].cols *
                     ((a.j[k].s64 ? 8 : 4) + (a.j[k].d64 ? 8 : 4) * (a.j[k].beta != 0.0 ? 2 : 1));
        }
        const int gz = std::min(mc, 64);
        TIMED_LAUNCH("copy", 0.0, bytes, copy_kernel_g, dim3((unsigned)ceil_div(mr, 256), (unsigned)a.n, (unsigned)gz), 256,
                     0, st, a);
    }
}

void sumsq_group(const std::vector<NormJob>& jobs, cudaStream_t st) {
    for (size_t i0 = 0; i0 < jobs.size(); i0 += MAXJOBS) {
        NormArgs a;
        a.n = (int)std::min<size_t>(MAXJOBS, jobs.size() - i0);
        int mc = 0;
        for (int k = 0; k < a.n; ++k) {
            a.j[k] = jobs[i0 + k];
            mc = std::max(mc, a.j[k].cols);
        }
        if (mc == 0) continue;
        LAUNCH(sumsq_kernel, dim3(mc, (unsigned)a.n), 256, 0, st, a);
    }
}

}  // namespace sqbem
