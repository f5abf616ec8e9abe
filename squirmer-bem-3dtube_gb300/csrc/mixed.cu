// mixed.cu -- recursive LU and triangular solves on the split-BF16 tensor-core
// GEMM, grouped over equally sized matrices (see mixed.cuh).
//
// LU(c0, w)   factors the panel of columns [c0, c0 + w) over rows [c0, n):
//             w = 128: leaf -- the 128 x 128 diagonal block is factored and its
//             triangles inverted in shared memory (diag_kernel), then
//             L21 = A21 U11^{-1} on the tensor cores (certified |L21| <= 1);
//             otherwise LU(left half), U12 = L11^{-1} A12 (TRSM_L), the Schur
//             update A22 -= L21 U12 with K = w/2, and LU(right half).
// TRSM_L/U    solve with the unit-lower / upper factor: leaf X = L^{-1}_b B or
//             U^{-1}_b B with the stored block inverses; otherwise two halves and
//             one GEMM update with K = w/2.
// Operand layouts: the left operand of every GEMM is K-major along rows
// (row-major split copy R), the right operand K-major along columns
// (column-major split copy C); each producer step writes the copies its
// consumers need.  FP32 master values are updated by the GEMM epilogues.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "mixed.cuh"
#include "tc_gemm.cuh"

namespace cg = cooperative_groups;

namespace sqbem {

void MixedLU::alloc(int nt, cudaStream_t st) {
    n_true = nt;
    n = pad128(nt);
    const size_t nn = (size_t)n * n, nb = (size_t)(n / MX_NB) * MX_NB * MX_NB;
    A.alloc(nn, st);
    Rh.alloc(nn, st); Rl.alloc(nn, st);
    Ch.alloc(nn, st); Cl.alloc(nn, st);
    Li.alloc(nb, st); Ui.alloc(nb, st);
    LiRh.alloc(nb, st); LiRl.alloc(nb, st);
    UiRh.alloc(nb, st); UiRl.alloc(nb, st);
    UiCh.alloc(nb, st); UiCl.alloc(nb, st);
    LiCh.alloc(nb, st); LiCl.alloc(nb, st);
}

namespace {

// ---------------------------------------------------------------- conversion
constexpr int MAXJOBS = 64;
struct ConvArgs {
    int n;
    ConvJob j[MAXJOBS];
};

// 32 x 32 tiles through shared memory: the loads run along the source's
// contiguous index and the stores along the destination's, so a conversion that
// also transposes (column-major FP32 -> row-major split) stays coalesced on
// both sides; no 64-bit division per element.
constexpr int CV_T = 32, CV_RY = 8;
__global__ void __launch_bounds__(CV_T * CV_RY) conv_kernel(const __grid_constant__ ConvArgs args) {
    __shared__ float tile[CV_T][CV_T + 1];  // [column in tile][row in tile]
    const ConvJob& J = args.j[blockIdx.y];
    const int rows = J.rows, cols = J.cols;
    const int ntr = (rows + CV_T - 1) / CV_T, ntc = (cols + CV_T - 1) / CV_T;
    const int t = blockIdx.x;
    if (t >= ntr * ntc) return;
    const int r0 = (t % ntr) * CV_T, c0 = (t / ntr) * CV_T;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const float* src = J.src;
    const long long srs = J.s_rs, scs = J.s_cs;
    if (srs == 1) {
#pragma unroll
        for (int k = 0; k < CV_T; k += CV_RY) {
            const int r = r0 + tx, c = c0 + ty + k;
            if (r < rows && c < cols) tile[ty + k][tx] = src[r + (long long)c * scs];
        }
    } else {
#pragma unroll
        for (int k = 0; k < CV_T; k += CV_RY) {
            const int r = r0 + ty + k, c = c0 + tx;
            if (r < rows && c < cols) tile[tx][ty + k] = src[(long long)r * srs + c * scs];
        }
    }
    __syncthreads();
    bf16* const hi = J.hi;
    bf16* const lo = J.lo;
    const long long drs = J.d_rs, dcs = J.d_cs;
#pragma unroll
    for (int k = 0; k < CV_T; k += CV_RY) {
        int r, c;
        float x;
        if (drs == 1) {
            r = r0 + tx; c = c0 + ty + k;
            x = tile[ty + k][tx];
        } else {
            r = r0 + ty + k; c = c0 + tx;
            x = tile[tx][ty + k];
        }
        if (r < rows && c < cols) {
            const long long o = (long long)r * drs + (long long)c * dcs;
            const bf16 h = __float2bfloat16_rn(x);
            hi[o] = h;
            lo[o] = __float2bfloat16_rn(x - __bfloat162float(h));
        }
    }
}

// ---------------------------------------------------------------- diagonal leaf
struct DiagJob {
    float* A;  // the 128 x 128 block, column-major, leading dimension lda
    long long lda;
    float* Li;
    float* Ui;
    bf16 *LiRh, *LiRl, *UiRh, *UiRl, *UiCh, *UiCl, *LiCh, *LiCl;
};

constexpr int DIAG_THREADS = 512;
constexpr int DP = MX_NB + 1;  // padded row of the shared block

__device__ __forceinline__ void put_split(bf16* h, bf16* l, long long i, float x) {
    const bf16 a = __float2bfloat16_rn(x);
    h[i] = a;
    l[i] = __float2bfloat16_rn(x - __bfloat162float(a));
}

// LU of the block without exchanges, flagging |l| > 1 (bit 0) and a zero or
// non-finite pivot (bit 1); then L^{-1} and U^{-1}.  The whole block lives in
// shared memory (with both inverses: 3 x 128 x 129 floats).
//
// LU, blocked right-looking with 16-column panels:
//   diag    warp 0 factors the 16 x 16 diagonal block, a row per lane, the
//           pivot row broadcast by shuffles (no barrier per column);
//   L21     the rows below, one per thread and independent of each other:
//           l_ij = (a_ij - sum_{k<j} l_ik U_kj) / U_jj in registers; the
//           certificate compares |a_ij - sum| with |U_jj| exactly (what partial
//           pivoting compares), the multiplier uses the pivot's reciprocal;
//   U12     at the same time, by other threads: one column per thread solves
//           with the unit-lower 16 x 16 block, the column in registers;
//   A22     rank-16 update in 4 x 4 register tiles: a warp takes 4 rows, a lane
//           4 columns 32 apart (conflict-free loads of the U12 row, broadcasts
//           of the L21 column), half a shared load per multiply-add.
// Inverses: blocked by 16 with 4 x 4 register tiles (see below).
struct DiagArgs {
    int* flag;
    DiagJob j[MAXJOBS];
};

constexpr int DG_PW = 16;  // LU panel width

__global__ void __launch_bounds__(DIAG_THREADS) diag_kernel(const __grid_constant__ DiagArgs args) {
    extern __shared__ float sh[];
    constexpr int N = MX_NB;
    float(*a)[DP] = reinterpret_cast<float(*)[DP]>(sh);
    float(*xl)[DP] = reinterpret_cast<float(*)[DP]>(sh + N * DP);
    float(*xu)[DP] = reinterpret_cast<float(*)[DP]>(sh + 2 * N * DP);
    float* rd = sh + 3 * N * DP;  // 1 / U(r, r)
    float(*tl)[DP] = reinterpret_cast<float(*)[DP]>(sh + 3 * N * DP + N);            // 16 x N scratch (L^{-1})
    float(*tu)[DP] = reinterpret_cast<float(*)[DP]>(sh + 3 * N * DP + N + DG_PW * DP);  // 16 x N scratch (U^{-1})
    const DiagJob& J = args.j[blockIdx.x];
    const int tid = threadIdx.x;
    {
        const float* A = J.A;
        const long long lda = J.lda;
        for (int e = tid; e < N * N; e += DIAG_THREADS) a[e % N][e / N] = A[(e % N) + (e / N) * lda];
    }
    __syncthreads();
    int bad = 0;
    __shared__ float rinv[DG_PW];  // 1 / U(j, j) of the current panel
    for (int c0 = 0; c0 < N; c0 += DG_PW) {
        if (tid < 32) {
            // the 16 x 16 diagonal block by warp 0: lane t keeps row c0 + t in
            // registers; the pivot row travels by shuffles (no barrier)
            const int t = tid;
            float row[DG_PW];
#pragma unroll
            for (int cc = 0; cc < DG_PW; ++cc) row[cc] = t < DG_PW ? a[c0 + t][c0 + cc] : 0.f;
#pragma unroll
            for (int jj = 0; jj < DG_PW; ++jj) {
                const float piv = __shfl_sync(0xffffffffu, row[jj], jj);
                if (t == 0 && !(piv != 0.f && isfinite(piv))) bad |= 2;
                const float rp = 1.f / piv;
                float pr[DG_PW];
#pragma unroll
                for (int cc = jj + 1; cc < DG_PW; ++cc) pr[cc] = __shfl_sync(0xffffffffu, row[cc], jj);
                if (t > jj && t < DG_PW) {
                    const float rj = row[jj];
                    const float l = rj * rp;
                    if (!(fabsf(rj) <= fabsf(piv))) bad |= isfinite(l) ? 1 : 2;
#pragma unroll
                    for (int cc = jj + 1; cc < DG_PW; ++cc) row[cc] = fmaf(-l, pr[cc], row[cc]);
                    row[jj] = l;
                }
            }
            if (t < DG_PW) {
                float d = row[0];
#pragma unroll
                for (int cc = 0; cc < DG_PW; ++cc) {
                    a[c0 + t][c0 + cc] = row[cc];
                    if (cc == t) d = row[cc];
                }
                rinv[t] = 1.f / d;
            }
        }
        __syncthreads();
        if (tid < 128) {
            // L21: rows below the block, one per thread, independent of each other:
            // l_ij = (a_ij - sum_{k<j} l_ik U_kj) / U_jj, certified |numerator| <= |U_jj|
            const int i = c0 + DG_PW + tid;
            if (i < N) {
                float x[DG_PW];
#pragma unroll
                for (int j = 0; j < DG_PW; ++j) x[j] = a[i][c0 + j];
#pragma unroll
                for (int j = 0; j < DG_PW; ++j) {
#pragma unroll
                    for (int k = 0; k < j; ++k) x[j] = fmaf(-x[k], a[c0 + k][c0 + j], x[j]);
                    const float u = a[c0 + j][c0 + j];
                    const float l = x[j] * rinv[j];
                    if (!(fabsf(x[j]) <= fabsf(u))) bad |= isfinite(l) ? 1 : 2;
                    x[j] = l;
                }
#pragma unroll
                for (int j = 0; j < DG_PW; ++j) a[i][c0 + j] = x[j];
            }
        } else if (tid < 256) {
            // U12 = L11^{-1} A12 at the same time, one column per thread, in registers
            const int c = c0 + DG_PW + (tid - 128);
            if (c < N) {
                float x[DG_PW];
#pragma unroll
                for (int r = 0; r < DG_PW; ++r) x[r] = a[c0 + r][c];
#pragma unroll
                for (int r = 1; r < DG_PW; ++r)
#pragma unroll
                    for (int k = 0; k < r; ++k) x[r] = fmaf(-a[c0 + r][c0 + k], x[k], x[r]);
#pragma unroll
                for (int r = 1; r < DG_PW; ++r) a[c0 + r][c] = x[r];
            }
        }
        __syncthreads();
        {  // A22 -= L21 U12 in 4 x 4 tiles: rows i0 .. i0 + 3 per warp, columns c1 + lane + 32 p
            const int m = N - c0 - DG_PW, c1 = c0 + DG_PW;
            const int warp = tid >> 5, lane = tid & 31;
            for (int g = warp; g < m / 4; g += DIAG_THREADS / 32) {
                const int i0 = c1 + 4 * g;
                float acc[4][4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        const int c = c1 + lane + 32 * p;
                        acc[q][p] = c < N ? a[i0 + q][c] : 0.f;
                    }
#pragma unroll
                for (int k = 0; k < DG_PW; ++k) {
                    float lv[4], uv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) lv[q] = a[i0 + q][c0 + k];
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        const int c = c1 + lane + 32 * p;
                        uv[p] = c < N ? a[c0 + k][c] : 0.f;
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(-lv[q], uv[p], acc[q][p]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        const int c = c1 + lane + 32 * p;
                        if (c < N) a[i0 + q][c] = acc[q][p];
                    }
            }
        }
        __syncthreads();
    }
    if (bad) atomicOr(args.flag, bad);
    {
        float* A = J.A;
        const long long lda = J.lda;
        for (int e = tid; e < N * N; e += DIAG_THREADS) A[(e % N) + (e / N) * lda] = a[e % N][e / N];
    }
    for (int r = tid; r < N; r += DIAG_THREADS) rd[r] = 1.f / a[r][r];
    __syncthreads();
    for (int e = tid; e < N * N; e += DIAG_THREADS) {
        const int r = e % N, c = e / N;
        xl[r][c] = r == c ? 1.f : 0.f;
        xu[r][c] = r == c ? rd[r] : 0.f;
    }
    __syncthreads();
    // Inverses, blocked by 16: first the 16 x 16 diagonal blocks (a thread per
    // block column), then one block row at a time as two small GEMMs with 4 x 4
    // register tiles (half a shared load per FMA instead of two):
    //   L^{-1}: X_ij = -X_ii sum_{j <= k < i} L_ik X_kj      (block rows ascending)
    //   U^{-1}: X_ij = -X_ii sum_{i < k <= j} U_ik X_kj      (block rows descending)
    // threads 0-255 form L^{-1}, 256-511 U^{-1}, each half with its own named barrier.
    constexpr int B = DG_PW, NBK = N / DG_PW;
    if (tid < N) {
        const int blk = tid / B, c = tid % B, C = B * blk + c;
        for (int r = c + 1; r < B; ++r) {
            float v = 0.f;
            for (int k = c; k < r; ++k) v = fmaf(a[B * blk + r][B * blk + k], xl[B * blk + k][C], v);
            xl[B * blk + r][C] = -v;
        }
    } else if (tid >= 2 * N && tid < 3 * N) {
        const int blk = (tid - 2 * N) / B, c = (tid - 2 * N) % B, C = B * blk + c;
        for (int r = c - 1; r >= 0; --r) {
            float v = 0.f;
            for (int k = r + 1; k <= c; ++k) v = fmaf(a[B * blk + r][B * blk + k], xu[B * blk + k][C], v);
            xu[B * blk + r][C] = -v * rd[B * blk + r];
        }
    }
    __syncthreads();
    if (tid < 2 * N) {
        const int t = tid, tr = t % 4, tc = t / 4;
        for (int i = 1; i < NBK; ++i) {
            const bool act = t < B * i;  // 16 i tiles of 4 x 4 over the 16 x 16 i block row
            float acc[4][4];
            if (act) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) acc[q][p] = 0.f;
                for (int k = B * ((4 * tc) / B); k < B * i; ++k) {
                    float av[4], xv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) av[q] = a[B * i + 4 * tr + q][k];
#pragma unroll
                    for (int p = 0; p < 4; ++p) xv[p] = xl[k][4 * tc + p];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(av[q], xv[p], acc[q][p]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) tl[4 * tr + q][4 * tc + p] = acc[q][p];
            }
            asm volatile("bar.sync 2, 256;" ::: "memory");
            if (act) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) acc[q][p] = 0.f;
#pragma unroll 4
                for (int s2 = 0; s2 < B; ++s2) {
                    float av[4], xv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) av[q] = xl[B * i + 4 * tr + q][B * i + s2];
#pragma unroll
                    for (int p = 0; p < 4; ++p) xv[p] = tl[s2][4 * tc + p];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(av[q], xv[p], acc[q][p]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) xl[B * i + 4 * tr + q][4 * tc + p] = -acc[q][p];
            }
            asm volatile("bar.sync 2, 256;" ::: "memory");
        }
    } else {
        const int t = tid - 2 * N, tr = t % 4, tc = t / 4;
        for (int i = NBK - 2; i >= 0; --i) {
            const int ncol = N - B * (i + 1);
            const bool act = t < ncol;  // ncol tiles of 4 x 4 over the 16 x ncol block row
            const int col0 = B * (i + 1) + 4 * tc;
            float acc[4][4];
            if (act) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) acc[q][p] = 0.f;
                for (int k = B * (i + 1); k < B * (col0 / B) + B; ++k) {
                    float av[4], xv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) av[q] = a[B * i + 4 * tr + q][k];
#pragma unroll
                    for (int p = 0; p < 4; ++p) xv[p] = xu[k][col0 + p];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(av[q], xv[p], acc[q][p]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) tu[4 * tr + q][col0 + p] = acc[q][p];
            }
            asm volatile("bar.sync 3, 256;" ::: "memory");
            if (act) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) acc[q][p] = 0.f;
#pragma unroll 4
                for (int s2 = 0; s2 < B; ++s2) {
                    float av[4], xv[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) av[q] = xu[B * i + 4 * tr + q][B * i + s2];
#pragma unroll
                    for (int p = 0; p < 4; ++p) xv[p] = tu[s2][col0 + p];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(av[q], xv[p], acc[q][p]);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) xu[B * i + 4 * tr + q][col0 + p] = -acc[q][p];
            }
            asm volatile("bar.sync 3, 256;" ::: "memory");
        }
    }
    __syncthreads();
    for (int e = tid; e < N * N; e += DIAG_THREADS) {
        const int r = e % N, c = e / N;
        J.Li[r + c * N] = xl[r][c];
        J.Ui[r + c * N] = xu[r][c];
        put_split(J.UiCh, J.UiCl, (long long)c * N + r, xu[r][c]);
        put_split(J.LiCh, J.LiCl, (long long)c * N + r, xl[r][c]);
    }
    for (int e = tid; e < N * N; e += DIAG_THREADS) {
        const int r = e / N, c = e % N;  // row-major: consecutive threads along a row
        put_split(J.LiRh, J.LiRl, (long long)r * N + c, xl[r][c]);
        put_split(J.UiRh, J.UiRl, (long long)r * N + c, xu[r][c]);
    }
}

constexpr int DIAG_SMEM = (3 * MX_NB * DP + MX_NB + 2 * DG_PW * DP) * (int)sizeof(float);

void diag_group(const std::vector<DiagJob>& jobs, const MixedCtx& cx) {
    static std::once_flag attr;
    std::call_once(attr, [] {
        CUDA_CHECK(cudaFuncSetAttribute(diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM));
    });
    for (size_t i0 = 0; i0 < jobs.size(); i0 += MAXJOBS) {
        DiagArgs a;
        a.flag = cx.flag;
        const int n = (int)std::min<size_t>(MAXJOBS, jobs.size() - i0);
        for (int k = 0; k < n; ++k) a.j[k] = jobs[i0 + k];
        TIMED_LAUNCH("lu_diag", 0.0, 0.0, diag_kernel, n, DIAG_THREADS, DIAG_SMEM, cx.st, a);
    }
}

// ---------------------------------------------------------------- views
// Left operand: rows [r0, r0 + nr) x columns [c0, c0 + nc) of a row-major split copy.
SplitMat rview(bf16* h, bf16* l, long long ld, int r0, int c0, int nr, int nc) {
    const long long o = (long long)r0 * ld + c0;
    return {h + o, l + o, nr, nc, ld};
}
// Right operand: rows [r0, r0 + nr) (= K) x columns [c0, c0 + nc) (= N) of a
// column-major split copy.
SplitMat cview(bf16* h, bf16* l, long long ld, int r0, int c0, int nr, int nc) {
    const long long o = (long long)c0 * ld + r0;
    return {h + o, l + o, nc, nr, ld};
}

// A target being solved in place: FP32 column-major X plus split copies.
struct Target {
    float* X;
    long long ldx;
    bf16 *Ch, *Cl;  // column-major split (required)
    long long ldc;
    bf16 *Rh, *Rl;  // row-major split (optional)
    long long ldr;
};

void run(std::vector<TcProblem>& P, std::vector<TcOperands>& O, const MixedCtx& cx) {
    if (!P.empty()) tc_gemm(P, O, cx.err, cx.flag, cx.st);
    P.clear();
    O.clear();
}

// TRSM with the unit-lower (lower = true) or upper factor of every member on
// rows [k0, k0 + w), columns [j0, j0 + nc) of its target.
// tri: the right-hand side is lower triangular from column j0 on (the identity
// of an inversion), so in the lower solve column c of X stays zero above row c
// and only columns c < k0 + w (relative to j0: c - j0 < k0 + w) take part.
// wide (the members carry their composed 256-block inverses; scratch: one
// 256 x ncols column-major split plane pair per member): the recursion splits at
// multiples of 256 and its leaves are 256 rows wide -- one conversion and one
// GEMM with K = 256 instead of two 128-row leaves and the K = 128 update
// between them; a trailing odd 128-block takes the 128-row leaf.
struct WideScratch {
    std::vector<bf16*> hi, lo;
};
void trsm(const std::vector<MixedLU*>& g, const std::vector<Target>& T, bool lower, int k0, int w, int j0,
          const std::vector<int>& ncols_in, const MixedCtx& cx, bool tri = false, const WideScratch* ws = nullptr) {
    std::vector<TcProblem> P;
    std::vector<TcOperands> O;
    std::vector<int> ncols = ncols_in;
    if (tri && lower)
        for (int& c : ncols) c = std::min(c, k0 + w);
    constexpr int W2 = 2 * MX_NB;
    if (ws && w == W2) {
        // wide leaf: S = split(X rows [k0, k0 + 256)), X = inv256 * S (S is a copy: the
        // two 128-row output tiles both read all 256 rows of it)
        std::vector<ConvJob> cj;
        for (size_t m = 0; m < g.size(); ++m) {
            if (ncols[m] <= 0) continue;
            const Target& t = T[m];
            cj.push_back({t.X + k0 + (long long)j0 * t.ldx, 1, t.ldx, W2, ncols[m], ws->hi[m], ws->lo[m], 1, W2});
        }
        convert_group(cj, cx.st);
        const long long qo = (long long)(k0 / W2) * W2 * W2;
        for (size_t m = 0; m < g.size(); ++m) {
            if (ncols[m] <= 0) continue;
            MixedLU& L = *g[m];
            const Target& t = T[m];
            TcProblem p;
            p.M = W2; p.N = ncols[m]; p.K = W2;
            p.alpha = 1.f; p.beta = 0.f;
            p.C = t.X + k0 + (long long)j0 * t.ldx; p.c_rs = 1; p.c_cs = t.ldx;
            p.O_hi = t.Ch + k0 + (long long)j0 * t.ldc; p.O_lo = t.Cl + k0 + (long long)j0 * t.ldc;
            p.o_rs = 1; p.o_cs = t.ldc;
            if (t.Rh && !(tri && lower)) {
                p.P_hi = t.Rh + (long long)k0 * t.ldr + j0; p.P_lo = t.Rl + (long long)k0 * t.ldr + j0;
                p.p_rs = t.ldr; p.p_cs = 1;
            }
            TcOperands o;
            o.A = lower ? SplitMat{L.L2h.get() + qo, L.L2l.get() + qo, W2, W2, W2}
                        : SplitMat{L.U2h.get() + qo, L.U2l.get() + qo, W2, W2, W2};
            o.B = SplitMat{ws->hi[m], ws->lo[m], ncols[m], W2, W2};
            P.push_back(p);
            O.push_back(o);
        }
        run(P, O, cx);
        return;
    }
    if (w == MX_NB) {
        // leaf: B -> split (column-major), X = inv_b * B, keep the split copies equal to X
        std::vector<ConvJob> cj;
        for (size_t m = 0; m < g.size(); ++m) {
            if (ncols[m] <= 0) continue;
            const Target& t = T[m];
            cj.push_back({t.X + k0 + (long long)j0 * t.ldx, 1, t.ldx, MX_NB, ncols[m], t.Ch + k0 + (long long)j0 * t.ldc,
                          t.Cl + k0 + (long long)j0 * t.ldc, 1, t.ldc});
        }
        convert_group(cj, cx.st);
        const int b = k0 / MX_NB;
        for (size_t m = 0; m < g.size(); ++m) {
            if (ncols[m] <= 0) continue;
            MixedLU& L = *g[m];
            const Target& t = T[m];
            const long long bo = (long long)b * MX_NB * MX_NB;
            TcProblem p;
            p.M = MX_NB; p.N = ncols[m]; p.K = MX_NB;
            p.alpha = 1.f; p.beta = 0.f;
            p.C = t.X + k0 + (long long)j0 * t.ldx; p.c_rs = 1; p.c_cs = t.ldx;
            p.O_hi = t.Ch + k0 + (long long)j0 * t.ldc; p.O_lo = t.Cl + k0 + (long long)j0 * t.ldc;
            p.o_rs = 1; p.o_cs = t.ldc;
            // the row-major copy; an inversion's lower solve skips it (the upper
            // solve rewrites every row)
            if (t.Rh && !(tri && lower)) {
                p.P_hi = t.Rh + (long long)k0 * t.ldr + j0; p.P_lo = t.Rl + (long long)k0 * t.ldr + j0;
                p.p_rs = t.ldr; p.p_cs = 1;
            }
            TcOperands o;
            o.A = lower ? SplitMat{L.LiRh.get() + bo, L.LiRl.get() + bo, MX_NB, MX_NB, MX_NB}
                        : SplitMat{L.UiRh.get() + bo, L.UiRl.get() + bo, MX_NB, MX_NB, MX_NB};
            o.B = cview(t.Ch, t.Cl, t.ldc, k0, j0, MX_NB, ncols[m]);
            P.push_back(p);
            O.push_back(o);
        }
        run(P, O, cx);
        return;
    }
    const int w1 = ws ? std::max(W2, (w / W2 / 2) * W2) : std::max(MX_NB, (w / MX_NB / 2) * MX_NB), w2 = w - w1;
    // lower: first half solves, then updates the second; upper: the reverse
    const int ka = lower ? k0 : k0 + w1, wa = lower ? w1 : w2;  // solved first
    const int kb = lower ? k0 + w1 : k0, wb = lower ? w2 : w1;  // updated, solved second
    trsm(g, T, lower, ka, wa, j0, ncols, cx, tri, ws);
    for (size_t m = 0; m < g.size(); ++m) {
        const int nc = tri && lower ? std::min(ncols[m], ka + wa) : ncols[m];
        if (nc <= 0) continue;
        MixedLU& L = *g[m];
        const Target& t = T[m];
        TcProblem p;
        p.M = wb; p.N = nc; p.K = wa;
        p.alpha = -1.f; p.beta = 1.f;
        p.C = t.X + kb + (long long)j0 * t.ldx; p.c_rs = 1; p.c_cs = t.ldx;
        TcOperands o;
        o.A = rview(L.Rh.get(), L.Rl.get(), L.n, kb, ka, wb, wa);  // factor block (rows kb, columns ka)
        o.B = cview(t.Ch, t.Cl, t.ldc, ka, j0, wa, nc);             // solved rows of X
        P.push_back(p);
        O.push_back(o);
    }
    run(P, O, cx);
    trsm(g, T, lower, kb, wb, j0, ncols, cx, tri, ws);
}

void leaf(const std::vector<MixedLU*>& g, int c0, const MixedCtx& cx) {
    std::vector<DiagJob> dj;
    const int b = c0 / MX_NB;
    for (MixedLU* L : g) {
        const long long bo = (long long)b * MX_NB * MX_NB;
        dj.push_back({L->A.get() + c0 + (long long)c0 * L->n, L->n, L->Li.get() + bo, L->Ui.get() + bo,
                      L->LiRh.get() + bo, L->LiRl.get() + bo, L->UiRh.get() + bo, L->UiRl.get() + bo,
                      L->UiCh.get() + bo, L->UiCl.get() + bo, L->LiCh.get() + bo, L->LiCl.get() + bo});
    }
    diag_group(dj, cx);
    const int n = g[0]->n, rows = n - c0 - MX_NB;
    if (rows <= 0) return;
    // L21 = A21 U11^{-1}: A21 -> row-major split, GEMM writes L21 (FP32 + row-major split)
    std::vector<ConvJob> cj;
    for (MixedLU* L : g) {
        const long long ld = L->n;
        cj.push_back({L->A.get() + (c0 + MX_NB) + (long long)c0 * ld, 1, ld, rows, MX_NB,
                      L->Rh.get() + (long long)(c0 + MX_NB) * ld + c0, L->Rl.get() + (long long)(c0 + MX_NB) * ld + c0,
                      ld, 1});
    }
    convert_group(cj, cx.st);
    std::vector<TcProblem> P;
    std::vector<TcOperands> O;
    for (MixedLU* L : g) {
        const long long ld = L->n, bo = (long long)b * MX_NB * MX_NB;
        TcProblem p;
        p.M = rows; p.N = MX_NB; p.K = MX_NB;
        p.alpha = 1.f; p.beta = 0.f;
        p.C = L->A.get() + (c0 + MX_NB) + (long long)c0 * ld; p.c_rs = 1; p.c_cs = ld;
        p.O_hi = L->Rh.get() + (long long)(c0 + MX_NB) * ld + c0;
        p.O_lo = L->Rl.get() + (long long)(c0 + MX_NB) * ld + c0;
        p.o_rs = ld; p.o_cs = 1;
        p.check_unit = 1;
        TcOperands o;
        o.A = rview(L->Rh.get(), L->Rl.get(), ld, c0 + MX_NB, c0, rows, MX_NB);
        o.B = SplitMat{L->UiCh.get() + bo, L->UiCl.get() + bo, MX_NB, MX_NB, MX_NB};
        P.push_back(p);
        O.push_back(o);
    }
    run(P, O, cx);
}

void lu_rec(const std::vector<MixedLU*>& g, int c0, int w, const MixedCtx& cx) {
    if (w == MX_NB) {
        leaf(g, c0, cx);
        return;
    }
    const int w1 = std::max(MX_NB, (w / MX_NB / 2) * MX_NB), w2 = w - w1;
    const int n = g[0]->n;
    lu_rec(g, c0, w1, cx);
    // U12 = L11^{-1} A12 on rows [c0, c0 + w1), columns [c0 + w1, c0 + w)
    std::vector<Target> T;
    std::vector<int> nc;
    for (MixedLU* L : g) {
        T.push_back({L->A.get(), L->n, L->Ch.get(), L->Cl.get(), L->n, L->Rh.get(), L->Rl.get(), L->n});
        nc.push_back(w2);
    }
    trsm(g, T, true, c0, w1, c0 + w1, nc, cx);
    // A22 -= L21 U12 (rows [c0 + w1, n), columns [c0 + w1, c0 + w), K = w1)
    std::vector<TcProblem> P;
    std::vector<TcOperands> O;
    const int rows = n - c0 - w1;
    for (MixedLU* L : g) {
        const long long ld = L->n;
        TcProblem p;
        p.M = rows; p.N = w2; p.K = w1;
        p.alpha = -1.f; p.beta = 1.f;
        p.C = L->A.get() + (c0 + w1) + (long long)(c0 + w1) * ld; p.c_rs = 1; p.c_cs = ld;
        TcOperands o;
        o.A = rview(L->Rh.get(), L->Rl.get(), ld, c0 + w1, c0, rows, w1);
        o.B = cview(L->Ch.get(), L->Cl.get(), ld, c0, c0 + w1, w1, w2);
        P.push_back(p);
        O.push_back(o);
    }
    run(P, O, cx);
    lu_rec(g, c0 + w1, w2, cx);
}

}  // namespace

// Column-major to column-major (no transposition), every pointer and column
// stride allowing 16-byte FP32 and 8-byte BF16 vectors, rows a multiple of 4:
// one thread per 4 rows of a column, no shared memory.
__global__ void __launch_bounds__(256) conv_direct_kernel(const __grid_constant__ ConvArgs args) {
    const ConvJob& J = args.j[blockIdx.y];
    const int r4 = J.rows / 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= r4 * J.cols) return;
    const int c = t / r4, r = (t - c * r4) * 4;
    const float4 v = *reinterpret_cast<const float4*>(J.src + r + (long long)c * J.s_cs);
    const float x[4] = {v.x, v.y, v.z, v.w};
    uint2 hv, lv;
    bf16* hp = reinterpret_cast<bf16*>(&hv);
    bf16* lp = reinterpret_cast<bf16*>(&lv);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const bf16 h = __float2bfloat16_rn(x[q]);
        hp[q] = h;
        lp[q] = __float2bfloat16_rn(x[q] - __bfloat162float(h));
    }
    const long long o = r + (long long)c * J.d_cs;
    *reinterpret_cast<uint2*>(J.hi + o) = hv;
    *reinterpret_cast<uint2*>(J.lo + o) = lv;
}

namespace {
bool direct_ok(const ConvJob& j) {
    return j.s_rs == 1 && j.d_rs == 1 && j.rows % 4 == 0 && j.s_cs % 4 == 0 && j.d_cs % 4 == 0 &&
           ((uintptr_t)j.src & 15) == 0 && ((uintptr_t)j.hi & 7) == 0 && ((uintptr_t)j.lo & 7) == 0 &&
           (long long)(j.rows / 4) * j.cols <= 0x7fffffffLL;
}
}  // namespace

void convert_group(const std::vector<ConvJob>& jobs, cudaStream_t st) {
    if (jobs.empty()) return;
    for (size_t i0 = 0; i0 < jobs.size(); i0 += MAXJOBS) {
        ConvArgs a;
        a.n = (int)std::min<size_t>(MAXJOBS, jobs.size() - i0);
        long long mx = 0, mxd = 0;
        double bytes = 0;
        bool direct = true;
        for (int k = 0; k < a.n; ++k) {
            a.j[k] = jobs[i0 + k];
            const long long tiles = (long long)((a.j[k].rows + CV_T - 1) / CV_T) * ((a.j[k].cols + CV_T - 1) / CV_T);
            mx = std::max(mx, tiles);
            mxd = std::max(mxd, (long long)(a.j[k].rows / 4) * a.j[k].cols);
            direct = direct && direct_ok(a.j[k]);
            bytes += 8.0 * a.j[k].rows * a.j[k].cols;  // FP32 read, two BF16 written
        }
        if (mx == 0) continue;
        if (mx > 0x7fffffffLL) fail(SQBEM_ERR_ARG, "convert: block too large");
        if (direct)
            TIMED_LAUNCH("convert", 0.0, bytes, conv_direct_kernel, dim3((unsigned)ceil_div(mxd, 256), (unsigned)a.n),
                         256, 0, st, a);
        else
            TIMED_LAUNCH("convert", 0.0, bytes, conv_kernel, dim3((unsigned)mx, (unsigned)a.n), dim3(CV_T, CV_RY), 0,
                         st, a);
    }
}

// ---------------------------------------------------------------- triangular solves, few right-hand sides
// x <- U^{-1} L^{-1} x for R <= 2 columns.  Each member is solved by a cluster
// of TS_CL CTAs; every CTA holds all of x in its shared memory.  The solve runs
// by 128-row blocks: s = x_b - (off-diagonal blocks) x, the block's rows split
// over the cluster (one row per warp, reading the row-major split factor along
// its contiguous index, hi + lo, 16 bytes per lane); each CTA writes its rows of
// s into the shared memory of every CTA of the cluster; after the cluster
// barrier every CTA forms x_b = inv(diag block) s itself (the 128 x 128 FP32
// block inverse, read from L2).  s is double-buffered, so one barrier per block
// suffices: a CTA writes block k + 1's sums only after all CTAs have reached
// block k's barrier, i.e. have finished reading block k - 1's.  Input and output
// are FP64 (rows beyond n_true are zero); the arithmetic is FP32 like the
// tensor-core solves.
constexpr int TS_THREADS = 1024;
constexpr int TS_CL = 4;                // CTAs per member (thread-block cluster)
constexpr int TS_ROWS = MX_NB / TS_CL;  // block rows per CTA: one per warp
static_assert(TS_ROWS == TS_THREADS / 32, "one block row per warp");
constexpr int TS_PARTS = TS_THREADS / MX_NB;  // the diagonal product's q range split this many ways
struct TrsvJob {
    const bf16* Rh;
    const bf16* Rl;
    const float* Li;
    const float* Ui;
    const double* in;
    long long ldi;
    double* out;
    long long ldo;
    int n_true;
};
struct TrsvArgs {
    int n, r;
    TrsvJob j[MAXJOBS];
};

// x lives in shared memory per column, at position xpos(k): lane l of a warp
// reads entries k0 + 8 l + q (q = 0..7) of its row's 8-column segment, so entry k
// goes to (k & ~255) + 32 (k & 7) + ((k >> 3) & 31) -- the 32 lanes hit 32
// consecutive words (no bank conflict).  Columns are padded to a multiple of 256.
__device__ __forceinline__ int xpos(int k) { return (k & ~255) + ((k & 7) << 5) + ((k >> 3) & 31); }
inline int trsv_npad(int n) { return (n + 255) & ~255; }
// shared memory of one CTA: x (npad x R), s (2 x 128 x R), partial products (TS_PARTS x 128 x R)
inline size_t trsv_smem(int n, int R) {
    return ((size_t)trsv_npad(n) + 2 * MX_NB + TS_PARTS * MX_NB) * R * sizeof(float);
}

template <int R>
__global__ void __cluster_dims__(TS_CL, 1, 1) __launch_bounds__(TS_THREADS)
    trsv_kernel(const __grid_constant__ TrsvArgs args) {
    extern __shared__ float tsm[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const TrsvJob& J = args.j[blockIdx.x / TS_CL];
    const int n = args.n, nt = J.n_true, r = args.r;
    const int npad = (n + 255) & ~255;
    float* x = tsm;                        // column c: x[c * npad + xpos(row)]
    float* sb = tsm + (size_t)npad * R;    // sb[buf][rl * R + c]
    float* part = sb + 2 * MX_NB * R;      // part[(h * 128 + rl) * R + c]
    const bf16* Rh = J.Rh;
    const bf16* Rl = J.Rl;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int e = tid; e < n * R; e += TS_THREADS) {
        const int row = e / R, c = e % R;
        x[c * npad + xpos(row)] = (row < nt && c < r) ? (float)J.in[row + c * J.ldi] : 0.f;
    }
    __syncthreads();
    const int nb = n / MX_NB;
    int buf = 0;
    for (int pass = 0; pass < 2; ++pass) {  // 0: L (forward), 1: U (backward)
        for (int step = 0; step < nb; ++step) {
            const int b = pass == 0 ? step : nb - 1 - step;
            const int k0 = pass == 0 ? 0 : (b + 1) * MX_NB, k1 = pass == 0 ? b * MX_NB : n;
            {
                // s = x_b - A(row, [k0, k1)) x([k0, k1)) for this warp's row; each lane
                // loads 8 consecutive entries of hi and of lo per step (k0, k1 and n are
                // multiples of 128, so the 16-byte loads are aligned and in bounds)
                const int rl = rank * TS_ROWS + warp;
                const int row = b * MX_NB + rl;
                float acc[R];
#pragma unroll
                for (int c = 0; c < R; ++c) acc[c] = 0.f;
                const long long base = (long long)row * n;
#pragma unroll 2
                for (int k = k0 + 8 * lane; k < k1; k += 256) {
                    const uint4 hv = *reinterpret_cast<const uint4*>(Rh + base + k);
                    const uint4 lv = *reinterpret_cast<const uint4*>(Rl + base + k);
                    const bf16* hp = reinterpret_cast<const bf16*>(&hv);
                    const bf16* lp = reinterpret_cast<const bf16*>(&lv);
                    const int xp = xpos(k);  // k is a multiple of 8: entry k + q sits at xp + 32 q
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float a = __bfloat162float(hp[q]) + __bfloat162float(lp[q]);
#pragma unroll
                        for (int c = 0; c < R; ++c) acc[c] = fmaf(a, x[c * npad + xp + 32 * q], acc[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < R; ++c) {
                    float v = acc[c];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    acc[c] = x[c * npad + xpos(row)] - v;
                }
                if (lane < TS_CL) {  // lane q writes into the shared memory of cluster CTA q
                    float* dst = cl.map_shared_rank(sb, lane) + buf * MX_NB * R + rl * R;
#pragma unroll
                    for (int c = 0; c < R; ++c) dst[c] = acc[c];
                }
            }
            cl.sync();
            // x_b = inv(diag block b) s  (column-major 128 x 128 FP32 inverse): thread
            // (h, rl) sums q in [h * 16, h * 16 + 16), then the parts add in order h
            const float* Inv = (pass == 0 ? J.Li : J.Ui) + (size_t)b * MX_NB * MX_NB;
            const float* s = sb + buf * MX_NB * R;
            {
                const int rl = tid % MX_NB, h = tid / MX_NB;
                constexpr int QN = MX_NB / TS_PARTS;
                float v[R];
#pragma unroll
                for (int c = 0; c < R; ++c) v[c] = 0.f;
#pragma unroll
                for (int q = h * QN; q < h * QN + QN; ++q) {
                    const float a = __ldg(Inv + rl + q * MX_NB);
#pragma unroll
                    for (int c = 0; c < R; ++c) v[c] = fmaf(a, s[q * R + c], v[c]);
                }
#pragma unroll
                for (int c = 0; c < R; ++c) part[(h * MX_NB + rl) * R + c] = v[c];
            }
            __syncthreads();
            if (tid < MX_NB * R) {
                const int rl = tid % MX_NB, c = tid / MX_NB;
                float v = 0.f;
#pragma unroll
                for (int h = 0; h < TS_PARTS; ++h) v += part[(h * MX_NB + rl) * R + c];
                x[c * npad + xpos(b * MX_NB + rl)] = v;
            }
            __syncthreads();
            buf ^= 1;
        }
    }
    // each CTA writes its share of the rows
    for (int e = tid + rank * TS_THREADS; e < nt * R; e += TS_THREADS * TS_CL) {
        const int row = e / R, c = e % R;
        if (c < r) J.out[row + c * J.ldo] = (double)x[c * npad + xpos(row)];
    }
    // no CTA leaves while a peer could still address its shared memory
    cl.sync();
}

namespace {
template <int R>
void trsv_launch(const std::vector<const MixedLU*>& g, const std::vector<TrsvIO>& io, int c0, int r, cudaStream_t st) {
    const int n = g[0]->n;
    const size_t smem = trsv_smem(n, R);
    static std::once_flag attr;
    std::call_once(attr, [] {
        CUDA_CHECK(cudaFuncSetAttribute(trsv_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    });
    for (size_t i0 = 0; i0 < g.size(); i0 += MAXJOBS) {
        TrsvArgs a;
        a.n = n;
        a.r = r;
        const int m = (int)std::min<size_t>(MAXJOBS, g.size() - i0);
        for (int k = 0; k < m; ++k) {
            const MixedLU& L = *g[i0 + k];
            const TrsvIO& q = io[i0 + k];
            a.j[k] = {L.Rh.get(), L.Rl.get(), L.Li.get(), L.Ui.get(), q.in + (long long)c0 * q.ldi, q.ldi,
                      q.out + (long long)c0 * q.ldo, q.ldo, q.n_true};
        }
        const double by = (double)m * ((double)n * n * 4.0 + 2.0 * n * r * 8.0);
        TIMED_LAUNCH("trsv", 0.0, by, trsv_kernel<R>, m * TS_CL, TS_THREADS, smem, st, a);
    }
}
}  // namespace

void trsv_group_io(const std::vector<const MixedLU*>& g, const std::vector<TrsvIO>& io, int r, cudaStream_t st) {
    if (g.empty()) return;
    if (r < 1 || r > 8 || io.size() != g.size()) fail(SQBEM_ERR_ARG, "trsv: 1 to 8 right-hand sides");
    const int n = g[0]->n;
    for (size_t k = 0; k < g.size(); ++k) {
        if (g[k]->n != n) fail(SQBEM_ERR_ARG, "trsv: group members differ in size");
        const int nt = io[k].n_true;
        if (nt < 1 || nt > n || io[k].ldi < nt || io[k].ldo < nt) fail(SQBEM_ERR_ARG, "trsv: bad row count");
    }
    if (trsv_smem(n, 2) > 227 * 1024) fail(SQBEM_ERR_ARG, "trsv: %d unknowns exceed shared memory", n);
    if (r > 2 && trsv_smem(n, 8) <= 227 * 1024) {
        trsv_launch<8>(g, io, 0, r, st);
        return;
    }
    for (int c0 = 0; c0 < r; c0 += 2) trsv_launch<2>(g, io, c0, std::min(2, r - c0), st);
}

void trsv_group(const std::vector<const MixedLU*>& g, const std::vector<const double*>& in,
                const std::vector<double*>& out, const std::vector<int>& n_true, int r, cudaStream_t st) {
    std::vector<TrsvIO> io(g.size());
    for (size_t k = 0; k < g.size(); ++k) io[k] = {in[k], n_true[k], out[k], n_true[k], n_true[k]};
    trsv_group_io(g, io, r, st);
}

void mixed_lu_factor(const std::vector<MixedLU*>& g, const MixedCtx& cx) {
    if (g.empty()) return;
    const int n = g[0]->n;
    for (MixedLU* L : g)
        if (L->n != n) fail(SQBEM_ERR_ARG, "mixed_lu_factor: group members differ in size");
    lu_rec(g, 0, n, cx);
}

namespace {
// The three quadrants of each composed 256-block inverse that are copies or
// zeros: L2 = [L11i 0; . L22i], U2 = [U11i .; 0 U22i] (row-major split, ld 256);
// the off-diagonal quadrants come from the GEMMs of compose_wide.
struct FillJob {
    const bf16 *lrh, *lrl, *urh, *url;  // LiR, UiR split copies of the 128-blocks (row-major)
    bf16 *l2h, *l2l, *u2h, *u2l;
    int nb2;
};
struct FillArgs {
    FillJob j[MAXJOBS];
};
__global__ void compose_fill_kernel(const __grid_constant__ FillArgs args) {
    const FillJob& J = args.j[blockIdx.y];
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    constexpr int B = MX_NB, B2 = 2 * MX_NB;
    if (e >= (long long)J.nb2 * B2 * B2) return;
    const int q = (int)(e / (B2 * B2)), rc = (int)(e % (B2 * B2)), r = rc / B2, c = rc % B2;
    const long long o = (long long)q * B2 * B2 + rc;
    const bf16 zero = __float2bfloat16_rn(0.f);
    if (r < B && c < B) {  // block 2q
        const long long i = (long long)(2 * q) * B * B + r * B + c;
        J.l2h[o] = J.lrh[i]; J.l2l[o] = J.lrl[i];
        J.u2h[o] = J.urh[i]; J.u2l[o] = J.url[i];
    } else if (r >= B && c >= B) {  // block 2q + 1
        const long long i = (long long)(2 * q + 1) * B * B + (r - B) * B + (c - B);
        J.l2h[o] = J.lrh[i]; J.l2l[o] = J.lrl[i];
        J.u2h[o] = J.urh[i]; J.u2l[o] = J.url[i];
    } else if (r < B) {  // upper-right: zero in L2, the GEMM's in U2
        J.l2h[o] = zero; J.l2l[o] = zero;
    } else {  // lower-left: zero in U2, the GEMM's in L2
        J.u2h[o] = zero; J.u2l[o] = zero;
    }
}

// inv([L11 0; L21 L22]) = [L11i 0; -L22i L21 L11i  L22i] and
// inv([U11 U12; 0 U22]) = [U11i -U11i U12 U22i; 0 U22i] for every pair of
// 128-blocks: two grouped GEMM launches (T = L21 L11i and U12 U22i, then the
// products with -L22i and -U11i) on top of the factor's split copies.
void compose_wide(const std::vector<MixedLU*>& g, const MixedCtx& cx) {
    const int n = g[0]->n, nb2 = n / (2 * MX_NB);
    constexpr int B = MX_NB, B2 = 2 * MX_NB;
    if (nb2 == 0) {
        for (MixedLU* L : g) L->wide = true;
        return;
    }
    const size_t per = (size_t)nb2 * B2 * B2, tper = (size_t)nb2 * B * B;
    std::vector<DevBuf<bf16>> th(g.size()), tl(g.size()), uh(g.size()), ul(g.size());
    for (size_t m0 = 0; m0 < g.size(); m0 += MAXJOBS) {
        FillArgs a;
        const int cnt = (int)std::min<size_t>(MAXJOBS, g.size() - m0);
        for (int k = 0; k < cnt; ++k) {
            MixedLU& L = *g[m0 + k];
            L.L2h.alloc(per, cx.st); L.L2l.alloc(per, cx.st);
            L.U2h.alloc(per, cx.st); L.U2l.alloc(per, cx.st);
            a.j[k] = {L.LiRh.get(), L.LiRl.get(), L.UiRh.get(), L.UiRl.get(), L.L2h.get(), L.L2l.get(),
                      L.U2h.get(), L.U2l.get(), nb2};
        }
        LAUNCH(compose_fill_kernel, dim3((unsigned)ceil_div((long long)per, 256), (unsigned)cnt), 256, 0, cx.st, a);
    }
    std::vector<TcProblem> P;
    std::vector<TcOperands> O;
    for (size_t m = 0; m < g.size(); ++m) {
        MixedLU& L = *g[m];
        th[m].alloc(tper, cx.st); tl[m].alloc(tper, cx.st);
        uh[m].alloc(tper, cx.st); ul[m].alloc(tper, cx.st);
        for (int q = 0; q < nb2; ++q) {
            const int k0 = q * B2, b0 = 2 * q, b1 = 2 * q + 1;
            const long long bo0 = (long long)b0 * B * B, bo1 = (long long)b1 * B * B, to = (long long)q * B * B;
            TcProblem p;  // T_L = L21 L11i -> column-major split
            p.M = B; p.N = B; p.K = B;
            p.O_hi = th[m].get() + to; p.O_lo = tl[m].get() + to; p.o_rs = 1; p.o_cs = B;
            TcOperands o;
            o.A = rview(L.Rh.get(), L.Rl.get(), L.n, k0 + B, k0, B, B);
            o.B = SplitMat{L.LiCh.get() + bo0, L.LiCl.get() + bo0, B, B, B};
            P.push_back(p);
            O.push_back(o);
            TcProblem pu = p;  // T_U = U12 U22i
            pu.O_hi = uh[m].get() + to; pu.O_lo = ul[m].get() + to;
            TcOperands ou;
            ou.A = rview(L.Rh.get(), L.Rl.get(), L.n, k0, k0 + B, B, B);
            ou.B = SplitMat{L.UiCh.get() + bo1, L.UiCl.get() + bo1, B, B, B};
            P.push_back(pu);
            O.push_back(ou);
        }
    }
    run(P, O, cx);
    for (size_t m = 0; m < g.size(); ++m) {
        MixedLU& L = *g[m];
        for (int q = 0; q < nb2; ++q) {
            const int b0 = 2 * q, b1 = 2 * q + 1;
            const long long bo0 = (long long)b0 * B * B, bo1 = (long long)b1 * B * B, to = (long long)q * B * B;
            const long long qo = (long long)q * B2 * B2;
            TcProblem p;  // L2 lower-left = -L22i T_L
            p.M = B; p.N = B; p.K = B; p.alpha = -1.f;
            p.O_hi = L.L2h.get() + qo + (long long)B * B2; p.O_lo = L.L2l.get() + qo + (long long)B * B2;
            p.o_rs = B2; p.o_cs = 1;
            TcOperands o;
            o.A = SplitMat{L.LiRh.get() + bo1, L.LiRl.get() + bo1, B, B, B};
            o.B = SplitMat{th[m].get() + to, tl[m].get() + to, B, B, B};
            P.push_back(p);
            O.push_back(o);
            TcProblem pu = p;  // U2 upper-right = -U11i T_U
            pu.O_hi = L.U2h.get() + qo + B; pu.O_lo = L.U2l.get() + qo + B;
            TcOperands ou;
            ou.A = SplitMat{L.UiRh.get() + bo0, L.UiRl.get() + bo0, B, B, B};
            ou.B = SplitMat{uh[m].get() + to, ul[m].get() + to, B, B, B};
            P.push_back(pu);
            O.push_back(ou);
        }
        L.wide = true;
    }
    run(P, O, cx);
}
}  // namespace

void mixed_lu_solve(const std::vector<MixedLU*>& g, const std::vector<Rhs>& rhs, const MixedCtx& cx,
                    bool identity_rhs) {
    if (g.empty()) return;
    std::vector<Target> T;
    std::vector<int> nc;
    int maxc = 0;
    for (size_t m = 0; m < g.size(); ++m) {
        const Rhs& r = rhs[m];
        T.push_back({r.X, r.ldx, r.Sh, r.Sl, r.lds, r.Rh, r.Rl, r.ldr});
        nc.push_back(r.nrhs);
        maxc = std::max(maxc, r.nrhs);
    }
    if (maxc == 0) return;
    const int n = g[0]->n;
    bool all_wide = true;
    for (MixedLU* L : g) all_wide = all_wide && L->wide;
    if (!all_wide) compose_wide(g, cx);
    // the wide leaves' conversion targets, one 256-row split slab per member
    std::vector<DevBuf<bf16>> sh(g.size()), sl(g.size());
    WideScratch ws;
    for (size_t m = 0; m < g.size(); ++m) {
        sh[m].alloc((size_t)2 * MX_NB * std::max(nc[m], 1), cx.st);
        sl[m].alloc((size_t)2 * MX_NB * std::max(nc[m], 1), cx.st);
        ws.hi.push_back(sh[m].get());
        ws.lo.push_back(sl[m].get());
    }
    trsm(g, T, true, 0, n, 0, nc, cx, identity_rhs, &ws);
    trsm(g, T, false, 0, n, 0, nc, cx, false, &ws);
}

}  // namespace sqbem
