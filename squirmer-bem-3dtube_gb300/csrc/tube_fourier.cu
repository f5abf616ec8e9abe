// tube_fourier.cu -- Fourier blocks of the tube and solves through them (see
// tube_fourier.cuh).
#include <cooperative_groups.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "tc_gemm.cuh"
#include "tube_fourier.cuh"

namespace cg = cooperative_groups;

namespace sqbem {

namespace {

constexpr int FT_MAXF = FT_MAX_SECTORS / 2 + 1;  // frequencies held at most
constexpr int FT_JOBS = 48;                      // jobs per grouped launch
constexpr double TWO_PI = 6.283185307179586476925286766559;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ---------------------------------------------------------------- the blocks
// C^_f[(a, al), (b, be)] = sum_d w^{f d} sum_g T0[3 a + al, 3 panel(b, d) + g] R_d[g][be],
// accumulated in FP64 (high frequencies cancel), stored as FP32 complex.
// Thread: row r = (a, al); blockIdx.y: column c = (b, be); blockIdx.z: job.
struct ChatJob {
    const float* T0;
    const int* panel;
    float2* C;  // nf blocks of n3 x n3, column-major
};
struct ChatArgs {
    int n;
    int nth, nb, nf;
    double2 tw[FT_MAX_SECTORS];  // (cos, sin) of 2 pi k / nth
    ChatJob j[FT_JOBS];
};

__global__ void chat_kernel(const __grid_constant__ ChatArgs args) {
    const ChatJob& J = args.j[blockIdx.z];
    const int nth = args.nth, n3 = 3 * args.nb;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n3) return;
    const int c = blockIdx.y, b = c / 3, be = c % 3;
    double re[FT_MAXF], im[FT_MAXF];
#pragma unroll
    for (int f = 0; f < FT_MAXF; ++f) re[f] = im[f] = 0.0;
    for (int d = 0; d < nth; ++d) {
        const int q = J.panel[b * nth + d];
        const float* col = J.T0 + r + (long long)(3 * q) * n3;
        const double cs = args.tw[d].x, sn = args.tw[d].y;
        double v;  // (T0 R_d)[r, 3 q + be]
        if (be == 2) v = col[2LL * n3];
        else if (be == 0) v = cs * col[0] + sn * col[n3];
        else v = -sn * col[0] + cs * col[n3];
        int k = 0;  // f d mod nth
#pragma unroll
        for (int f = 0; f < FT_MAXF; ++f) {
            if (f < args.nf) {
                re[f] += v * args.tw[k].x;
                im[f] += v * args.tw[k].y;
                k += d;
                if (k >= nth) k -= nth;
            }
        }
    }
#pragma unroll
    for (int f = 0; f < FT_MAXF; ++f)
        if (f < args.nf) J.C[(long long)f * n3 * n3 + (long long)c * n3 + r] = make_float2((float)re[f], (float)im[f]);
}

// ---------------------------------------------------------------- inversion
// In-place Gauss-Jordan inversion with partial pivoting of one n x n complex
// block per cluster of CL CTAs: CTA q holds columns [q w, q w + w) in its
// shared memory.  Step k: the CTA owning column k finds the pivot row p (largest
// |a_ik|, i >= k) and writes p and the column into every CTA's shared memory
// (double-buffered, so one cluster barrier per step suffices); every CTA swaps
// rows k and p, scales row k by 1 / a_pk and eliminates column k from the other
// rows of its own columns; column k itself becomes column k of the inverse.  The
// row exchanges are undone as column exchanges in reverse order when the
// columns are written back.  A zero pivot sets bit 1 of *flag.
constexpr int GJ_THREADS = 512;
constexpr int GJ_MAXB = 1024;
struct GjArgs {
    int n, w, nblk;
    int* flag;
    float2* C[GJ_MAXB];
};

template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(GJ_THREADS, 1) gj_kernel(const __grid_constant__ GjArgs args) {
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ float2 gsm[];
    const int n = args.n, w = args.w;
    const int rank = (int)cl.block_rank();
    const int blk = blockIdx.x / CL;
    float2* A = gsm;                          // n x w, column-major, leading dimension n
    float2* colk = gsm + (size_t)n * w;       // 2 x n: the pivot column of the step (double-buffered)
    int* meta = reinterpret_cast<int*>(colk + 2 * n);  // [2]: pivot row per buffer (-1: zero pivot)
    int* piv = meta + 2;                      // n: pivot row of every step
    int* pos = piv + n;                       // n: output column of every stored column
    float2* mk = reinterpret_cast<float2*>(pos + n);  // n: multipliers of the step (2 + 2 n ints: 8-byte aligned)
    const int c0 = rank * w, wl = max(0, min(w, n - c0));
    float2* C = blk < args.nblk ? args.C[blk] : nullptr;
    if (C)
        for (int e = threadIdx.x; e < n * wl; e += blockDim.x) A[e] = C[(long long)c0 * n + e];
    cl.sync();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    bool bad = false;
    for (int k = 0; k < n; ++k) {
        const int buf = k & 1;
        if (rank == k / w) {
            const float2* ca = A + (size_t)(k - c0) * n;
            // every thread copies a share of the column into every CTA; warp 0 also
            // finds the pivot row
            for (int e = threadIdx.x; e < CL * n; e += blockDim.x) {
                const int q = e / n, i = e - q * n;
                cl.map_shared_rank(colk, q)[buf * n + i] = ca[i];
            }
            if (warp == 0) {
                float best = -1.f;
                int bi = k;
                for (int i = k + lane; i < n; i += 32) {
                    const float2 v = ca[i];
                    const float m = v.x * v.x + v.y * v.y;
                    if (m > best) { best = m; bi = i; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
                }
                if (lane < CL) cl.map_shared_rank(meta, lane)[buf] = best > 0.f ? bi : -1;
            }
        }
        cl.sync();
        const int p = meta[buf];
        if (p < 0) { bad = true; break; }  // the same in every CTA of the cluster
        if (threadIdx.x == 0) piv[k] = p;
        const float2* ck = colk + buf * n;  // column k before the exchange
        const float2 pv = ck[p];
        const float s2 = 1.f / (pv.x * pv.x + pv.y * pv.y);
        const float2 d = make_float2(pv.x * s2, -pv.y * s2);  // 1 / pivot
        // the multipliers after the exchange, row k's set to zero
        for (int i = threadIdx.x; i < n; i += blockDim.x) mk[i] = i == k ? make_float2(0.f, 0.f) : ck[i == p ? k : i];
        // exchange rows k and p and scale the new row k (one lane per column)
        for (int jl = threadIdx.x; jl < wl; jl += blockDim.x) {
            float2* col = A + (size_t)jl * n;
            const float2 vk = col[k], vp = col[p];
            col[p] = vk;
            col[k] = c0 + jl == k ? d : cmul(vp, d);
        }
        __syncthreads();
        // eliminate: column j -= m * (row k), row k itself untouched (m_k = 0);
        // column k of the inverse: -m_i / pivot (row k: 1 / pivot)
        for (int jl = warp; jl < wl; jl += nw) {
            float2* col = A + (size_t)jl * n;
            if (c0 + jl == k) {
                for (int i = lane; i < n; i += 32)
                    if (i != k) {
                        const float2 t = cmul(mk[i], d);
                        col[i] = make_float2(-t.x, -t.y);
                    }
            } else {
                const float2 rk = col[k];
                for (int i = lane; i < n; i += 32) {
                    const float2 m = mk[i], c = col[i];
                    col[i] = make_float2(c.x - (m.x * rk.x - m.y * rk.y), c.y - (m.x * rk.y + m.y * rk.x));
                }
            }
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0 && rank == 0) atomicOr(args.flag, 2);
        return;
    }
    if (threadIdx.x == 0) {
        // stored column cur[c] is output column c: the exchanges (k, piv[k]) in reverse order
        int* cur = pos;  // built in place, then inverted below through colk's space
        for (int c = 0; c < n; ++c) cur[c] = c;
        for (int k = n - 1; k >= 0; --k) {
            const int p = piv[k];
            if (p != k) { const int t = cur[k]; cur[k] = cur[p]; cur[p] = t; }
        }
        int* inv = reinterpret_cast<int*>(colk);  // the pivot columns are no longer needed
        for (int c = 0; c < n; ++c) inv[cur[c]] = c;
        for (int c = 0; c < n; ++c) pos[c] = inv[c];
    }
    __syncthreads();
    if (C)
        for (int jl = warp; jl < wl; jl += nw) {
            float2* dst = C + (long long)pos[c0 + jl] * n;
            const float2* src = A + (size_t)jl * n;
            for (int i = lane; i < n; i += 32) dst[i] = src[i];
        }
}

// The real form [[Re, -Im], [Im, Re]] of every inverse (n x n complex,
// column-major) as split BF16, row-major with leading dimension ldk, through
// 32 x 32 shared-memory tiles: reads along the source columns, writes along the
// destination rows.  blockIdx.z: block.
struct RfArgs {
    int n, ldk, nblk;
    const float2* C[GJ_MAXB];
    bf16* hi[GJ_MAXB];
    bf16* lo[GJ_MAXB];
};

__global__ void realform_kernel(const __grid_constant__ RfArgs args) {
    __shared__ float tile[32][33];
    const int n = args.n, m2 = 2 * n;
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;  // tile of the real form
    const float2* C = args.C[blockIdx.z];
    // load: element (r, c) of the real form, r = r0 + tx, c = c0 + ty + 8 q
    for (int q = 0; q < 4; ++q) {
        const int r = r0 + threadIdx.x, c = c0 + threadIdx.y + 8 * q;
        float v = 0.f;
        if (r < m2 && c < m2) {
            const int rr = r < n ? r : r - n, cc = c < n ? c : c - n;
            const float2 x = C[(long long)cc * n + rr];
            v = (r < n) == (c < n) ? x.x : (r < n ? -x.y : x.y);
        }
        tile[threadIdx.y + 8 * q][threadIdx.x] = v;
    }
    __syncthreads();
    // store: row r = r0 + ty + 8 q, column c = c0 + tx
    bf16* H = args.hi[blockIdx.z];
    bf16* L = args.lo[blockIdx.z];
    for (int q = 0; q < 4; ++q) {
        const int r = r0 + threadIdx.y + 8 * q, c = c0 + threadIdx.x;
        if (r < m2 && c < m2) {
            const float v = tile[threadIdx.x][threadIdx.y + 8 * q];
            const bf16 h = __float2bfloat16_rn(v);
            H[(long long)r * args.ldk + c] = h;
            L[(long long)r * args.ldk + c] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
}

// ---------------------------------------------------------------- transforms
// Forward: X^_f[(a, al), j] = (1 / nth) sum_s w^{-f s} (R_s^T x_{panel(a, s)})_al for
// column j, written as the split column-major operand of the frequency's GEMM:
// rows [0, n3) the real parts, [n3, 2 n3) the imaginary parts, leading dimension
// ldk, one plane of ldk x nc per frequency.  Thread: r = (a, al); blockIdx.x:
// column; blockIdx.y: job.
struct DftJob {
    const int* panel;
    const float2* tw;
    const void* x;  // forward: input X; inverse: the GEMM result Y^
    long long ldx;
    void* y;        // forward: unused; inverse: output Y
    long long ldy;
    bf16* h;        // forward: X^ split; inverse: optional split copy of Y, element
    bf16* l;        // (r, j) at r * hrs + j * hcs
    long long hrs, hcs;
    int nc, nb, nth, nf, ldk;
};
struct DftArgs {
    int n;
    float2 tw[FT_MAX_SECTORS];  // (cos, sin) of 2 pi k / nth (the kernels specialised on nth read these)
    DftJob j[FT_JOBS];
};

template <class TI>
__global__ void __launch_bounds__(192) fdft_kernel(const __grid_constant__ DftArgs args) {
    const DftJob& J = args.j[blockIdx.y];
    const int j = blockIdx.x;
    if (j >= J.nc) return;
    const int n3 = 3 * J.nb, nth = J.nth, nf = J.nf;
    const TI* x = reinterpret_cast<const TI*>(J.x) + (long long)j * J.ldx;
    const float scale = 1.f / (float)nth;
    for (int r = threadIdx.x; r < n3; r += blockDim.x) {
        const int a = r / 3, al = r - 3 * a;
        float re[FT_MAXF], im[FT_MAXF];
#pragma unroll
        for (int f = 0; f < FT_MAXF; ++f) re[f] = im[f] = 0.f;
        for (int s = 0; s < nth; ++s) {
            const int p = J.panel[a * nth + s];
            const float2 rs = J.tw[s];
            float v;  // (R_s^T x_p)_al
            if (al == 2) v = (float)x[3 * p + 2];
            else {
                const float x0 = (float)x[3 * p], x1 = (float)x[3 * p + 1];
                v = al == 0 ? rs.x * x0 + rs.y * x1 : -rs.y * x0 + rs.x * x1;
            }
            int k = 0;  // f s mod nth
#pragma unroll
            for (int f = 0; f < FT_MAXF; ++f) {
                if (f < nf) {
                    const float2 t = J.tw[k];
                    re[f] += v * t.x;
                    im[f] -= v * t.y;
                    k += s;
                    if (k >= nth) k -= nth;
                }
            }
        }
#pragma unroll
        for (int f = 0; f < FT_MAXF; ++f) {
            if (f < nf) {
                const long long o = ((long long)f * J.nc + j) * J.ldk;
                const float vr = re[f] * scale, vi = im[f] * scale;
                const bf16 hr = __float2bfloat16_rn(vr), hi = __float2bfloat16_rn(vi);
                J.h[o + r] = hr;
                J.l[o + r] = __float2bfloat16_rn(vr - __bfloat162float(hr));
                J.h[o + n3 + r] = hi;
                J.l[o + n3 + r] = __float2bfloat16_rn(vi - __bfloat162float(hi));
            }
        }
    }
}

// Inverse: y~_s = sum over all frequencies of w^{f s} y^_f = Re y^_0 + 2 sum_{0 < f < nth/2}
// Re(w^{f s} y^_f) (+ Re((-1)^s y^_{nth/2}) for even nth), then y_panel(a, s) = R_s y~_s.
// Y^ is the FP32 GEMM result: per frequency ldk x nc, column-major, rows [0, n3)
// real, [n3, 2 n3) imaginary.  Thread: representative a (strided); blockIdx.x:
// column; blockIdx.y: job.
template <class TO>
__global__ void __launch_bounds__(64) idft_kernel(const __grid_constant__ DftArgs args) {
    const DftJob& J = args.j[blockIdx.y];
    const int j = blockIdx.x;
    if (j >= J.nc) return;
    const int n3 = 3 * J.nb, nth = J.nth, nf = J.nf;
    const float* yh = reinterpret_cast<const float*>(J.x) + (long long)j * J.ldk;
    const long long plane = (long long)J.nc * J.ldk;
    TO* y = reinterpret_cast<TO*>(J.y) + (long long)j * J.ldy;
    const bool even = (nth & 1) == 0;
    // components 0 and 1 (rotated together), then component 2
    for (int a = threadIdx.x; a < J.nb; a += blockDim.x)
    for (int pass = 0; pass < 2; ++pass) {
        float r0[FT_MAXF], i0[FT_MAXF], r1[FT_MAXF], i1[FT_MAXF];
#pragma unroll
        for (int f = 0; f < FT_MAXF; ++f) {
            r0[f] = i0[f] = r1[f] = i1[f] = 0.f;
            if (f < nf) {
                const float wgt = (f == 0 || (even && 2 * f == nth)) ? 1.f : 2.f;
                const float* pf = yh + f * plane;
                if (pass == 0) {
                    r0[f] = wgt * pf[3 * a];
                    i0[f] = wgt * pf[n3 + 3 * a];
                    r1[f] = wgt * pf[3 * a + 1];
                    i1[f] = wgt * pf[n3 + 3 * a + 1];
                } else {
                    r0[f] = wgt * pf[3 * a + 2];
                    i0[f] = wgt * pf[n3 + 3 * a + 2];
                }
            }
        }
        for (int s = 0; s < nth; ++s) {
            float v0 = 0.f, v1 = 0.f;
            int k = 0;
#pragma unroll
            for (int f = 0; f < FT_MAXF; ++f) {
                if (f < nf) {
                    const float2 t = J.tw[k];
                    v0 += t.x * r0[f] - t.y * i0[f];
                    if (pass == 0) v1 += t.x * r1[f] - t.y * i1[f];
                    k += s;
                    if (k >= nth) k -= nth;
                }
            }
            const int p = J.panel[a * nth + s];
            const float2 rs = J.tw[s];
            float o[2];
            int nout;
            long long row;
            if (pass == 0) {
                o[0] = rs.x * v0 - rs.y * v1;
                o[1] = rs.y * v0 + rs.x * v1;
                nout = 2;
                row = 3LL * p;
            } else {
                o[0] = v0;
                nout = 1;
                row = 3LL * p + 2;
            }
            for (int q = 0; q < nout; ++q) {
                y[row + q] = (TO)o[q];
                if (J.h) {
                    const long long e = (row + q) * J.hrs + (long long)j * J.hcs;
                    const bf16 h = __float2bfloat16_rn(o[q]);
                    J.h[e] = h;
                    J.l[e] = __float2bfloat16_rn(o[q] - __bfloat162float(h));
                }
            }
        }
    }
}

// Both transforms with a thread per representative a and column (blockIdx.x;
// job: blockIdx.y), all three components of its rows in the thread: the rotation
// R_s needs no exchange between lanes, every panel load and twiddle serves three
// rows, and with the sector and frequency loops unrolled the twiddles are
// constant operands of the multiply-adds.
template <int NTH, class TI>
__global__ void __launch_bounds__(64) fdft_rep(const __grid_constant__ DftArgs args) {
    constexpr int NF = NTH / 2 + 1;
    const DftJob& J = args.j[blockIdx.y];
    const int j = blockIdx.x;
    if (j >= J.nc) return;
    const int n3 = 3 * J.nb;
    const TI* x = reinterpret_cast<const TI*>(J.x) + (long long)j * J.ldx;
    const float scale = 1.f / (float)NTH;
    for (int a = threadIdx.x; a < J.nb; a += blockDim.x) {
        const int* pa = J.panel + a * NTH;
        float v[3][NTH];  // R_s^T x_{panel(a, s)}
#pragma unroll
        for (int s = 0; s < NTH; ++s) {
            const TI* xp = x + 3LL * __ldg(pa + s);
            const float x0 = (float)__ldg(xp), x1 = (float)__ldg(xp + 1);
            const float c = args.tw[s].x, sn = args.tw[s].y;
            v[0][s] = c * x0 + sn * x1;
            v[1][s] = -sn * x0 + c * x1;
            v[2][s] = (float)__ldg(xp + 2);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int r = 3 * a + c;
            float re[NF], im[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                re[f] = v[c][0];
                im[f] = 0.f;
            }
            // sectors s and NTH - s: shared cosines, opposite sines
#pragma unroll
            for (int s = 1; 2 * s < NTH; ++s) {
                const float sum = v[c][s] + v[c][NTH - s], dif = v[c][s] - v[c][NTH - s];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    re[f] += sum * args.tw[(f * s) % NTH].x;
                    im[f] -= dif * args.tw[(f * s) % NTH].y;
                }
            }
            if ((NTH & 1) == 0) {
#pragma unroll
                for (int f = 0; f < NF; ++f) re[f] += (f & 1) ? -v[c][NTH / 2] : v[c][NTH / 2];
            }
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const long long o = ((long long)f * J.nc + j) * J.ldk;
                const float vr = re[f] * scale, vi = im[f] * scale;
                const bf16 hr = __float2bfloat16_rn(vr), hi = __float2bfloat16_rn(vi);
                J.h[o + r] = hr;
                J.l[o + r] = __float2bfloat16_rn(vr - __bfloat162float(hr));
                J.h[o + n3 + r] = hi;
                J.l[o + n3 + r] = __float2bfloat16_rn(vi - __bfloat162float(hi));
            }
        }
    }
}

// Thread per (representative a, component c) of one column: the 2 nf spectrum
// values of its row in registers, the twiddles constant operands (NTH known at
// compile time).  The rotation R_s mixes components 0 and 1, which sit on
// neighbouring lanes: a warp takes 10 representatives on lanes 0 .. 29 (lanes
// 30, 31 idle), so the pair never straddles two warps.
template <int NTH, class TO>
__global__ void __launch_bounds__(192) idft_nth(const __grid_constant__ DftArgs args) {
    constexpr int NF = NTH / 2 + 1;
    const DftJob& J = args.j[blockIdx.y];
    const int j = blockIdx.x;
    if (j >= J.nc) return;
    const int n3 = 3 * J.nb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const float* yh = reinterpret_cast<const float*>(J.x) + (long long)j * J.ldk;
    const long long plane = (long long)J.nc * J.ldk;
    TO* y = reinterpret_cast<TO*>(J.y) + (long long)j * J.ldy;
    const int c = lane % 3;
    for (int a0 = 10 * warp; a0 < J.nb; a0 += 10 * nw) {
        const int a = a0 + lane / 3;
        const bool act = lane < 30 && a < J.nb;
        const int r = 3 * a + c;
        float yr[NF], yi[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const float wgt = (f == 0 || 2 * f == NTH) ? 1.f : 2.f;
            yr[f] = act ? wgt * yh[f * plane + r] : 0.f;
            yi[f] = act ? wgt * yh[f * plane + n3 + r] : 0.f;
        }
        const int* pa = J.panel + (act ? a : 0) * NTH;
        // the sector loop rolled: the twiddle index f s mod NTH is the same on
        // every lane, so the twiddles are broadcast constant-cache loads, and the
        // thread holds only its 2 NF spectrum values
        // y~_s = A_s - B_s and y~_{NTH-s} = A_s + B_s with A_s = sum_f cos(2 pi f s / NTH) y^r_f and
        // B_s = sum_f sin(2 pi f s / NTH) y^i_f: the two sectors from one pair of sums
        auto emit = [&](int s, float v) {
            // partner component: c = 0 <-> 1 (c = 2 keeps its own value)
            const float w = __shfl_sync(0xffffffffu, v, c == 0 ? lane + 1 : (c == 1 ? lane - 1 : lane));
            const float cs = args.tw[s].x, sn = args.tw[s].y;
            const float o = c == 0 ? cs * v - sn * w : (c == 1 ? sn * w + cs * v : v);
            if (act) {
                const long long row = 3LL * __ldg(pa + s) + c;
                y[row] = (TO)o;
                if (J.h) {
                    const long long e = row * J.hrs + (long long)j * J.hcs;
                    const bf16 h = __float2bfloat16_rn(o);
                    J.h[e] = h;
                    J.l[e] = __float2bfloat16_rn(o - __bfloat162float(h));
                }
            }
        };
#pragma unroll 1
        for (int s = 0; 2 * s <= NTH; ++s) {
            float A = 0.f, B = 0.f;
            int k = 0;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const float2 t = args.tw[k];
                A += t.x * yr[f];
                B += t.y * yi[f];
                k += s;
                if (k >= NTH) k -= NTH;
            }
            emit(s, A - B);
            if (s > 0 && 2 * s < NTH) emit(NTH - s, A + B);
        }
    }
}

// C^_f in FP32 for a compile-time sector count (thread: row r; blockIdx.y: column)
template <int NTH>
__global__ void chat_nth(const __grid_constant__ ChatArgs args, const __grid_constant__ DftArgs tw) {
    constexpr int NF = NTH / 2 + 1;
    const ChatJob& J = args.j[blockIdx.z];
    const int n3 = 3 * args.nb;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n3) return;
    const int c = blockIdx.y, b = c / 3, be = c % 3;
    const int* pb = J.panel + b * NTH;
    float re[NF], im[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) re[f] = im[f] = 0.f;
#pragma unroll
    for (int d = 0; d < NTH; ++d) {
        const float* col = J.T0 + r + (long long)(3 * pb[d]) * n3;
        const float cs = tw.tw[d].x, sn = tw.tw[d].y;
        float v;  // (T0 R_d)[r, 3 q + be]
        if (be == 2) v = col[2LL * n3];
        else if (be == 0) v = cs * col[0] + sn * col[n3];
        else v = -sn * col[0] + cs * col[n3];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            re[f] += v * tw.tw[(f * d) % NTH].x;
            im[f] += v * tw.tw[(f * d) % NTH].y;
        }
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) J.C[(long long)f * n3 * n3 + (long long)c * n3 + r] = make_float2(re[f], im[f]);
}

int gj_cluster(int n) {
    // shared memory of one CTA: its columns, two pivot columns and the index
    // arrays; two CTAs per block where they fit (measured faster than four)
    for (int cl : {2, 4}) {
        const int w = (n + cl - 1) / cl;
        const size_t bytes = (size_t)n * w * sizeof(float2) + 3 * n * sizeof(float2) + (2 + 2 * n) * sizeof(int);
        if (bytes <= 220 * 1024) return cl;
    }
    return 0;
}

size_t gj_smem(int n, int cl) {
    const int w = (n + cl - 1) / cl;
    return (size_t)n * w * sizeof(float2) + 3 * n * sizeof(float2) + (2 + 2 * n) * sizeof(int);
}

// The dynamic shared memory limits of the kernels that need more than 48 KB, set
// once per process to the largest size any launch asks for: concurrent host
// threads launch blocks of different orders, and a per-launch setting could
// lower the limit between another thread's setting and its launch.
constexpr int FT_SMEM_MAX = 220 * 1024;
void set_smem_limits() {
    static std::once_flag once;
    std::call_once(once, [] {
        CUDA_CHECK(cudaFuncSetAttribute(gj_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, FT_SMEM_MAX));
        CUDA_CHECK(cudaFuncSetAttribute(gj_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, FT_SMEM_MAX));
    });
}

}  // namespace

bool fourier_supported(const TubeSymmetry& sym) {
    return sym.ok && sym.nth >= 2 && sym.nth <= FT_MAX_SECTORS && 3 * sym.nb <= FT_MAX_ORDER &&
           gj_cluster(3 * sym.nb) > 0;
}

void fourier_build(const std::vector<FourierTube*>& fts, const std::vector<const TubeSymmetry*>& syms,
                   const std::vector<const float*>& T0s, const MixedCtx& cx) {
    // tubes of equal sector count and block order go through the same launches
    std::map<std::pair<int, int>, std::vector<size_t>> by;
    for (size_t k = 0; k < fts.size(); ++k) {
        const TubeSymmetry& S = *syms[k];
        if (!fourier_supported(S)) fail(SQBEM_ERR_ARG, "fourier_build: tube outside the Fourier path's limits");
        FourierTube& F = *fts[k];
        F.nth = S.nth;
        F.nb = S.nb;
        F.nf = S.nth / 2 + 1;
        F.n3 = 3 * S.nb;
        F.m2 = 2 * F.n3;
        F.ldk = (F.m2 + 7) / 8 * 8;
        F.nt = 3 * S.nb * S.nth;
        F.panel.alloc(S.panel.size(), cx.st);
        F.panel.upload(S.panel.data(), S.panel.size());
        std::vector<float2> tw(S.nth);
        for (int i = 0; i < S.nth; ++i)
            tw[i] = make_float2((float)std::cos(TWO_PI * i / S.nth), (float)std::sin(TWO_PI * i / S.nth));
        F.tw.alloc(S.nth, cx.st);
        F.tw.upload(tw.data(), S.nth);
        const size_t rf = (size_t)F.nf * F.m2 * F.ldk;
        F.Ah.alloc(rf, cx.st);
        F.Al.alloc(rf, cx.st);
        by[{S.nth, S.nb}].push_back(k);
    }
    for (const auto& kv : by) {
        const int nth = kv.first.first, nb = kv.first.second, n3 = 3 * nb, nf = nth / 2 + 1;
        const std::vector<size_t>& ids = kv.second;
        DevBuf<float2> C(ids.size() * nf * (size_t)n3 * n3, cx.st);
        for (size_t i0 = 0; i0 < ids.size(); i0 += FT_JOBS) {
            ChatArgs a;
            a.n = (int)std::min<size_t>(FT_JOBS, ids.size() - i0);
            a.nth = nth; a.nb = nb; a.nf = nf;
            for (int d = 0; d < nth; ++d) a.tw[d] = make_double2(std::cos(TWO_PI * d / nth), std::sin(TWO_PI * d / nth));
            for (int q = 0; q < a.n; ++q) {
                const size_t k = ids[i0 + q];
                a.j[q] = {T0s[k], fts[k]->panel.get(), C.get() + (i0 + q) * nf * (size_t)n3 * n3};
            }
            const double cby = 4.0 * 9.0 * a.n * nb * (double)nb * nth + 8.0 * a.n * nf * (double)n3 * n3;
            const dim3 cg3(ceil_div(n3, 64), n3, a.n);
            DftArgs tw;
            for (int d = 0; d < nth; ++d)
                tw.tw[d] = make_float2((float)std::cos(TWO_PI * d / nth), (float)std::sin(TWO_PI * d / nth));
            if (nth == 24) TIMED_LAUNCH("fourier_inverse", 0.0, cby, chat_nth<24>, cg3, 64, 0, cx.st, a, tw);
            else if (nth == 30) TIMED_LAUNCH("fourier_inverse", 0.0, cby, chat_nth<30>, cg3, 64, 0, cx.st, a, tw);
            else if (nth == 36) TIMED_LAUNCH("fourier_inverse", 0.0, cby, chat_nth<36>, cg3, 64, 0, cx.st, a, tw);
            else TIMED_LAUNCH("fourier_inverse", 0.0, cby, chat_kernel, cg3, 64, 0, cx.st, a);
        }
        const int cl = gj_cluster(n3);
        const size_t smem = gj_smem(n3, cl);
        const int nblk_all = (int)(ids.size() * nf);
        for (int b0 = 0; b0 < nblk_all; b0 += GJ_MAXB) {
            GjArgs g;
            g.n = n3;
            g.w = (n3 + cl - 1) / cl;
            g.nblk = std::min(GJ_MAXB, nblk_all - b0);
            g.flag = cx.flag;
            RfArgs r;
            r.n = n3;
            r.nblk = g.nblk;
            for (int b = 0; b < g.nblk; ++b) {
                const int gb = b0 + b;
                const size_t k = ids[gb / nf];
                const int f = gb % nf;
                g.C[b] = C.get() + (size_t)gb * n3 * n3;
                r.C[b] = g.C[b];
                r.hi[b] = fts[k]->Ah.get() + (size_t)f * fts[k]->m2 * fts[k]->ldk;
                r.lo[b] = fts[k]->Al.get() + (size_t)f * fts[k]->m2 * fts[k]->ldk;
                r.ldk = fts[k]->ldk;
            }
            // credited: 8 n^3 FP32 flops per complex inversion; bytes: the block read and written
            const double gfl = 8.0 * g.nblk * (double)n3 * n3 * n3, gby = 16.0 * g.nblk * (double)n3 * n3;
            set_smem_limits();
            if (cl == 2) TIMED_LAUNCH("fourier_inverse", gfl, gby, gj_kernel<2>, 2 * g.nblk, GJ_THREADS, smem, cx.st, g);
            else TIMED_LAUNCH("fourier_inverse", gfl, gby, gj_kernel<4>, 4 * g.nblk, GJ_THREADS, smem, cx.st, g);
            const int t = ceil_div(2 * n3, 32);
            TIMED_LAUNCH("fourier_inverse", 0.0, g.nblk * (8.0 * n3 * n3 + 16.0 * n3 * n3), realform_kernel,
                         dim3(t, t, g.nblk), dim3(32, 8), 0, cx.st, r);
        }
    }
}

void fourier_solve(const std::vector<FourierJob>& jobs, const MixedCtx& cx) {
    if (jobs.empty()) return;
    const bool in64 = jobs[0].x64 != nullptr, out64 = jobs[0].y64 != nullptr;
    for (const FourierJob& J : jobs)
        if ((J.x64 != nullptr) != in64 || (J.y64 != nullptr) != out64 || !J.ft)
            fail(SQBEM_ERR_ARG, "fourier_solve: mixed precisions in one call");
    // per job: X^ (split) and Y^ (FP32), nf planes of ldk x nc each
    std::vector<DevBuf<bf16>> xh(jobs.size()), xl(jobs.size());
    std::vector<DevBuf<float>> yh(jobs.size());
    for (size_t k = 0; k < jobs.size(); ++k) {
        const FourierTube& F = *jobs[k].ft;
        const size_t sz = (size_t)F.nf * F.ldk * jobs[k].nc;
        xh[k].alloc(sz, cx.st);
        xl[k].alloc(sz, cx.st);
        yh[k].alloc(sz, cx.st);
    }
    auto dft_job = [&](size_t k, bool forward) {
        const FourierJob& J = jobs[k];
        const FourierTube& F = *J.ft;
        DftJob d;
        d.panel = F.panel.get();
        d.tw = F.tw.get();
        d.nc = J.nc; d.nb = F.nb; d.nth = F.nth; d.nf = F.nf; d.ldk = F.ldk;
        if (forward) {
            d.x = in64 ? (const void*)J.x64 : (const void*)J.x32;
            d.ldx = J.ldx;
            d.y = nullptr; d.ldy = 0;
            d.h = xh[k].get(); d.l = xl[k].get(); d.hrs = 1; d.hcs = 0;
        } else {
            d.x = yh[k].get(); d.ldx = 0;
            d.y = out64 ? (void*)J.y64 : (void*)J.y32;
            d.ldy = J.ldy;
            d.h = J.yh; d.l = J.yl; d.hrs = J.srs; d.hcs = J.scs;
        }
        return d;
    };
    int maxnc = 0;
    for (const FourierJob& J : jobs) maxnc = std::max(maxnc, J.nc);
    // credited bytes of a transform: X (or Y) once, X^ (or Y^) once
    auto dft_bytes = [&](size_t i0, int n, bool forward) {
        double b = 0;
        for (int q = 0; q < n; ++q) {
            const FourierJob& J = jobs[i0 + q];
            const double io = (double)J.ft->nt * J.nc * ((forward ? in64 : out64) ? 8.0 : 4.0);
            const double hat = (double)J.ft->nf * J.ft->m2 * J.nc * (forward ? 4.0 : 4.0);
            b += io + hat + (!forward && J.yh ? 4.0 * J.ft->nt * J.nc : 0.0);
        }
        return b;
    };
    // launches of up to FT_JOBS consecutive jobs with the same sector count
    auto batches = [&]() {
        std::vector<std::pair<size_t, int>> b;
        for (size_t i0 = 0; i0 < jobs.size();) {
            int n = 1;
            while (i0 + n < jobs.size() && n < FT_JOBS && jobs[i0 + n].ft->nth == jobs[i0].ft->nth) ++n;
            b.push_back({i0, n});
            i0 += n;
        }
        return b;
    };
    auto set_tw = [&](DftArgs& a, int nth) {
        for (int k = 0; k < nth; ++k)
            a.tw[k] = make_float2((float)std::cos(TWO_PI * k / nth), (float)std::sin(TWO_PI * k / nth));
    };
    for (const auto& bt : batches()) {
        const size_t i0 = bt.first;
        DftArgs a;
        a.n = bt.second;
        for (int q = 0; q < a.n; ++q) a.j[q] = dft_job(i0 + q, true);
        const int nth = jobs[i0].ft->nth;
        set_tw(a, nth);
        const double by = dft_bytes(i0, a.n, true);
        const dim3 gd(maxnc, a.n);
        if (in64) {
            if (nth == 24) TIMED_LAUNCH("fourier_dft", 0.0, by, (fdft_rep<24, double>), gd, 64, 0, cx.st, a);
            else if (nth == 30) TIMED_LAUNCH("fourier_dft", 0.0, by, (fdft_rep<30, double>), gd, 64, 0, cx.st, a);
            else if (nth == 36) TIMED_LAUNCH("fourier_dft", 0.0, by, (fdft_rep<36, double>), gd, 64, 0, cx.st, a);
            else TIMED_LAUNCH("fourier_dft", 0.0, by, fdft_kernel<double>, gd, 192, 0, cx.st, a);
        } else {
            if (nth == 24) TIMED_LAUNCH("fourier_dft", 0.0, by, (fdft_rep<24, float>), gd, 64, 0, cx.st, a);
            else if (nth == 30) TIMED_LAUNCH("fourier_dft", 0.0, by, (fdft_rep<30, float>), gd, 64, 0, cx.st, a);
            else if (nth == 36) TIMED_LAUNCH("fourier_dft", 0.0, by, (fdft_rep<36, float>), gd, 64, 0, cx.st, a);
            else TIMED_LAUNCH("fourier_dft", 0.0, by, fdft_kernel<float>, gd, 192, 0, cx.st, a);
        }
    }
    // one GEMM of order 2 n3 per job and frequency: Y^_f = inv(C^_f) X^_f in real form
    std::vector<TcProblem> P;
    std::vector<TcOperands> O;
    for (size_t k = 0; k < jobs.size(); ++k) {
        const FourierTube& F = *jobs[k].ft;
        const int nc = jobs[k].nc;
        for (int f = 0; f < F.nf; ++f) {
            const size_t ao = (size_t)f * F.m2 * F.ldk, xo = (size_t)f * F.ldk * nc;
            TcProblem p;
            p.M = F.m2; p.N = nc; p.K = F.m2;
            p.alpha = 1.f; p.beta = 0.f;
            p.C = yh[k].get() + xo; p.c_rs = 1; p.c_cs = F.ldk;
            TcOperands o;
            o.A = {const_cast<bf16*>(F.Ah.get()) + ao, const_cast<bf16*>(F.Al.get()) + ao, F.m2, F.m2, F.ldk};
            o.B = {xh[k].get() + xo, xl[k].get() + xo, nc, F.m2, F.ldk};
            P.push_back(p);
            O.push_back(o);
        }
    }
    tc_gemm(P, O, cx.err, nullptr, cx.st);
    for (const auto& bt : batches()) {
        const size_t i0 = bt.first;
        DftArgs a;
        a.n = bt.second;
        for (int q = 0; q < a.n; ++q) a.j[q] = dft_job(i0 + q, false);
        const int nth = jobs[i0].ft->nth;
        set_tw(a, nth);
        const double by = dft_bytes(i0, a.n, false);
        const dim3 gs(maxnc, a.n), bs(192);
        const size_t sm = 0;
        if (out64) {
            if (nth == 24) TIMED_LAUNCH("fourier_dft", 0.0, by, (idft_nth<24, double>), gs, bs, sm, cx.st, a);
            else if (nth == 30) TIMED_LAUNCH("fourier_dft", 0.0, by, (idft_nth<30, double>), gs, bs, sm, cx.st, a);
            else if (nth == 36) TIMED_LAUNCH("fourier_dft", 0.0, by, (idft_nth<36, double>), gs, bs, sm, cx.st, a);
            else TIMED_LAUNCH("fourier_dft", 0.0, by, idft_kernel<double>, dim3(maxnc, a.n), 64, 0, cx.st, a);
        } else {
            if (nth == 24) TIMED_LAUNCH("fourier_dft", 0.0, by, (idft_nth<24, float>), gs, bs, sm, cx.st, a);
            else if (nth == 30) TIMED_LAUNCH("fourier_dft", 0.0, by, (idft_nth<30, float>), gs, bs, sm, cx.st, a);
            else if (nth == 36) TIMED_LAUNCH("fourier_dft", 0.0, by, (idft_nth<36, float>), gs, bs, sm, cx.st, a);
            else TIMED_LAUNCH("fourier_dft", 0.0, by, idft_kernel<float>, dim3(maxnc, a.n), 64, 0, cx.st, a);
        }
    }
}

}  // namespace sqbem
