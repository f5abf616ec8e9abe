// tc_gemm.cu -- persistent grouped GEMM on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory, operands staged by TMA).
//
// CTA = 6 warps, one CTA per SM:
//   warp 0     TMA producer: for every k-block of 64 loads the four 128 x 64 BF16
//              tiles (A_hi, A_lo, B_hi, B_lo; 128-byte swizzle) into a stage of a
//              3-stage shared-memory ring, completion tracked by mbarriers.
//   warp 1     allocates 256 TMEM columns (two 128 x 128 FP32 accumulators) and
//              issues, from one lane, 3 x 4 tcgen05.mma (M = 128, N = 128,
//              K = 16) per k-block: hi*hi + hi*lo + lo*hi; tcgen05.commit frees
//              the stage and, after the last k-block, hands the accumulator to
//              the epilogue.
//   warps 2-5  epilogue: tcgen05.ld (32 lanes x 32 columns per instruction; warp
//              w reads TMEM lanes 32 (w % 4) ..), alpha / beta, FP32 store and
//              optional split-BF16 stores, then release the accumulator.
// Two accumulators let the epilogue of tile t overlap the MMAs of tile t + 1.
// Tiles of all problems are enumerated in one list; CTA b takes tiles b,
// b + gridDim, ...  Every mbarrier wait is bounded (sqbem_set_limits; by default
// about 2 s of SM clock); on expiry the kernel raises *err, drains its own
// copies and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "tc_gemm.cuh"

namespace sqbem {

namespace {

constexpr int BM = 128, BK = 64;
constexpr int A_TILE = BM * BK * 2;  // 16 KB per A plane of a stage
constexpr int NTHREADS = 192;

// Tile variants of the kernel; the autotuner (tune_gemm.py) picks one per shape
// class of the launches.  A stage holds A_hi, A_lo (128 x 64 each) and B_hi, B_lo
// (BN x 64 each); the two TMEM accumulators take 2 BN columns.
template <int BN_, int STAGES_>
struct Tile {
    static constexpr int BN = BN_, STAGES = STAGES_;
    static constexpr int B_TILE = BN * BK * 2;
    static constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
    static constexpr int TMEM_COLS = 2 * BN;
    // instruction descriptor: D = F32, A = B = BF16, both K-major, N = BN, M = BM
    static constexpr uint32_t IDESC =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
    static_assert(SMEM_BYTES <= 227 * 1024, "shared memory per CTA");
    static_assert(TMEM_COLS <= 512, "tensor memory columns");
};
using TileA = Tile<128, 3>;  // variant 0: 128 x 128 tiles, 3 stages of 64 KB
using TileB = Tile<256, 2>;  // variant 1: 128 x 256 tiles, 2 stages of 96 KB
// Waits that keep the CTA alive until its own copies and MMAs have landed (before
// shared memory and TMEM are given up) use the default limit, never the
// caller's: leaving earlier would let a copy write into released memory.
constexpr long long DRAIN_CYCLES = DEFAULT_WAIT_CYCLES;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of the given parity; false (and *err = 1) after
// `limit` SM cycles or if another role already gave up.  The error flag (a
// global load) and the clock are polled only every 64 tries: a global load
// inside every poll would delay the reaction to a completed phase by an L2 round
// trip.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, long long limit) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    for (int it = 1;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 63) == 0) {
            if (*(volatile int*)err) return false;
            if (clock64() - t0 > limit) {
                atomicExch(err, 1);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)map) : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 32 consecutive FP32 columns from tensor memory.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Problems of one launch travel as a __grid_constant__ kernel parameter (TMA
// reads the tensor maps straight from parameter space; no device copies, so a
// launch can be captured into a CUDA graph).
#ifndef SQBEM_TC_MAXP
#define SQBEM_TC_MAXP 48
#endif
constexpr int MAXP = SQBEM_TC_MAXP;
struct KArgs {
    int nprob;
    int total_tiles;
    long long wait;  // SM cycles per bounded wait (gemm_wait_cycles())
    int stall;       // test hook (sqbem_test_gemm_stall): CTA 0's MMA issuer first waits on a
                     // barrier that nothing arrives on, so that wait runs out
    int* err;
    int* flag;
    TcProblem probs[MAXP];
    CUtensorMap maps[4 * MAXP];  // A_hi, A_lo, B_hi, B_lo per problem
};

__device__ __forceinline__ int find_problem(const TcProblem* probs, int nprob, int t) {
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {  // last problem with tile_start <= t
        const int mid = (lo + hi + 1) >> 1;
        if (probs[mid].tile_start <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <class T>
__global__ void __launch_bounds__(NTHREADS, 1) tc_gemm_kernel(const __grid_constant__ KArgs args) {
    constexpr int BN = T::BN, STAGES = T::STAGES, STAGE_BYTES = T::STAGE_BYTES, B_TILE = T::B_TILE;
    constexpr int TMEM_COLS = T::TMEM_COLS;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);
    const uint32_t tfull0 = smem_u32(bars + 2 * STAGES), tempty0 = smem_u32(bars + 2 * STAGES + 2);
    const uint32_t done_bar = smem_u32(bars + 2 * STAGES + 4);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 5);
    const uint32_t stall_bar = smem_u32(bars + 2 * STAGES + 6);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int* err = args.err;
    const long long wait = args.wait;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, 128);
        }
        mbar_init(done_bar, 1);
        mbar_init(stall_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        int s = 0;
        uint32_t ph = 0;
        int armed[STAGES] = {};
        int last_p = -1;
        (void)last_p;
        for (int t = blockIdx.x; t < args.total_tiles; t += gridDim.x) {
            const int p = find_problem(args.probs, args.nprob, t);
            const TcProblem& P = args.probs[p];
            const CUtensorMap* m = &args.maps[4 * p];
            if (p != last_p) {
                for (int j = 0; j < 4; ++j) prefetch_tensormap(m + j);
                last_p = p;
            }
            const int local = t - P.tile_start;
            const int tm = local / P.tiles_n, tn = local % P.tiles_n;
            const int nkb = (P.K + BK - 1) / BK;
            const bool three = P.products != 2;  // two products: A_lo is not read
            bool ok = true;
            for (int kb = 0; kb < nkb; ++kb) {
                if (!mbar_wait(empty0 + 8 * s, ph ^ 1, err, wait)) { ok = false; break; }
                const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
                const uint32_t fb = full0 + 8 * s;
                mbar_expect_tx(fb, three ? STAGE_BYTES : STAGE_BYTES - A_TILE);
                tma_load_2d(st, m + 0, kb * BK, tm * BM, fb);
                if (three) tma_load_2d(st + A_TILE, m + 1, kb * BK, tm * BM, fb);
                tma_load_2d(st + 2 * A_TILE, m + 2, kb * BK, tn * BN, fb);
                tma_load_2d(st + 2 * A_TILE + B_TILE, m + 3, kb * BK, tn * BN, fb);
                armed[s] += 1;
                if (++s == STAGES) { s = 0; ph ^= 1; }
            }
            if (!ok) break;
        }
        // drain: every armed stage must have completed before the CTA exits
        for (int q = 0; q < STAGES; ++q)
            if (armed[q] > 0) {
                const uint32_t par = (uint32_t)((armed[q] - 1) & 1);
                const long long t0 = clock64();
                while (!mbar_try(full0 + 8 * q, par) && clock64() - t0 < DRAIN_CYCLES) {
                }
            }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        int s = 0;
        uint32_t ph = 0;
        int acc = 0;
        uint32_t aph = 0;
        // the test hook's wait: nothing arrives on stall_bar, so it ends by the limit
        const bool stalled = args.stall && blockIdx.x == 0 && !mbar_wait(stall_bar, 0, err, wait);
        for (int t = stalled ? args.total_tiles : blockIdx.x; t < args.total_tiles; t += gridDim.x) {
            const int p = find_problem(args.probs, args.nprob, t);
            const int nkb = (args.probs[p].K + BK - 1) / BK;
            const bool three = args.probs[p].products != 2;
            if (!mbar_wait(tempty0 + 8 * acc, aph ^ 1, err, wait)) break;
            tc_fence_after();
            const uint32_t d = tmem_base + (uint32_t)(acc * BN);
            bool ok = true;
            for (int kb = 0; kb < nkb; ++kb) {
                if (!mbar_wait(full0 + 8 * s, ph, err, wait)) { ok = false; break; }
                tc_fence_after();
                const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
                const uint64_t ah = smem_desc(st), al = smem_desc(st + A_TILE);
                const uint64_t bh = smem_desc(st + 2 * A_TILE), bl = smem_desc(st + 2 * A_TILE + B_TILE);
#pragma unroll
                for (int k = 0; k < BK / 16; ++k) {
                    const uint64_t off = (uint64_t)(k * 32) >> 4;  // 16 BF16 = 32 bytes along K
                    mma_bf16(d, ah + off, bh + off, T::IDESC, (kb > 0 || k > 0) ? 1u : 0u);
                    mma_bf16(d, ah + off, bl + off, T::IDESC, 1u);
                    if (three) mma_bf16(d, al + off, bh + off, T::IDESC, 1u);
                }
                mma_commit(empty0 + 8 * s);
                if (++s == STAGES) { s = 0; ph ^= 1; }
            }
            if (!ok) break;
            mma_commit(tfull0 + 8 * acc);
            if (++acc == 2) { acc = 0; aph ^= 1; }
        }
        // all MMAs issued by this CTA complete before TMEM is released
        mma_commit(done_bar);
        const long long t0 = clock64();
        while (!mbar_try(done_bar, 0) && clock64() - t0 < DRAIN_CYCLES) {
        }
    } else if (warp >= 2) {
        // ---------------- epilogue
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        int acc = 0;
        uint32_t aph = 0;
        int any_big = 0;
        for (int t = blockIdx.x; t < args.total_tiles; t += gridDim.x) {
            const int p = find_problem(args.probs, args.nprob, t);
            const TcProblem& P = args.probs[p];
            const int local = t - P.tile_start;
            const int tm = local / P.tiles_n, tn = local % P.tiles_n;
            // the problem's fields once per tile, in registers (parameter-space reads
            // inside the element loop cost ~30 cycles each)
            const int m = tm * BM + row;
            const bool row_ok = m < P.M;
            const int N = P.N;
            const float alpha = P.alpha, beta = P.beta;
            const bool chk = P.check_unit != 0;
            float* const Cp = P.C;
            const long long crs = P.c_rs, ccs = P.c_cs;
            bf16* const Oh = P.O_hi;
            bf16* const Ol = P.O_lo;
            const long long ors = P.o_rs, ocs = P.o_cs;
            bf16* const Ph = P.P_hi;
            bf16* const Pl = P.P_lo;
            const long long prs = P.p_rs, pcs = P.p_cs;
            const bool rd = Cp && beta != 0.f && row_ok;
            // C of a 32-column chunk is read before any of it is written: a load
            // issued after the previous column's store would wait for it (the
            // compiler cannot rule out aliasing), one round trip per column.
            // The first chunk is fetched before the accumulator is ready.
            float cnext[32];
            auto load_c = [&](int c0) {
                const int n0 = tn * BN + c0;
                const int cnt = min(32, N - n0);
                const float* c = Cp + (long long)m * crs + (long long)n0 * ccs;
#pragma unroll
                for (int j = 0; j < 32; ++j) cnext[j] = j < cnt ? c[(long long)j * ccs] : 0.f;
            };
            if (rd) load_c(0);
            if (!mbar_wait(tfull0 + 8 * acc, aph, err, wait)) break;
            tc_fence_after();
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                float cv[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) cv[j] = cnext[j];
                if (rd && c0 + 32 < BN && tn * BN + c0 + 32 < N) load_c(c0 + 32);
                float v[32];
                tmem_ld32(tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * BN + c0), v);
                const int n0 = tn * BN + c0;
                const int cnt = min(32, N - n0);
                if (!row_ok || cnt <= 0) continue;
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = rd ? fmaf(beta, cv[j], alpha * v[j]) : alpha * v[j];
                if (Cp) {
                    float* const c = Cp + (long long)m * crs + (long long)n0 * ccs;
                    if (ccs == 1 && cnt == 32 && ((uintptr_t)c & 15) == 0) {
                        // this thread's 32 columns are contiguous (row-major C)
#pragma unroll
                        for (int j = 0; j < 32; j += 4)
                            *reinterpret_cast<float4*>(c + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < cnt) c[(long long)j * ccs] = v[j];
                    }
                }
                if (chk)
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (j < cnt && !(fabsf(v[j]) <= 1.f)) any_big = 1;
                // split outputs: 16-byte vectors where the thread's columns are contiguous
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    bf16* const H = w == 0 ? Oh : Ph;
                    bf16* const Lo = w == 0 ? Ol : Pl;
                    if (!H) continue;
                    const long long rs = w == 0 ? ors : prs, cs = w == 0 ? ocs : pcs;
                    const long long base = (long long)m * rs + (long long)n0 * cs;
                    if (cs == 1 && cnt == 32 && ((base & 7) == 0) && (((uintptr_t)H & 15) == 0) &&
                        (((uintptr_t)Lo & 15) == 0)) {
#pragma unroll
                        for (int j = 0; j < 32; j += 8) {
                            uint4 hv, lv;
                            bf16* hp = reinterpret_cast<bf16*>(&hv);
                            bf16* lp = reinterpret_cast<bf16*>(&lv);
#pragma unroll
                            for (int q = 0; q < 8; ++q) {
                                const bf16 h = __float2bfloat16_rn(v[j + q]);
                                hp[q] = h;
                                lp[q] = __float2bfloat16_rn(v[j + q] - __bfloat162float(h));
                            }
                            *reinterpret_cast<uint4*>(H + base + j) = hv;
                            *reinterpret_cast<uint4*>(Lo + base + j) = lv;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            if (j >= cnt) break;
                            const bf16 h = __float2bfloat16_rn(v[j]);
                            const long long o = base + (long long)j * cs;
                            H[o] = h;
                            Lo[o] = __float2bfloat16_rn(v[j] - __bfloat162float(h));
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(tempty0 + 8 * acc);
            if (++acc == 2) { acc = 0; aph ^= 1; }
        }
        if (any_big && args.flag) atomicOr(args.flag, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS)
                     : "memory");
}

// ---------------------------------------------------------------- split conversion
__global__ void split_kernel(const float* __restrict__ src, long long s_rs, long long s_cs, int rows, int cols,
                             bf16* __restrict__ hi, bf16* __restrict__ lo, long long d_rs, long long d_cs) {
    // iterate with the destination's contiguous index fastest
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)rows * cols) return;
    int r, c;
    if (d_rs == 1) { r = (int)(t % rows); c = (int)(t / rows); }
    else { c = (int)(t % cols); r = (int)(t / cols); }
    const float x = src[r * s_rs + c * s_cs];
    const bf16 h = __float2bfloat16_rn(x);
    hi[r * d_rs + c * d_cs] = h;
    lo[r * d_rs + c * d_cs] = __float2bfloat16_rn(x - __bfloat162float(h));
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

void get_encode() {
    std::call_once(g_encode_once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        CUDA_CHECK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) fail(SQBEM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
}

// Tensor map of a K-major BF16 plane: rows x k, row pitch ld elements, boxes of
// box_rows rows x 64 k with 128-byte swizzle, zero fill outside the matrix.
CUtensorMap make_map(const bf16* base, int rows, int k, long long ld, int box_rows) {
    if (((uintptr_t)base & 15) != 0 || (ld * 2) % 16 != 0 || rows <= 0 || k <= 0)
        fail(SQBEM_ERR_ARG, "tensor map: misaligned operand (ld %lld)", ld);
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
    cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(SQBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return m;
}

int g_num_sms = 0;
std::once_flag g_sms_once;
std::atomic<int> g_test_stalls{0};

}  // namespace

void split_convert(const float* src, long long s_rs, long long s_cs, int rows, int cols, bf16* hi, bf16* lo,
                   long long d_rs, long long d_cs, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return;
    LAUNCH(split_kernel, ceil_div((long long)rows * cols, 256), 256, 0, st, src, s_rs, s_cs, rows, cols, hi, lo, d_rs,
           d_cs);
}

// ---------------------------------------------------------------- variants and tuning
namespace {
struct VariantInfo {
    int bn, stages, smem;
    void (*kernel)(KArgs);
};
const VariantInfo kVariants[] = {
    {TileA::BN, TileA::STAGES, TileA::SMEM_BYTES, tc_gemm_kernel<TileA>},
    {TileB::BN, TileB::STAGES, TileB::SMEM_BYTES, tc_gemm_kernel<TileB>},
};
constexpr int NVARIANTS = (int)(sizeof(kVariants) / sizeof(kVariants[0]));

// The tuning table: rows "kmax nmax variant"; a launch takes the first row with
// K <= kmax and N <= nmax (its largest problem's K and N).  Read once from
// SQBEM_TC_TABLE or, by default, tuning/tc_gemm.txt next to the library's lib/
// folder; without a table every launch takes variant 0.  SQBEM_TC_VARIANT forces
// one variant for every launch (used by the tuner).
struct TableRow {
    int kmax, nmax, variant;
};
std::vector<TableRow> g_table;
int g_forced = -1;
std::once_flag g_table_once;

std::string default_table_path() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&tc_gemm_variants), &info) && info.dli_fname) {
        std::string lib(info.dli_fname);
        const size_t slash = lib.rfind('/');
        const std::string dir = slash == std::string::npos ? "." : lib.substr(0, slash);
        return dir + "/../tuning/tc_gemm.txt";
    }
    return "";
}

void load_table() {
    std::call_once(g_table_once, [] {
        if (const char* f = std::getenv("SQBEM_TC_VARIANT")) {
            const int v = std::atoi(f);
            if (v >= 0 && v < NVARIANTS) g_forced = v;
        }
        const char* env = std::getenv("SQBEM_TC_TABLE");
        const std::string path = env ? std::string(env) : default_table_path();
        FILE* fp = path.empty() ? nullptr : std::fopen(path.c_str(), "r");
        if (!fp) return;
        char line[256];
        while (std::fgets(line, sizeof line, fp)) {
            TableRow r;
            if (line[0] == '#') continue;
            if (std::sscanf(line, "%d %d %d", &r.kmax, &r.nmax, &r.variant) == 3 && r.variant >= 0 &&
                r.variant < NVARIANTS)
                g_table.push_back(r);
        }
        std::fclose(fp);
    });
}
}  // namespace

int tc_gemm_variants() { return NVARIANTS; }

void tc_gemm_variant_info(int v, int* bn, int* stages) {
    if (v < 0 || v >= NVARIANTS) fail(SQBEM_ERR_ARG, "tc_gemm: no variant %d", v);
    if (bn) *bn = kVariants[v].bn;
    if (stages) *stages = kVariants[v].stages;
}

int tc_gemm_choose(int kmax, int nmax) {
    load_table();
    if (g_forced >= 0) return g_forced;
    for (const TableRow& r : g_table)
        if (kmax <= r.kmax && nmax <= r.nmax) return r.variant;
    return 0;
}

void tc_gemm(const std::vector<TcProblem>& probs_in, const std::vector<TcOperands>& ops, int* err, int* flag,
             cudaStream_t st, int variant) {
    if (probs_in.size() != ops.size()) fail(SQBEM_ERR_ARG, "tc_gemm: operand count");
    get_encode();
    std::call_once(g_sms_once, [] {
        int dev = 0;
        CUDA_CHECK(cudaGetDevice(&dev));
        CUDA_CHECK(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
        for (const VariantInfo& v : kVariants)
            CUDA_CHECK(cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem));
    });
    if (variant < 0) {
        int kmax = 0, nmax = 0;
        for (const TcProblem& P : probs_in) {
            kmax = std::max(kmax, P.K);
            nmax = std::max(nmax, P.N);
        }
        variant = tc_gemm_choose(kmax, nmax);
    }
    if (variant >= NVARIANTS) fail(SQBEM_ERR_ARG, "tc_gemm: no variant %d", variant);
    const VariantInfo& V = kVariants[variant];
    KArgs a;
    auto h0 = std::chrono::steady_clock::now();
    auto flush = [&](double flops, double bytes) {
        if (a.nprob == 0) return;
        const int grid = std::min(a.total_tiles, g_num_sms);
        if (kstats_on()) {
            const double host_us =
                std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - h0).count();
            int mm = 0, mn = 0, mk = 0;
            for (int q = 0; q < a.nprob; ++q) {
                mm = std::max(mm, a.probs[q].M);
                mn = std::max(mn, a.probs[q].N);
                mk = std::max(mk, a.probs[q].K);
            }
            char note[160];
            std::snprintf(note, sizeof note, "nprob=%d tiles=%d grid=%d M=%d N=%d K=%d variant=%d host_us=%.1f",
                          a.nprob, a.total_tiles, grid, mm, mn, mk, variant, host_us);
            kstat_note(note);
        }
        TIMED_LAUNCH("tc_gemm", flops, bytes, V.kernel, grid, NTHREADS, V.smem, st, a);
        h0 = std::chrono::steady_clock::now();
    };
    a.nprob = 0;
    a.total_tiles = 0;
    a.err = err;
    a.flag = flag;
    a.wait = gemm_wait_cycles();
    a.stall = 0;
    int stalls = g_test_stalls.load();
    while (stalls > 0 && !g_test_stalls.compare_exchange_weak(stalls, stalls - 1)) {
    }
    if (stalls > 0) a.stall = 1;  // this call takes one requested stall
    double flops = 0, bytes = 0;
    for (size_t i = 0; i < probs_in.size(); ++i) {
        TcProblem P = probs_in[i];
        const TcOperands& o = ops[i];
        if (P.M <= 0 || P.N <= 0) continue;
        if (P.K <= 0) fail(SQBEM_ERR_ARG, "tc_gemm: K must be positive");
        if (P.products != 2 && P.products != 3) fail(SQBEM_ERR_ARG, "tc_gemm: 2 or 3 products");
        if (o.A.rows < P.M || o.A.k < P.K || o.B.rows < P.N || o.B.k < P.K)
            fail(SQBEM_ERR_ARG, "tc_gemm: operand smaller than the problem");
        if (a.nprob == MAXP) {
            flush(flops, bytes);
            a.nprob = 0;
            a.total_tiles = 0;
            flops = bytes = 0;
        }
        P.tiles_n = ceil_div(P.N, V.bn);
        P.tile_start = a.total_tiles;
        a.total_tiles += ceil_div(P.M, BM) * P.tiles_n;
        // maps cover exactly the problem's extent: rows beyond M / N and k beyond K read as zero
        a.maps[4 * a.nprob + 0] = make_map(o.A.hi, P.M, P.K, o.A.ld, BM);
        a.maps[4 * a.nprob + 1] = P.products == 2 ? a.maps[4 * a.nprob] : make_map(o.A.lo, P.M, P.K, o.A.ld, BM);
        a.maps[4 * a.nprob + 2] = make_map(o.B.hi, P.N, P.K, o.B.ld, V.bn);
        a.maps[4 * a.nprob + 3] = make_map(o.B.lo, P.N, P.K, o.B.ld, V.bn);
        a.probs[a.nprob++] = P;
        // tensor-pipe work: two or three BF16 products per element product
        flops += P.products * 2.0 * P.M * P.N * P.K;
        // algorithmic bytes: each operand plane once, C read (beta != 0) and
        // written, and every split-BF16 output pair (2 + 2 bytes per element)
        bytes += (P.products == 2 ? 2.0 : 4.0) * P.M * P.K + 4.0 * P.K * P.N +
                 ((P.C && P.beta != 0.f ? 4.0 : 0.0) + (P.C ? 4.0 : 0.0) + (P.O_hi ? 4.0 : 0.0) +
                  (P.P_hi ? 4.0 : 0.0)) * P.M * P.N;
    }
    flush(flops, bytes);
}

}  // namespace sqbem

using namespace sqbem;

namespace sqbem {
namespace {

// A stream of its own for one host-facing call, destroyed on every exit path.
struct CallStream {
    cudaStream_t s = nullptr;
    CallStream() { CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~CallStream() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

void gemm_host(int variant, int products, int M, int N, int K, float alpha, const float* A, int lda, const float* B,
               int ldb, float beta, float* C, int ldc) {
    if (M < 0 || N < 0 || K <= 0 || !A || !B || !C || lda < M || ldb < K || ldc < M ||
        (products != 2 && products != 3) || variant < -1 || variant >= NVARIANTS)
        fail(SQBEM_ERR_ARG, "gemm_mixed: bad arguments");
    if (M == 0 || N == 0) return;
    require_device();
    CallStream cs;
    const cudaStream_t st = cs.s;
    const long long ld = pad_ld(K);
    DevBuf<float> dA((size_t)lda * K, st), dB((size_t)ldb * N, st), dC((size_t)ldc * N, st);
    DevBuf<bf16> ah((size_t)M * ld, st), al((size_t)M * ld, st), bh((size_t)N * ld, st), bl((size_t)N * ld, st);
    DevBuf<int> err(1, st);
    err.zero();
    dA.upload(A, (size_t)lda * K);
    dB.upload(B, (size_t)ldb * N);
    dC.upload(C, (size_t)ldc * N);
    // A (col-major M x K) -> K-major rows; B (col-major K x N) -> K-major columns
    split_convert(dA.get(), 1, lda, M, K, ah.get(), al.get(), ld, 1, st);
    split_convert(dB.get(), 1, ldb, K, N, bh.get(), bl.get(), 1, ld, st);
    TcProblem P;
    P.M = M; P.N = N; P.K = K; P.alpha = alpha; P.beta = beta;
    P.C = dC.get(); P.c_rs = 1; P.c_cs = ldc;
    P.products = products;
    TcOperands o;
    o.A = {ah.get(), al.get(), M, K, ld};
    o.B = {bh.get(), bl.get(), N, K, ld};
    tc_gemm({P}, {o}, err.get(), nullptr, st, variant);
    int h_err = 0;
    err.download(&h_err, 1);
    dC.download(C, (size_t)ldc * N);
    CUDA_CHECK(cudaStreamSynchronize(st));
    if (h_err) fail(SQBEM_ERR_TIMEOUT, "gemm_mixed: a bounded wait in the tensor-core GEMM expired");
}

// deterministic pseudo-random BF16 planes in [-1, 1) for the timing entry point
__global__ void fill_planes_kernel(bf16* p, size_t n, unsigned seed) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    p[i] = __float2bfloat16_rn((float)(h & 0xffff) / 32768.f - 1.f);
}

}  // namespace
}  // namespace sqbem

extern "C" int sqbem_gemm_mixed(int M, int N, int K, float alpha, const float* A, int lda, const float* B, int ldb,
                                float beta, float* C, int ldc) {
    return guarded([&] { gemm_host(-1, 3, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc); });
}

extern "C" int sqbem_gemm_mixed_ex(int variant, int products, int M, int N, int K, float alpha, const float* A,
                                   int lda, const float* B, int ldb, float beta, float* C, int ldc) {
    return guarded([&] { gemm_host(variant, products, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc); });
}

extern "C" int sqbem_gemm_variants(int* count) {
    if (count) *count = NVARIANTS;
    return SQBEM_OK;
}

extern "C" int sqbem_gemm_timing(int variant, int products, int M, int N, int K, int count, float beta, int reps,
                                 double* seconds) {
    return guarded([&] {
        if (M <= 0 || N <= 0 || K <= 0 || count <= 0 || count > MAXP || reps <= 0 || !seconds ||
            (products != 2 && products != 3) || variant < -1 || variant >= NVARIANTS)
            fail(SQBEM_ERR_ARG, "gemm_timing: bad arguments");
        const long long ld = pad_ld(K);
        const double total = (double)count * (4.0 * ((double)M + N) * ld + 4.0 * (double)M * N);
        if (total > 16e9) fail(SQBEM_ERR_ARG, "gemm_timing: %.1f GB of operands exceed the 16 GB cap", total / 1e9);
        require_device();
        CallStream cs;
        const cudaStream_t st = cs.s;
        std::vector<DevBuf<bf16>> planes;
        std::vector<DevBuf<float>> cs_(count);
        std::vector<TcProblem> P(count);
        std::vector<TcOperands> O(count);
        for (int q = 0; q < count; ++q) {
            for (int w = 0; w < 4; ++w) {
                const size_t n = (size_t)(w < 2 ? M : N) * ld;
                planes.emplace_back(n, st);
                LAUNCH(fill_planes_kernel, ceil_div((long long)n, 256), 256, 0, st, planes.back().get(), n,
                       0x9e3779b9u * (unsigned)(4 * q + w + 1));
            }
            cs_[q].alloc((size_t)M * N, st);
            cs_[q].zero();
            TcProblem& p = P[q];
            p.M = M; p.N = N; p.K = K; p.alpha = 1.f; p.beta = beta;
            p.C = cs_[q].get(); p.c_rs = 1; p.c_cs = M;
            p.products = products;
            const size_t b = planes.size() - 4;
            O[q].A = {planes[b].get(), planes[b + 1].get(), M, K, ld};
            O[q].B = {planes[b + 2].get(), planes[b + 3].get(), N, K, ld};
        }
        DevBuf<int> err(1, st);
        err.zero();
        tc_gemm(P, O, err.get(), nullptr, st, variant);  // warm-up
        cudaEvent_t e0, e1;
        CUDA_CHECK(cudaEventCreate(&e0));
        CUDA_CHECK(cudaEventCreate(&e1));
        CUDA_CHECK(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) tc_gemm(P, O, err.get(), nullptr, st, variant);
        CUDA_CHECK(cudaEventRecord(e1, st));
        CUDA_CHECK(cudaEventSynchronize(e1));
        float ms = 0;
        CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        int h_err = 0;
        err.download(&h_err, 1);
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (h_err) fail(SQBEM_ERR_TIMEOUT, "gemm_timing: a bounded wait in the tensor-core GEMM expired");
        *seconds = ms * 1e-3 / reps;
    });
}

extern "C" int sqbem_test_gemm_stall(int calls) {
    return guarded([&] {
        if (calls < 0) fail(SQBEM_ERR_ARG, "test_gemm_stall: negative count");
        g_test_stalls.store(calls);
    });
}
