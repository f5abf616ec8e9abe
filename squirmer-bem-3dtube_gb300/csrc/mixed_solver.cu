// mixed_solver.cu -- the SQBEM_MIXED swimmer path over groups of instances.
//
// Build (per group): FP32 assembly of every block (FP64 relative vectors, FP64
// 448-point and self integrals); T's certified LU on the tensor cores (and, for a
// tube shared by many swimmers, T^{-1} by the LU solve of the identity);
// Y = T^{-1}[B | Ct] and [G_s | G_c] = [E | Cs] - D Y as grouped tensor-core
// GEMMs; G_s's certified LU; Z = G_s^{-1} G_c by block substitutions and
// S6 = F Z in FP64, S6 inverted on the device (6 x 6, FP64).
// Solve: iterative refinement of the full system in FP64 (see mixed_solver.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "assemble.cuh"
#include "common.cuh"
#include "matvec.cuh"
#include "mixed.cuh"
#include "mixed_solver.cuh"
#include "solver.cuh"
#include "tube_sym.cuh"

namespace sqbem {

namespace {

__global__ void pad_identity_kernel(float* A, long long ld, int n0, int n1) {
    const int i = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n1) A[i + (long long)i * ld] = 1.f;
}

void pad_identity(float* A, long long ld, int n0, int n1, cudaStream_t st) {
    if (n1 > n0) LAUNCH(pad_identity_kernel, ceil_div(n1 - n0, 128), 128, 0, st, A, ld, n0, n1);
}

BlockJob<float> fjob(const DevPanels& tgt, const DevPanels& src, bool same, double mu, float* S, long long lds,
                     float* D, long long ldd) {
    BlockJob<float> j;
    j.tgt = tgt.cent.get();
    j.nT = tgt.P;
    j.src = src.rec.get();
    j.nS = src.P;
    j.same_mesh = same ? 1 : 0;
    j.S = S;
    j.s_rs = 1;
    j.s_cs = lds;
    j.D = D;
    j.d_rs = 1;
    j.d_cs = ldd;
    j.sscale = 1.0 / (EIGHT_PI * mu);
    j.dscale = -1.0 / EIGHT_PI;
    return j;
}

// SQBEM_TUBE_SYMMETRY=0 assembles every tube block directly and factors it
// (for comparisons); SQBEM_TUBE_FOURIER=0 keeps the symmetric assembly but
// factors the tube block instead of inverting its Fourier blocks.
bool tube_symmetry_enabled() {
    const char* e = std::getenv("SQBEM_TUBE_SYMMETRY");
    return !(e && e[0] == '0');
}
bool tube_fourier_enabled() {
    const char* e = std::getenv("SQBEM_TUBE_FOURIER");
    return tube_symmetry_enabled() && !(e && e[0] == '0');
}

int cap_pairs(int a, int b) { return (int)std::min<long long>((long long)a * b, 64LL << 20); }

int read_int(const int* d, cudaStream_t st) {
    int h = 0;
    CUDA_CHECK(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    count_d2h(sizeof(int));
    CUDA_CHECK(cudaStreamSynchronize(st));
    return h;
}

void check_ctx(const MixedCtx& cx, const char* what) {
    if (read_int(cx.err, cx.st)) fail(SQBEM_ERR_TIMEOUT, "%s: a bounded wait in the tensor-core GEMM expired", what);
    const int f = read_int(cx.flag, cx.st);
    if (f & 2) fail(SQBEM_ERR_SINGULAR, "%s failed: zero pivot", what);
    if (f & 4) fail(SQBEM_ERR_SINGULAR, "dgesv failed (rigid-body 6 x 6 system)");
    if (f & 1)
        fail(SQBEM_ERR_SINGULAR, "%s: partial pivoting would exchange rows; the mixed LU does not pivot", what);
}

// S6^{-1} for every member: Gauss-Jordan elimination with partial pivoting in
// FP64, one thread per 6 x 6 system (FP64 on the GPU for the rigid-body solve;
// round-to-nearest operations without contraction, so the result does not
// depend on the compiler's FMA choices).  A zero pivot sets bit 2 of *flag.
constexpr int INV6_MAX = 64;
struct Inv6Args {
    int n;
    int* flag;
    const double* S;      // member k at S + 36 k, column-major 6 x 6
    double* Si[INV6_MAX];
};

__global__ void invert6_kernel(const __grid_constant__ Inv6Args args) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= args.n) return;
    const double* A = args.S + 36 * (long long)k;
    double a[6][12];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            a[i][j] = A[i + 6 * j];
            a[i][6 + j] = i == j ? 1.0 : 0.0;
        }
    for (int c = 0; c < 6; ++c) {
        int p = c;
        for (int r = c + 1; r < 6; ++r)
            if (fabs(a[r][c]) > fabs(a[p][c])) p = r;
        if (!(fabs(a[p][c]) > 0)) {
            atomicOr(args.flag, 4);
            return;
        }
        if (p != c)
            for (int j = 0; j < 12; ++j) {
                const double t = a[p][j];
                a[p][j] = a[c][j];
                a[c][j] = t;
            }
        const double d = a[c][c];
        for (int j = 0; j < 12; ++j) a[c][j] = __ddiv_rn(a[c][j], d);
        for (int r = 0; r < 6; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int j = 0; j < 12; ++j) a[r][j] = __dsub_rn(a[r][j], __dmul_rn(f, a[c][j]));
            }
    }
    double* out = args.Si[k];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) out[i + 6 * j] = a[i][6 + j];
}

CopyJob cp32_64(const float* s, long long lds, double* d, long long ldd, int rows, int cols) {
    CopyJob j;
    j.s32 = s; j.lds = lds; j.d64 = d; j.ldd = ldd; j.rows = rows; j.cols = cols;
    return j;
}
CopyJob cp64_32(const double* s, long long lds, float* d, long long ldd, int rows, int cols) {
    CopyJob j;
    j.s64 = s; j.lds = lds; j.d32 = d; j.ldd = ldd; j.rows = rows; j.cols = cols;
    return j;
}
CopyJob cp32_32(const float* s, long long lds, float* d, long long ldd, int rows, int cols) {
    CopyJob j;
    j.s32 = s; j.lds = lds; j.d32 = d; j.ldd = ldd; j.rows = rows; j.cols = cols;
    return j;
}
CopyJob cp64(const double* s, long long lds, double* d, long long ldd, int rows, int cols, double alpha = 1,
             double beta = 0) {
    CopyJob j;
    j.s64 = s; j.lds = lds; j.d64 = d; j.ldd = ldd; j.rows = rows; j.cols = cols; j.alpha = alpha; j.beta = beta;
    return j;
}
MvJob mv32(const float* A, long long lda, int m, int n, const double* x, long long ldx, int r, double* y,
           long long ldy, double alpha, double beta) {
    MvJob j;
    j.A32 = A; j.lda = lda; j.m = m; j.n = n; j.x = x; j.ldx = ldx; j.r = r; j.y = y; j.ldy = ldy;
    j.alpha = alpha; j.beta = beta;
    return j;
}
// the same in plain FP32 (a preconditioner product or a residual update with a
// small correction: its rounding enters only the next correction)
MvJob mv32p(const float* A, long long lda, int m, int n, const double* x, long long ldx, int r, double* y,
            long long ldy, double alpha, double beta) {
    MvJob j = mv32(A, lda, m, n, x, ldx, r, y, ldy, alpha, beta);
    j.plain = true;
    return j;
}
MvJob mv64(const double* A, long long lda, int m, int n, const double* x, long long ldx, int r, double* y,
           long long ldy, double alpha, double beta) {
    MvJob j = mv32(nullptr, lda, m, n, x, ldx, r, y, ldy, alpha, beta);
    j.A64 = A;
    return j;
}

}  // namespace

// ---------------------------------------------------------------- inverses
// inv[k] (n x n, column-major, ld n) <- A_k^{-1} from the factor L[k], with an
// optional row-major split copy (rh/rl).  Solves the identity in place.
static void invert_group(const std::vector<MixedLU*>& L, const std::vector<float*>& inv,
                         const std::vector<bf16*>& rh, const std::vector<bf16*>& rl, const MixedCtx& cx) {
    const size_t G = L.size();
    std::vector<DevBuf<bf16>> ch(G), cl(G);
    std::vector<Rhs> rhs(G);
    for (size_t k = 0; k < G; ++k) {
        const int n = L[k]->n;
        CUDA_CHECK(cudaMemsetAsync(inv[k], 0, sizeof(float) * (size_t)n * n, cx.st));
        pad_identity(inv[k], n, 0, n, cx.st);
        // split copies start as the exact split of the identity's zeros: the lower
        // solve skips the zero blocks above the diagonal, which later updates read
        ch[k].alloc((size_t)n * n, cx.st);
        cl[k].alloc((size_t)n * n, cx.st);
        ch[k].zero();
        cl[k].zero();
        Rhs& r = rhs[k];
        r.X = inv[k]; r.ldx = n; r.nrhs = n; r.Sh = ch[k].get(); r.Sl = cl[k].get(); r.lds = n;
        r.Rh = rh.empty() ? nullptr : rh[k];
        r.Rl = rl.empty() ? nullptr : rl[k];
        r.ldr = n;
    }
    mixed_lu_solve(L, rhs, cx, true);
}

// ---------------------------------------------------------------- tubes
void mixed_build_tubes(const std::vector<sqbem_tube*>& tubes, const MixedCtx& cx, bool explicit_inverse) {
    const size_t G = tubes.size();
    // rotationally symmetric tubes (all of the group): the FP32 block for the
    // residuals and the inverses of its Fourier blocks, no LU
    std::vector<TubeSymmetry> syms(G);
    bool four = tube_fourier_enabled() && G > 0;
    for (size_t k = 0; k < G && four; ++k) {
        syms[k] = tube_symmetry(tubes[k]->host_panels, tubes[k]->n_theta);
        four = fourier_supported(syms[k]);
    }
    if (four) {
        std::vector<DevBuf<float>> T0(G);
        std::vector<FourierTube*> fts;
        std::vector<const TubeSymmetry*> sp;
        std::vector<const float*> t0p;
        for (size_t k = 0; k < G; ++k) {
            sqbem_tube* t = tubes[k];
            MixedTube& M = t->mt;
            M.nt = 3 * t->Nt;
            M.ntp = pad128(M.nt);
            M.T.alloc((size_t)M.nt * M.nt, cx.st);
            assemble_tube_symmetric(t, syms[k], M.T.get(), M.nt, cx.st, &T0[k]);
            M.lu.reset();
            M.ft = std::make_unique<FourierTube>();
            fts.push_back(M.ft.get());
            sp.push_back(&syms[k]);
            t0p.push_back(T0[k].get());
        }
        fourier_build(fts, sp, t0p, cx);
        check_ctx(cx, "mixed tube (Fourier blocks)");
        // A tube shared by many swimmers could also keep T^{-1} (solving the identity
        // through the blocks: FP32 for the refinement's products, split row-major as
        // the left operand of every swimmer's Y = T^{-1} [B | Ct]).  The per-swimmer
        // Fourier solves are cheaper than those dense products (K = 3 Nt): on the
        // 256-swimmer ensemble 4250 against 3871 solves/s, so the dense inverse is
        // formed only when SQBEM_FOURIER_EXPLICIT=1 asks for it.
        const char* fe = std::getenv("SQBEM_FOURIER_EXPLICIT");
        if (explicit_inverse && fe && std::atoi(fe) != 0) {
            for (size_t k = 0; k < G; ++k) {
                MixedTube& M = tubes[k]->mt;
                const size_t nn = (size_t)M.ntp * M.ntp;
                M.Ti.alloc(nn, cx.st);
                M.TiRh.alloc(nn, cx.st);
                M.TiRl.alloc(nn, cx.st);
                DevBuf<float> I((size_t)M.nt * M.nt, cx.st);
                I.zero();
                pad_identity(I.get(), M.nt, 0, M.nt, cx.st);
                FourierJob j;
                j.ft = M.ft.get();
                j.x32 = I.get(); j.ldx = M.nt; j.nc = M.nt;
                j.y32 = M.Ti.get(); j.ldy = M.ntp;
                j.yh = M.TiRh.get(); j.yl = M.TiRl.get(); j.srs = M.ntp; j.scs = 1;
                fourier_solve({j}, cx);
            }
            check_ctx(cx, "mixed tube inverse (Fourier blocks)");
        }
        return;
    }
    std::vector<MixedLU> lu(G);
    std::vector<MixedLU*> lus;
    std::vector<CopyJob> cj;
    for (size_t k = 0; k < G; ++k) {
        sqbem_tube* t = tubes[k];
        MixedTube& M = t->mt;
        M.nt = 3 * t->Nt;
        lu[k].alloc(M.nt, cx.st);
        M.ntp = lu[k].n;
        const int np = M.ntp;
        lu[k].A.zero();
        // the tube block from the rows of one sector where the mesh is
        // rotationally symmetric (every tube this library meshes), else directly
        const TubeSymmetry sym = tube_symmetry_enabled() ? tube_symmetry(t->host_panels, t->n_theta) : TubeSymmetry{};
        if (sym.ok) {  // deflated from the sector-0 rows
            assemble_tube_symmetric(t, sym, lu[k].A.get(), np, cx.st);
        } else {
            auto job = fjob(t->panels, t->panels, true, t->mu, lu[k].A.get(), np, nullptr, 0);
            assemble_block(job, cap_pairs(t->Nt, t->Nt), cx.st, true);
            deflate<float>(lu[k].A.get(), 1, np, t->panels, t->mu, cx.st);
        }
        pad_identity(lu[k].A.get(), np, M.nt, np, cx.st);
        M.T.alloc((size_t)M.nt * M.nt, cx.st);
        cj.push_back(cp32_32(lu[k].A.get(), np, M.T.get(), M.nt, M.nt, M.nt));
        lus.push_back(&lu[k]);
    }
    copy_group(cj, cx.st);
    mixed_lu_factor(lus, cx);
    check_ctx(cx, "dgetrf (mixed tube factor)");
    if (!explicit_inverse) {
        for (size_t k = 0; k < G; ++k) {
            lu[k].A.release();  // the solves read only the split factor and the block inverses
            lu[k].Ch.release();
            lu[k].Cl.release();
            tubes[k]->mt.lu = std::make_unique<MixedLU>(std::move(lu[k]));
        }
        return;
    }
    std::vector<float*> inv;
    std::vector<bf16*> rh, rl;
    for (sqbem_tube* t : tubes) {
        MixedTube& M = t->mt;
        const size_t nn = (size_t)M.ntp * M.ntp;
        M.Ti.alloc(nn, cx.st);
        M.TiRh.alloc(nn, cx.st);
        M.TiRl.alloc(nn, cx.st);
        inv.push_back(M.Ti.get());
        rh.push_back(M.TiRh.get());
        rl.push_back(M.TiRl.get());
    }
    invert_group(lus, inv, rh, rl, cx);
    check_ctx(cx, "mixed tube inverse");
}

// ---------------------------------------------------------------- swimmers
void mixed_build_swimmers(const std::vector<sqbem_swimmer*>& sw, const MixedCtx& cx,
                          const std::shared_ptr<const SphereBlocks>& share) {
    if (sw.empty()) return;
    const size_t G = sw.size();
    const bool bounded = sw[0]->tube != nullptr;
    // host time per phase on stderr when SQBEM_HOST_TIMING is set (profiling aid)
    static const bool timing = std::getenv("SQBEM_HOST_TIMING") != nullptr;
    auto tp = std::chrono::steady_clock::now();
    auto lap = [&](const char* what) {
        if (!timing) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "  swimmers G=%zu %-10s %.2f ms\n", G, what,
                     std::chrono::duration<double, std::milli>(now - tp).count());
        tp = now;
    };
    std::vector<CopyJob> cj;
    std::vector<MvJob> mj;
    std::vector<RigidJob> rj;
    std::vector<DevBuf<double>> tmp;
    tmp.reserve(3 * G);
    for (sqbem_swimmer* s : sw) {
        MixedSwimmer& M = s->mx;
        const int Ns = s->Ns, Nt = s->Nt;
        M.ns = 3 * Ns;
        M.nt = 3 * Nt;
        M.nc = M.ns + 6;
        M.nsp = pad128(M.ns);
        const int ns = M.ns, nt = M.nt;
        const bool shared = share && share->matches(s->host_panels, s->xc, s->mu);
        M.sphere = shared ? share : nullptr;
        if (!shared) M.E.alloc((size_t)ns * ns, cx.st);
        M.AuBs.alloc((size_t)ns * ns, cx.st);
        DevBuf<double> rsum((size_t)ns * 3, cx.st);
        if (shared) {  // the sphere's own row sums first, the tube's added below
            CUDA_CHECK(cudaMemcpyAsync(rsum.get(), share->rsum.get(), sizeof(double) * ns * 3,
                                       cudaMemcpyDeviceToDevice, cx.st));
            CUDA_CHECK(cudaMemcpyAsync(M.AuBs.get(), share->D.get(), sizeof(float) * (size_t)ns * ns,
                                       cudaMemcpyDeviceToDevice, cx.st));
        } else {
            rsum.zero();
        }
        if (bounded) {
            M.B.alloc((size_t)nt * ns, cx.st);
            M.AuBt.alloc((size_t)nt * ns, cx.st);
            auto j1 = fjob(s->tube->panels, s->panels, false, s->mu, M.B.get(), nt, M.AuBt.get(), nt);
            assemble_block(j1, cap_pairs(Nt, Ns), cx.st, true);
            M.D.alloc((size_t)ns * nt, cx.st);
            DevBuf<float> Dt((size_t)ns * nt, cx.st);
            auto j2 = fjob(s->panels, s->tube->panels, false, s->mu, M.D.get(), ns, Dt.get(), ns);
            assemble_block(j2, cap_pairs(Ns, Nt), cx.st, true);
            add_rowsums<float>(Dt.get(), 1, ns, ns, Nt, rsum.get(), cx.st);
        }
        if (!shared) {
            auto j3 = fjob(s->panels, s->panels, true, s->mu, M.E.get(), ns, M.AuBs.get(), ns);
            assemble_block(j3, cap_pairs(Ns, Ns), cx.st, true);
            add_rowsums<float>(M.AuBs.get(), 1, ns, ns, Ns, rsum.get(), cx.st);
            deflate<float>(M.E.get(), 1, ns, s->panels, s->mu, cx.st);
        }
        diag_complete<float>(M.AuBs.get(), 1, ns, Ns, rsum.get(), bounded ? 0.0 : 1.0, nullptr, cx.st);
        // rigid-body map, C = A_u K (accumulated in FP64, stored FP32)   (swimmer.hpp:222-234)
        const auto Kh = rigid_map(s->host_panels, s->xc);
        M.K.alloc(Kh.size(), cx.st);
        M.K.upload(Kh.data(), Kh.size());
        // (the panel offsets r_p = c_p - x_c give K's rotation entries)
        std::vector<double> rch(3 * (size_t)Ns);
        for (int p = 0; p < Ns; ++p)
            for (int k = 0; k < 3; ++k) rch[3 * p + k] = s->host_panels[p].c[k] - s->xc[k];
        tmp.emplace_back(rch.size(), cx.st);
        tmp.back().upload(rch.data(), rch.size());
        const double* rc = tmp.back().get();
        M.Cs.alloc((size_t)ns * 6, cx.st);
        tmp.emplace_back((size_t)ns * 6, cx.st);
        rj.push_back({M.AuBs.get(), ns, ns, Ns, rc, tmp.back().get(), ns});
        cj.push_back(cp64_32(tmp.back().get(), ns, M.Cs.get(), ns, ns, 6));
        if (bounded) {
            M.Ct.alloc((size_t)nt * 6, cx.st);
            tmp.emplace_back((size_t)nt * 6, cx.st);
            rj.push_back({M.AuBt.get(), nt, nt, Ns, rc, tmp.back().get(), nt});
            cj.push_back(cp64_32(tmp.back().get(), nt, M.Ct.get(), nt, nt, 6));
        }
        const auto F = constraint_rows(s->host_panels, s->xc, 1.0);
        M.F.alloc(F.size(), cx.st);
        M.F.upload(F.data(), F.size());
    }
    lap("members");
    matvec_group(mj, cx.st);
    rigid_product_group(rj, cx.st);
    copy_group(cj, cx.st);
    cj.clear();
    mj.clear();
    tmp.clear();
    lap("rigid");

    // G = [E | Cs] (- D Y with Y = T^{-1} [B | Ct] when bounded), G_s padded
    std::vector<MixedLU> glu(G);
    std::vector<MixedLU*> gl;
    std::vector<DevBuf<float>> Gc(G);
    for (size_t k = 0; k < G; ++k) {
        MixedSwimmer& M = sw[k]->mx;
        glu[k].alloc(M.ns, cx.st);
        glu[k].A.zero();
        cj.push_back(cp32_32(M.e(), M.ns, glu[k].A.get(), M.nsp, M.ns, M.ns));
        pad_identity(glu[k].A.get(), M.nsp, M.ns, M.nsp, cx.st);
        Gc[k].alloc((size_t)M.ns * 6, cx.st);
        cj.push_back(cp32_32(M.Cs.get(), M.ns, Gc[k].get(), M.ns, M.ns, 6));
        gl.push_back(&glu[k]);
    }
    copy_group(cj, cx.st);
    cj.clear();
    if (bounded) {
        // [B | Ct] -> split (column-major, ld ntp, zero rows beyond nt); D -> split (row-major, ld ntp)
        std::vector<DevBuf<bf16>> bch(G), bcl(G), yh(G), yl(G), dh(G), dl(G);
        std::vector<ConvJob> conv;
        for (size_t k = 0; k < G; ++k) {
            MixedSwimmer& M = sw[k]->mx;
            const int ntp = sw[k]->tube->mt.ntp;
            const size_t sz = (size_t)ntp * M.nc;
            if (sw[k]->tube->mt.explicit_inverse()) {
                bch[k].alloc(sz, cx.st); bcl[k].alloc(sz, cx.st); bch[k].zero(); bcl[k].zero();
            }
            yh[k].alloc(sz, cx.st); yl[k].alloc(sz, cx.st); yh[k].zero(); yl[k].zero();
            dh[k].alloc((size_t)M.ns * ntp, cx.st); dl[k].alloc((size_t)M.ns * ntp, cx.st);
            dh[k].zero(); dl[k].zero();
            if (sw[k]->tube->mt.explicit_inverse()) {  // the operand of Y = T^{-1} [B | Ct]
                conv.push_back({M.B.get(), 1, M.nt, M.nt, M.ns, bch[k].get(), bcl[k].get(), 1, ntp});
                conv.push_back({M.Ct.get(), 1, M.nt, M.nt, 6, bch[k].get() + (size_t)ntp * M.ns,
                                bcl[k].get() + (size_t)ntp * M.ns, 1, ntp});
            }
            conv.push_back({M.D.get(), 1, M.ns, M.ns, M.nt, dh[k].get(), dl[k].get(), ntp, 1});
        }
        lap("G setup");
        convert_group(conv, cx.st);
        lap("convert");
        // Y = T^{-1} [B | Ct]   (FP32 for the refinement, split for the Schur product)
        std::vector<TcProblem> P;
        std::vector<TcOperands> O;
        for (size_t k = 1; k < G; ++k)
            if (sw[k]->tube->mt.fourier() != sw[0]->tube->mt.fourier() ||
                sw[k]->tube->mt.explicit_inverse() != sw[0]->tube->mt.explicit_inverse())
                fail(SQBEM_ERR_ARG, "mixed swimmers of one group share a tube mode");
        if (sw[0]->tube->mt.fourier() && !sw[0]->tube->mt.explicit_inverse()) {
            // through the Fourier blocks; Y in its own buffer (ld nt), the split copy
            // in (yh, yl) with ld ntp
            std::vector<FourierJob> fj;
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                const MixedTube& Tt = sw[k]->tube->mt;
                const int ntp = Tt.ntp;
                M.Y.alloc((size_t)M.nt * M.nc, cx.st);
                M.ldY = M.nt;
                FourierJob a;
                a.ft = Tt.ft.get();
                a.x32 = M.B.get(); a.ldx = M.nt; a.nc = M.ns;
                a.y32 = M.Y.get(); a.ldy = M.nt;
                a.yh = yh[k].get(); a.yl = yl[k].get(); a.srs = 1; a.scs = ntp;
                fj.push_back(a);
                FourierJob b = a;
                b.x32 = M.Ct.get(); b.nc = 6;
                b.y32 = M.Y.get() + (size_t)M.nt * M.ns;
                b.yh = yh[k].get() + (size_t)ntp * M.ns; b.yl = yl[k].get() + (size_t)ntp * M.ns;
                fj.push_back(b);
            }
            fourier_solve(fj, cx);
        } else if (!sw[0]->tube->mt.explicit_inverse()) {
            // by the LU solves: X = [B | Ct] padded to ntp rows, solved in place; the
            // solves keep the column-major split copy (yh, yl) equal to the result
            std::vector<DevBuf<float>> yp(G);
            std::vector<MixedLU*> tl;
            std::vector<Rhs> rhs(G);
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                const MixedTube& Tt = sw[k]->tube->mt;
                const int ntp = Tt.ntp;
                yp[k].alloc((size_t)ntp * M.nc, cx.st);
                if (ntp > M.nt)  // rows nt .. ntp of every column; the copies below fill the rest
                    CUDA_CHECK(cudaMemset2DAsync(yp[k].get() + M.nt, sizeof(float) * ntp, 0,
                                                 sizeof(float) * (ntp - M.nt), M.nc, cx.st));
                cj.push_back(cp32_32(M.B.get(), M.nt, yp[k].get(), ntp, M.nt, M.ns));
                cj.push_back(cp32_32(M.Ct.get(), M.nt, yp[k].get() + (size_t)ntp * M.ns, ntp, M.nt, 6));
                tl.push_back(Tt.lu.get());
                Rhs& r = rhs[k];
                r.X = yp[k].get(); r.ldx = ntp; r.nrhs = M.nc; r.Sh = yh[k].get(); r.Sl = yl[k].get(); r.lds = ntp;
            }
            copy_group(cj, cx.st);
            cj.clear();
            mixed_lu_solve(tl, rhs, cx);
            for (size_t k = 0; k < G; ++k) {  // Y stays in the padded buffer
                MixedSwimmer& M = sw[k]->mx;
                M.Y = std::move(yp[k]);
                M.ldY = sw[k]->tube->mt.ntp;
            }
        }
        for (size_t k = 0; k < G && sw[0]->tube->mt.explicit_inverse(); ++k) {
            MixedSwimmer& M = sw[k]->mx;
            const MixedTube& Tt = sw[k]->tube->mt;
            const int ntp = Tt.ntp;
            M.Y.alloc((size_t)M.nt * M.nc, cx.st);
            M.ldY = M.nt;
            TcProblem p;
            p.M = M.nt; p.N = M.nc; p.K = M.nt; p.alpha = 1.f; p.beta = 0.f;
            p.C = M.Y.get(); p.c_rs = 1; p.c_cs = M.nt;
            p.O_hi = yh[k].get(); p.O_lo = yl[k].get(); p.o_rs = 1; p.o_cs = ntp;
            TcOperands o;
            o.A = {const_cast<bf16*>(Tt.TiRh.get()), const_cast<bf16*>(Tt.TiRl.get()), M.nt, M.nt, ntp};
            o.B = {bch[k].get(), bcl[k].get(), M.nc, M.nt, ntp};
            P.push_back(p);
            O.push_back(o);
        }
        if (!P.empty()) tc_gemm(P, O, cx.err, nullptr, cx.st);
        P.clear();
        O.clear();
        // [G_s | G_c] -= D Y
        for (size_t k = 0; k < G; ++k) {
            MixedSwimmer& M = sw[k]->mx;
            const int ntp = sw[k]->tube->mt.ntp;
            TcOperands o;
            o.A = {dh[k].get(), dl[k].get(), M.ns, ntp, ntp};
            o.B = {yh[k].get(), yl[k].get(), M.ns, ntp, ntp};
            TcProblem p;
            p.M = M.ns; p.N = M.ns; p.K = ntp; p.alpha = -1.f; p.beta = 1.f;
            p.C = glu[k].A.get(); p.c_rs = 1; p.c_cs = M.nsp;
            P.push_back(p);
            O.push_back(o);
            TcProblem q = p;
            q.N = 6;
            q.C = Gc[k].get(); q.c_cs = M.ns;
            TcOperands o2 = o;
            o2.B = {yh[k].get() + (size_t)ntp * M.ns, yl[k].get() + (size_t)ntp * M.ns, 6, ntp, ntp};
            P.push_back(q);
            O.push_back(o2);
        }
        tc_gemm(P, O, cx.err, nullptr, cx.st);
        lap("Y, D Y");
    }
    mixed_lu_factor(gl, cx);
    lap("LU");
    check_ctx(cx, "dgetrf (mixed Schur factor)");
    lap("LU wait");
    // keep G_s's factor (the solves read only the split factor and the block
    // inverses); Z = G_s^{-1} G_c by block substitutions, then S6 = F Z in FP64,
    // S6 inverted on the device
    std::vector<const MixedLU*> gf;
    for (size_t k = 0; k < G; ++k) {
        glu[k].A.release();
        glu[k].Ch.release();
        glu[k].Cl.release();
        sw[k]->mx.glu = std::make_unique<MixedLU>(std::move(glu[k]));
        gf.push_back(sw[k]->mx.glu.get());
    }
    std::vector<DevBuf<double>> gc64(G);
    DevBuf<double> s6((size_t)36 * G, cx.st);
    std::vector<TrsvIO> zio(G);
    for (size_t k = 0; k < G; ++k) {
        MixedSwimmer& M = sw[k]->mx;
        gc64[k].alloc((size_t)M.ns * 6, cx.st);
        cj.push_back(cp32_64(Gc[k].get(), M.ns, gc64[k].get(), M.ns, M.ns, 6));
        M.Z64.alloc((size_t)M.ns * 6, cx.st);
        zio[k] = {gc64[k].get(), M.ns, M.Z64.get(), M.ns, M.ns};
    }
    copy_group(cj, cx.st);
    cj.clear();
    trsv_group_io(gf, zio, 6, cx.st);
    for (size_t k = 0; k < G; ++k) {
        MixedSwimmer& M = sw[k]->mx;
        mj.push_back(mv64(M.F.get(), 6, 6, M.ns, M.Z64.get(), M.ns, 6, s6.get() + 36 * k, 6, 1.0, 0.0));
    }
    matvec_group(mj, cx.st);
    mj.clear();
    for (size_t k0 = 0; k0 < G; k0 += INV6_MAX) {
        Inv6Args a;
        a.n = (int)std::min<size_t>(INV6_MAX, G - k0);
        a.flag = cx.flag;
        a.S = s6.get() + 36 * k0;
        for (int k = 0; k < a.n; ++k) {
            MixedSwimmer& M = sw[k0 + k]->mx;
            M.S6i.alloc(36, cx.st);
            a.Si[k] = M.S6i.get();
        }
        LAUNCH(invert6_kernel, 1, INV6_MAX, 0, cx.st, a);
    }
    lap("Z, S6");
    check_ctx(cx, "mixed Schur inverse");
    lap("S6 wait");
}

// ---------------------------------------------------------------- refinement
void mixed_solve(const std::vector<sqbem_swimmer*>& sw, bool prescribed, const std::vector<const double*>& in, int r,
                 const std::vector<double*>& xs, const MixedCtx& cx, int* iterations, double* residual) {
    const size_t G = sw.size();
    if (G == 0) return;
    const bool bounded = sw[0]->tube != nullptr;
    struct Work {
        DevBuf<double> bt, bs, rt, rs, rc, rsp, yt, tmp6, dsw, dt, nrm;
    };
    const bool fourier_mode = bounded && sw[0]->tube->mt.fourier();
    const bool factor_mode = bounded && !fourier_mode && !sw[0]->tube->mt.explicit_inverse();
    std::vector<Work> W(G);
    std::vector<MvJob> mj;
    std::vector<CopyJob> cj;
    for (size_t k = 0; k < G; ++k) {
        MixedSwimmer& M = sw[k]->mx;
        Work& w = W[k];
        const int nt = M.nt, ns = M.ns, nc = M.nc;
        const size_t ntr = (size_t)std::max(nt, 1) * r;
        w.bt.alloc(ntr, cx.st); w.rt.alloc(ntr, cx.st); w.dt.alloc(ntr, cx.st); w.yt.alloc(ntr, cx.st);
        w.bs.alloc((size_t)ns * r, cx.st); w.rs.alloc((size_t)ns * r, cx.st); w.rsp.alloc((size_t)ns * r, cx.st);
        w.rc.alloc((size_t)6 * r, cx.st); w.tmp6.alloc((size_t)6 * r, cx.st);
        w.dsw.alloc((size_t)nc * r, cx.st); w.nrm.alloc((size_t)4 * r, cx.st);
        CUDA_CHECK(cudaMemsetAsync(xs[k], 0, sizeof(double) * (size_t)(nt + nc) * r, cx.st));
        CUDA_CHECK(cudaMemsetAsync(w.rc.get(), 0, sizeof(double) * 6 * r, cx.st));
        if (prescribed) {
            // rigid motion given: b = 0, x_w = w fixed (swimmer.hpp:142-153)
            CUDA_CHECK(cudaMemsetAsync(w.bt.get(), 0, sizeof(double) * ntr, cx.st));
            CUDA_CHECK(cudaMemsetAsync(w.bs.get(), 0, sizeof(double) * ns * r, cx.st));
            cj.push_back(cp64(in[k], 6, xs[k] + nt + ns, nt + nc, 6, r));
        } else {
            // slip: b_t = -A_uBt u, b_s = -A_uBs u  (swimmer.hpp:256-269)
            if (bounded) mj.push_back(mv32(M.AuBt.get(), nt, nt, ns, in[k], ns, r, w.bt.get(), nt, -1.0, 0.0));
            mj.push_back(mv32(M.AuBs.get(), ns, ns, ns, in[k], ns, r, w.bs.get(), ns, -1.0, 0.0));
        }
    }
    matvec_group(mj, cx.st);
    mj.clear();
    copy_group(cj, cx.st);
    cj.clear();

    // r = b - A x (FP64), in three rounds that write r_t, r_s, r_c at most once each;
    // x_zero: x = 0 (the start of a free-swimming solve), so r = b with r_c = 0
    auto compute_residual = [&](bool x_zero) {
        for (size_t k = 0; k < G; ++k) {
            MixedSwimmer& M = sw[k]->mx;
            if (bounded) cj.push_back(cp64(W[k].bt.get(), M.nt, W[k].rt.get(), M.nt, M.nt, r));
            cj.push_back(cp64(W[k].bs.get(), M.ns, W[k].rs.get(), M.ns, M.ns, r));
        }
        copy_group(cj, cx.st);
        cj.clear();
        if (x_zero) return;
        for (int round = 0; round < 3; ++round) {
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                const long long ldx = M.nt + M.nc;
                const double* xt = xs[k];
                const double* xsp = xs[k] + M.nt;
                const double* xw = xs[k] + M.nt + M.ns;
                double* rt = W[k].rt.get();
                double* rs = W[k].rs.get();
                if (round == 0) {
                    if (bounded) {
                        mj.push_back(mv32(sw[k]->tube->mt.T.get(), M.nt, M.nt, M.nt, xt, ldx, r, rt, M.nt, -1.0, 1.0));
                        mj.push_back(mv32(M.D.get(), M.ns, M.ns, M.nt, xt, ldx, r, rs, M.ns, -1.0, 1.0));
                    }
                    if (!prescribed)
                        mj.push_back(mv64(M.F.get(), 6, 6, M.ns, xsp, ldx, r, W[k].rc.get(), 6, -1.0, 0.0));
                } else if (round == 1) {
                    if (bounded) mj.push_back(mv32(M.B.get(), M.nt, M.nt, M.ns, xsp, ldx, r, rt, M.nt, -1.0, 1.0));
                    mj.push_back(mv32(M.e(), M.ns, M.ns, M.ns, xsp, ldx, r, rs, M.ns, -1.0, 1.0));
                } else {
                    if (bounded) mj.push_back(mv32(M.Ct.get(), M.nt, M.nt, 6, xw, ldx, r, rt, M.nt, -1.0, 1.0));
                    mj.push_back(mv32(M.Cs.get(), M.ns, M.ns, 6, xw, ldx, r, rs, M.ns, -1.0, 1.0));
                }
            }
            matvec_group(mj, cx.st);
            mj.clear();
        }
    };
    // r -= A d for the correction d = [d_t; d_s; d_w] just added to x (in
    // W.dt and W.dsw), in plain FP32: after the first step |d| is about 3e-5
    // |x|, so the FP32 rounding of A d lies ~1e-11 below |b|, far under the
    // stopping tolerance; the first step's residual (|d| = |x|) is formed from
    // b with the compensated sums.
    auto correct_residual = [&]() {
        for (int round = 0; round < (prescribed ? 2 : 3); ++round) {
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                const double* dt = W[k].dt.get();
                const double* ds = W[k].dsw.get();
                const double* dw = W[k].dsw.get() + M.ns;
                double* rt = W[k].rt.get();
                double* rs = W[k].rs.get();
                if (round == 0) {
                    if (bounded) {
                        mj.push_back(mv32p(sw[k]->tube->mt.T.get(), M.nt, M.nt, M.nt, dt, M.nt, r, rt, M.nt, -1.0, 1.0));
                        mj.push_back(mv32p(M.D.get(), M.ns, M.ns, M.nt, dt, M.nt, r, rs, M.ns, -1.0, 1.0));
                    }
                    if (!prescribed)
                        mj.push_back(mv64(M.F.get(), 6, 6, M.ns, ds, M.nc, r, W[k].rc.get(), 6, -1.0, 1.0));
                } else if (round == 1) {
                    if (bounded) mj.push_back(mv32p(M.B.get(), M.nt, M.nt, M.ns, ds, M.nc, r, rt, M.nt, -1.0, 1.0));
                    mj.push_back(mv32p(M.e(), M.ns, M.ns, M.ns, ds, M.nc, r, rs, M.ns, -1.0, 1.0));
                } else {  // d_w is zero in the prescribed solve
                    if (bounded) mj.push_back(mv32p(M.Ct.get(), M.nt, M.nt, 6, dw, M.nc, r, rt, M.nt, -1.0, 1.0));
                    mj.push_back(mv32p(M.Cs.get(), M.ns, M.ns, 6, dw, M.nc, r, rs, M.ns, -1.0, 1.0));
                }
            }
            matvec_group(mj, cx.st);
            mj.clear();
        }
    };
    // |r|^2 per right-hand side (tube, sphere and constraint rows together)
    auto norms = [&]() {
        std::vector<NormJob> nj;
        for (size_t k = 0; k < G; ++k) {
            MixedSwimmer& M = sw[k]->mx;
            Work& w = W[k];
            CUDA_CHECK(cudaMemsetAsync(w.nrm.get(), 0, sizeof(double) * 4 * r, cx.st));
            if (bounded) nj.push_back({w.rt.get(), M.nt, M.nt, r, w.nrm.get()});
            nj.push_back({w.rs.get(), M.ns, M.ns, r, w.nrm.get() + r});
            nj.push_back({w.rc.get(), 6, 6, r, w.nrm.get() + 2 * r});
        }
        sumsq_group(nj, cx.st);
        std::vector<double> h(4 * r * G);
        for (size_t k = 0; k < G; ++k) W[k].nrm.download(h.data() + 4 * r * k, 4 * r);
        CUDA_CHECK(cudaStreamSynchronize(cx.st));
        std::vector<double> out(G * r);
        for (size_t k = 0; k < G; ++k)
            for (int c = 0; c < r; ++c) out[k * r + c] = h[4 * r * k + c] + h[4 * r * k + r + c] + h[4 * r * k + 2 * r + c];
        return out;
    };
    compute_residual(!prescribed);  // r_c was zeroed with x above
    const std::vector<double> r0 = norms();
    int it = 0;
    double worst = 0;
    const int max_it = refine_max_iterations();
    for (size_t k = 0; k < G * r; ++k) worst = std::max(worst, r0[k] > 0 ? 1.0 : 0.0);
    for (it = 1; it <= max_it && worst > REFINE_TOL; ++it) {
        // (a) y_t = T^{-1} r_t   (b) r_s' = r_s - D y_t
        for (size_t k = 0; k < G; ++k) {
            MixedSwimmer& M = sw[k]->mx;
            cj.push_back(cp64(W[k].rs.get(), M.ns, W[k].rsp.get(), M.ns, M.ns, r));
            if (bounded && !factor_mode && !fourier_mode) {
                const MixedTube& Tt = sw[k]->tube->mt;
                mj.push_back(mv32p(Tt.Ti.get(), Tt.ntp, M.nt, M.nt, W[k].rt.get(), M.nt, r, W[k].yt.get(), M.nt, 1.0, 0.0));
            }
        }
        copy_group(cj, cx.st);
        cj.clear();
        matvec_group(mj, cx.st);
        mj.clear();
        if (factor_mode) {  // y_t by the block substitutions of the tube factor (one launch)
            std::vector<const MixedLU*> tl;
            std::vector<const double*> ins;
            std::vector<double*> outs;
            std::vector<int> nts;
            for (size_t k = 0; k < G; ++k) {
                tl.push_back(sw[k]->tube->mt.lu.get());
                ins.push_back(W[k].rt.get());
                outs.push_back(W[k].yt.get());
                nts.push_back(sw[k]->mx.nt);
            }
            trsv_group(tl, ins, outs, nts, r, cx.st);
        }
        if (fourier_mode) {  // y_t through the tube's Fourier blocks
            std::vector<FourierJob> fj;
            for (size_t k = 0; k < G; ++k) {
                FourierJob a;
                a.ft = sw[k]->tube->mt.ft.get();
                a.x64 = W[k].rt.get(); a.ldx = sw[k]->mx.nt; a.nc = r;
                a.y64 = W[k].yt.get(); a.ldy = sw[k]->mx.nt;
                fj.push_back(a);
            }
            fourier_solve(fj, cx);
        }
        if (bounded) {
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                mj.push_back(mv32p(M.D.get(), M.ns, M.ns, M.nt, W[k].yt.get(), M.nt, r, W[k].rsp.get(), M.ns, -1.0, 1.0));
            }
            matvec_group(mj, cx.st);
            mj.clear();
        }
        // (c) v = G_s^{-1} r_s' by block substitutions with G_s's factor, written
        // into the top of d_sw
        {
            std::vector<const MixedLU*> gf;
            std::vector<TrsvIO> io;
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                gf.push_back(M.glu.get());
                io.push_back({W[k].rsp.get(), M.ns, W[k].dsw.get(), M.nc, M.ns});
            }
            trsv_group_io(gf, io, r, cx.st);
        }
        if (prescribed) {
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                for (int c = 0; c < r; ++c)
                    CUDA_CHECK(cudaMemsetAsync(W[k].dsw.get() + M.ns + (size_t)c * M.nc, 0, 6 * sizeof(double), cx.st));
            }
        } else {
            // (d) dw = S6^{-1} (F v - r_c)   (e) ds = v - Z dw
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                mj.push_back(mv64(M.F.get(), 6, 6, M.ns, W[k].dsw.get(), M.nc, r, W[k].tmp6.get(), 6, 1.0, 0.0));
            }
            matvec_group(mj, cx.st);
            mj.clear();
            for (size_t k = 0; k < G; ++k) cj.push_back(cp64(W[k].rc.get(), 6, W[k].tmp6.get(), 6, 6, r, -1.0, 1.0));
            copy_group(cj, cx.st);
            cj.clear();
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                mj.push_back(mv64(M.S6i.get(), 6, 6, 6, W[k].tmp6.get(), 6, r, W[k].dsw.get() + M.ns, M.nc, 1.0, 0.0));
            }
            matvec_group(mj, cx.st);
            mj.clear();
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                mj.push_back(mv64(M.Z64.get(), M.ns, M.ns, 6, W[k].dsw.get() + M.ns, M.nc, r, W[k].dsw.get(), M.nc,
                                  -1.0, 1.0));
            }
            matvec_group(mj, cx.st);
            mj.clear();
        }
        // (f) d_t = y_t - Y [d_s; d_w]   (g) x += d
        if (bounded) {
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                cj.push_back(cp64(W[k].yt.get(), M.nt, W[k].dt.get(), M.nt, M.nt, r));
            }
            copy_group(cj, cx.st);
            cj.clear();
            for (size_t k = 0; k < G; ++k) {
                MixedSwimmer& M = sw[k]->mx;
                mj.push_back(mv32p(M.Y.get(), M.ldY, M.nt, M.nc, W[k].dsw.get(), M.nc, r, W[k].dt.get(), M.nt, -1.0, 1.0));
            }
            matvec_group(mj, cx.st);
            mj.clear();
        }
        for (size_t k = 0; k < G; ++k) {
            MixedSwimmer& M = sw[k]->mx;
            const long long ldx = M.nt + M.nc;
            if (bounded) cj.push_back(cp64(W[k].dt.get(), M.nt, xs[k], ldx, M.nt, r, 1.0, 1.0));
            cj.push_back(cp64(W[k].dsw.get(), M.nc, xs[k] + M.nt, ldx, prescribed ? M.ns : M.nc, r, 1.0, 1.0));
        }
        copy_group(cj, cx.st);
        cj.clear();
        // (h) new residual
        if (it == 1) compute_residual(false);
        else correct_residual();
        const std::vector<double> rn = norms();
        worst = 0;
        for (size_t k = 0; k < G * r; ++k) {
            const double rel = r0[k] > 0 ? std::sqrt(rn[k] / r0[k]) : 0.0;
            worst = std::max(worst, rel);
        }
        if (!(worst == worst)) fail(SQBEM_ERR_NOT_CONVERGED, "mixed refinement produced a non-finite residual");
    }
    if (read_int(cx.err, cx.st)) fail(SQBEM_ERR_TIMEOUT, "mixed solve: a bounded wait in the tensor-core GEMM expired");
    *iterations = it - 1;
    *residual = worst;
    if (worst > REFINE_TOL)
        fail(SQBEM_ERR_NOT_CONVERGED, "mixed refinement reached relative residual %.3e after %d iterations", worst,
             max_it);
}

}  // namespace sqbem
