// sphere_share.cu -- the sphere-sphere blocks shared by the swimmers of one call
// (see sphere_share.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "assemble.cuh"
#include "common.cuh"
#include "solver.cuh"
#include "sphere_share.cuh"

namespace sqbem {

namespace {
std::vector<double> centred_vertices(const std::vector<PanelRec>& panels, const double* xc) {
    std::vector<double> v(9 * panels.size());
    for (size_t p = 0; p < panels.size(); ++p)
        for (int k = 0; k < 9; ++k) v[9 * p + k] = panels[p].v[k] - xc[k % 3];
    return v;
}
}  // namespace

bool SphereBlocks::matches(const std::vector<PanelRec>& panels, const double* xc, double mu_) const {
    if ((int)panels.size() != Ns || mu_ != mu) return false;
    double scale = 0, dev = 0;
    for (size_t p = 0; p < panels.size(); ++p)
        for (int k = 0; k < 9; ++k) {
            const double c = panels[p].v[k] - xc[k % 3];
            scale = std::max(scale, std::fabs(Vc[9 * p + k]));
            dev = std::max(dev, std::fabs(c - Vc[9 * p + k]));
        }
    return dev <= 1e-12 * scale;
}

std::shared_ptr<const SphereBlocks> build_sphere_blocks(const std::vector<PanelRec>& panels, const double* xc,
                                                        double mu, cudaStream_t st) {
    auto sb = std::make_shared<SphereBlocks>();
    sb->Ns = (int)panels.size();
    sb->mu = mu;
    sb->Vc = centred_vertices(panels, xc);
    const int Ns = sb->Ns, ns = 3 * Ns;
    DevPanels dp;
    dp.set(make_panels(sb->Vc.data(), Ns), st);
    sb->E.alloc((size_t)ns * ns, st);
    sb->D.alloc((size_t)ns * ns, st);
    sb->rsum.alloc((size_t)ns * 3, st);
    sb->rsum.zero();
    BlockJob<float> j;
    j.tgt = dp.cent.get();
    j.nT = Ns;
    j.src = dp.rec.get();
    j.nS = Ns;
    j.same_mesh = 1;
    j.S = sb->E.get();
    j.s_rs = 1;
    j.s_cs = ns;
    j.D = sb->D.get();
    j.d_rs = 1;
    j.d_cs = ns;
    j.sscale = 1.0 / (EIGHT_PI * mu);
    j.dscale = -1.0 / EIGHT_PI;
    assemble_block(j, (int)std::min<long long>((long long)Ns * Ns, 64LL << 20), st, true);
    add_rowsums<float>(sb->D.get(), 1, ns, ns, Ns, sb->rsum.get(), st);
    deflate<float>(sb->E.get(), 1, ns, dp, mu, st);
    CUDA_CHECK(cudaStreamSynchronize(st));  // complete before other streams read it
    return sb;
}

}  // namespace sqbem
