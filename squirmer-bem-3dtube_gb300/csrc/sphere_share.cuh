// sphere_share.cuh -- the sphere-sphere blocks of the mixed path, shared by the
// swimmers of one call.
//
// The single- and double-layer blocks of a sphere's panels against its own
// panels (E before deflation and the raw double layer of A_uBs, swimmer.hpp:
// 208-216) depend only on the sphere's geometry relative to its centre, not on
// where the sphere sits or on the tube: a rigid translation moves targets and
// sources together.  Every instance of a batch with the same sphere level, and
// every evaluation of a trajectory ensemble, therefore has the same
// sphere-sphere blocks up to the rounding of the translated coordinates (a few
// units in the 16th digit, far below the FP32 storage of the blocks).  One
// call assembles them once per sphere geometry and every member copies or
// reads them; a member whose centred vertices differ from the shared ones by
// more than 1e-12 of the sphere's size assembles its own.  Sharing never
// extends beyond the call that built the blocks.
#pragma once
#include <memory>
#include <vector>

#include "assemble.cuh"
#include "common.cuh"

namespace sqbem {

struct SphereBlocks {
    int Ns = 0;
    double mu = 1;
    std::vector<double> Vc;  // centred vertices (9 per panel) the blocks were built from
    DevBuf<float> E;         // SL / (8 pi mu), deflated: the E block of every sharing swimmer
    DevBuf<float> D;         // -DL / (8 pi): A_uBs before its diagonal completion
    DevBuf<double> rsum;     // row sums of D over the sphere's own panels (3 per row)
    // true if a sphere with these panels around centre xc has these blocks
    bool matches(const std::vector<PanelRec>& panels, const double* xc, double mu) const;
};

// Assemble the shared blocks of the sphere whose panels (host records) sit
// around xc, on stream st; returns once they are complete.
std::shared_ptr<const SphereBlocks> build_sphere_blocks(const std::vector<PanelRec>& panels, const double* xc,
                                                        double mu, cudaStream_t st);

}  // namespace sqbem
