// tube_sym.cuh -- the tube's rotational symmetry in the mixed assembly.
//
// The tube mesh (tube_mesh / swimmer_tube_mesh, src/utils/mesh.hpp:149-196) places its nodes
// at the angles 2 pi i / n_theta on the wall and on every cap ring, so rotating
// the mesh by one sector about the axis maps it onto itself, panel for panel and
// vertex for vertex.  The single-layer block of the tube, with the Wielandt
// deflation (src/swimmer.hpp:48-74), is then determined by the rows of one
// sector: for target panel p in sector s and source panel q,
//     T[p, q] = R_s T[rep(p), rot_{-s}(q)] R_s^T,
// with R_s the rotation by 2 pi s / n_theta about z, rep(p) the sector-0 panel
// that p is the rotation of, and rot_{-s}(q) the panel q rotated back by s
// sectors.  The mixed path assembles those rows (1 / n_theta of the pairs) and
// fills the rest of T by rotating 3 x 3 blocks.
#pragma once
#include <vector>

#include "assemble.cuh"
#include "common.cuh"

struct sqbem_tube;

namespace sqbem {

struct TubeSymmetry {
    bool ok = false;
    int nth = 0;               // sectors
    int nb = 0;                // panels per sector
    std::vector<int> sector;   // per panel: its sector
    std::vector<int> rep;      // per panel: index (0 .. nb) of its sector-0 representative
    std::vector<int> panel;    // nb x nth: panel[a * nth + s] = representative a rotated by s sectors
    std::vector<int> rep_panel;  // nb: the panel index of representative a
};

// The symmetry of a panel set under rotations by 2 pi / nth about z, found from
// the geometry: every panel's vertices, rotated back to sector 0, must match a
// sector-0 panel's vertices (same order) to 1e-10 of the mesh size.  ok = false
// if any panel has no match.
TubeSymmetry tube_symmetry(const std::vector<PanelRec>& P, int nth);

// T (FP32, column-major, leading dimension ld, 3 Nt x 3 Nt) <- the tube's
// deflated single-layer block SL / (8 pi mu) + (8 pi mu sqrt(A))^{-1} m_i m_p^T A_p
// (src/swimmer.hpp:48-74) from the rows of sector 0, in the mixed path's FP32
// arithmetic.  T0_out (optional) receives those rows: 3 nb x 3 Nt,
// column-major, leading dimension 3 nb.
void assemble_tube_symmetric(const sqbem_tube* t, const TubeSymmetry& sym, float* T, long long ld,
                             cudaStream_t st, DevBuf<float>* T0_out = nullptr);

}  // namespace sqbem
