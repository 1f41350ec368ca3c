// Geometry of a vortex-particle case: body triangles plus the two-row buffer wake of
// quadrilaterals that the reference builds at the trailing edge.
//
// Restates geometry::readTri's VP branch (CPanel/geometry.cpp:261-400) and
// createVPWakeSurfaces (:1313-1345): sharp trailing edges (edge::checkTE, CPanel/
// edge.cpp:97-107), node projection along the averaged TE normal (cpNode::firstProjNode/
// secProjNode/nodeWakeProjAngle, CPanel/cpNode.cpp:95-132), quad geometry (panel::setGeom,
// CPanel/panel.cpp:73-103), wake lines and interpolation columns of the first row
// (wakePanel::setParentPanels/interpPanels, CPanel/wakePanel.cpp:48-81,120-152) and the
// shedding topology of the second row (edgesInOrder/pointsInOrder/getOtherWakePan,
// CPanel/wakePanel.cpp:311-405, CPanel/edge.cpp:135-146).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cpg {

// Packed quad record (32 doubles): vertices, centre, normal, local l and m, area, longSide.
enum QuadField { QF_V0 = 0, QF_C = 12, QF_N = 15, QF_L = 18, QF_M = 21, QF_AREA = 24, QF_LONG = 25, QF_STRIDE = 32 };

struct VPGeom {
    int64_t n_body = 0, n_w1 = 0, n_w2 = 0;
    double dt = 0;
    std::vector<double> body;      // n_body x 24 panel records in matrix order (PF_* layout)
    std::vector<double> w1, w2;    // quad records (QF_* layout)
    std::vector<int32_t> widx;     // 4 matrix columns per first-row panel
    std::vector<double> wcoef;     // interpolation coefficient per first-row panel
    std::vector<int32_t> parent;   // second-row panel -> its first-row parent (w1 index)
    // wake lines sorted by y (wake::addWakeLine): upper and lower body panel (matrix
    // order) and the y of the line's trailing-edge midpoint
    std::vector<int32_t> line_up, line_lo;
    std::vector<double> line_y;
    // shedding topology per second-row panel k
    std::vector<int32_t> eio;      // 4 edge ids in edgesInOrder order
    std::vector<int32_t> pio;      // 4 node ids in pointsInOrder order
    std::vector<int32_t> nbr_eio;  // w2 index across eio[1] and eio[3] (2 per panel, -1: none)
    std::vector<int32_t> nbr_raw;  // w2 index across raw edges 1 and 3 (getPartRadius)
    std::vector<double> nodes;     // all nodes, body then buffer wake (3 per node)
};

// nodes n_nodes x 3; tris n_tris x 3 (1-based); ids must all be < 1000 (the VP case
// rejects meshes that carry wake panels, CPanel/geometry.cpp:270-277).  dt <= 0: the
// time step of geometry::calcTimeStep (mean TE edge length / V).  Returns "" on success.
std::string build_vp_geometry(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                              int64_t n_tris, double V, double dt, VPGeom& G);

// Quad record (QF_* layout) of a free quadrilateral given by its 4 vertices (12 doubles),
// with the geometry of panel::setGeom (CPanel/panel.cpp:73-103; longSide over the 4 sides).
void pack_quad_record(const double* v12, double* out);

}  // namespace cpg
