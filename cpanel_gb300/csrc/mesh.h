// Host-side mesh ingest and topology for the GB300 panel path.
//
// Restates geometry::readTri (CPanel/geometry.cpp:132-484) for steady, subsonic,
// constant-strength cases: wake-node merging, edge topology, trailing-edge
// detection, wake lines, body-panel ordering, tip-patch flags and CHTLS clusters.
// Everything downstream (assembly, solve, post-processing) runs on the GPU from
// the flat tables built here.
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace cpg {

struct d3 {
    double x = 0, y = 0, z = 0;
};

// Edge index by node pair (the search of geometry::findEdge, CPanel/geometry.cpp:771-787):
// open addressing with linear probing, at most half full.  slot(key) is the value of key, -1
// until the caller sets it, so an edge takes its index when it is first seen, as in a search
// of the edge list.
struct EdgeMap {
    std::vector<uint64_t> keys;  // key + 1; 0 marks an empty slot
    std::vector<int> vals;
    uint64_t mask = 0;
    size_t used = 0;
    void reserve(size_t n) {
        size_t c = 64;
        while (c < 2 * n) c <<= 1;
        if (c <= keys.size()) return;
        std::vector<uint64_t> ok = std::move(keys);
        std::vector<int> ov = std::move(vals);
        keys.assign(c, 0);
        vals.assign(c, -1);
        mask = c - 1;
        used = 0;
        for (size_t i = 0; i < ok.size(); i++)
            if (ok[i]) slot(ok[i] - 1) = ov[i];
    }
    int& slot(uint64_t key) {
        if (2 * (used + 1) > keys.size()) reserve(used + 1 > 32 ? 2 * (used + 1) : 64);
        for (uint64_t h = (key * 0x9E3779B97F4A7C15ull) >> 20;; h++) {
            const uint64_t i = h & mask;
            if (keys[i] == key + 1) return vals[i];
            if (keys[i] == 0) {
                keys[i] = key + 1;
                used++;
                return vals[i];
            }
        }
    }
};

// Packed per-panel record staged by the assembly kernels (24 doubles, 192 bytes).
enum PanelField {
    PF_V0 = 0, PF_V1 = 3, PF_V2 = 6, PF_C = 9, PF_N = 12, PF_L = 15, PF_M = 18, PF_AREA = 21, PF_LONG = 22,
    PF_STRIDE = 24
};

struct TrefftzStation {
    // wake::trefftzPlane station i (CPanel/wake.cpp:167-176)
    double y;
    int32_t line_up1, line_lo1, line_up2, line_lo2;  // matrix indices of the bracketing wake lines
    double interp;                                    // wake::wakeStrength interpolation factor
    double Fy[6], Fz[6];                              // 1-D CHTLS weights of wake::Vradial
    int32_t pt0;                                      // first of 13 sample points: POI, 6 y-offsets, 6 z-offsets
};

struct TrefftzWake {
    double step;                       // Simpson step
    double y0 = 0, y1 = 0;             // wake::yMin, yMax: the end stations 0 and 164
    std::vector<TrefftzStation> st;    // 163 stations (i = 1..163)
};

struct HostMesh {
    int64_t n_nodes = 0;
    int64_t n_body = 0, n_wake = 0, n_lines = 0, n_tip = 0;
    // body panels in matrix order
    std::vector<double> body;          // n_body x PF_STRIDE
    std::vector<double> bez;           // n_body x 3 (bezNormal)
    std::vector<int32_t> tip, upper, lower, tsorder, surf_id, file_tri;
    std::vector<int32_t> cl_ptr, cl_idx;  // CHTLS cluster (matrix indices, self first)
    // wake panels in wPanels order
    std::vector<double> wake;          // n_wake x PF_STRIDE
    std::vector<int32_t> wake_file_tri;  // n_wake: the .tri triangle of each wake panel
    std::vector<int32_t> widx;         // n_wake x 4 interpolation columns
    std::vector<double> wcoef;         // n_wake
    // Trefftz plane, per live wake
    std::vector<TrefftzWake> trefftz;
    std::vector<double> tz_pts;        // all sample points, 3 per point
};

// Returns "" on success, else an error message.  tris are 1-based.  te_upper/te_lower
// (n_te matrix indices, optional) flag the upper and lower parents of trailing edges whose
// wake is not in the file (the vortex-particle buffer wake) before the CHTLS clusters grow.
// Runs f(slice, lo, hi) over [0, n) in contiguous slices on the host threads of the mesh builder
// (each slice on one thread; the calling thread takes part; small ranges run on the caller).
void host_parallel(size_t n, const std::function<void(unsigned, size_t, size_t)>& f);

std::string build_mesh(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                       int64_t n_tris, HostMesh& out, const int32_t* te_upper = nullptr,
                       const int32_t* te_lower = nullptr, int64_t n_te = 0);

// chtlsnd first-derivative weights (unconstrained branch, CPanel/chtlsnd.cpp:20-140,
// 189-196) for a 1-D set of offsets, used for the Trefftz-plane downwash.
void chtls_1d(const double* dx, int nf, int order, double* F);

}  // namespace cpg
