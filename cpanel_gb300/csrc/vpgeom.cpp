// Vortex-particle case geometry (host).  See vpgeom.h for the reference functions.
// Compiled with -ffp-contract=off: every geometric quantity is rounded as the
// reference's expressions are, so the device kernels' near/far and on-edge branches
// match the reference's.
#include "vpgeom.h"

#include <algorithm>
#include <array>
#include <cmath>

#include "mesh.h"

namespace cpg {
namespace {

constexpr double kPi = 3.14159265358979323846;

inline d3 add(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 sub(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 mul(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline d3 divs(d3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double nrm(d3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline d3 cross(d3 a, d3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline d3 unit(d3 a) {
    double z = a.x * a.x + a.y * a.y + a.z * a.z;
    return z > 0 ? divs(a, std::sqrt(z)) : a;
}

struct Pan {
    int nv = 3;
    int nd[4], ed[4];
    d3 c, n;
    double area = 0, longSide = 0;
    int id = 0;
    int upPan = -1, loPan = -1;  // wake panels: parents
};
struct Edge {
    int n1, n2;
    std::vector<int> body, wake;
    bool te = false;
};
struct Line {
    int up, lo;
    double y;
};

struct Topo {
    std::vector<d3> P;
    std::vector<Edge> E;
    EdgeMap emap;
    std::vector<Pan> body, wake;
    std::vector<Line> lines;

    int edge(int a, int b) {  // geometry::findEdge, CPanel/geometry.cpp:771-787
        int& slot = emap.slot(((uint64_t)std::min(a, b) << 32) | (uint64_t)std::max(a, b));
        if (slot >= 0) return slot;
        Edge e;
        e.n1 = a;
        e.n2 = b;
        E.push_back(e);
        slot = (int)E.size() - 1;
        return slot;
    }
    double len(int e) const { return nrm(sub(P[E[e].n2], P[E[e].n1])); }
    void geomTri(Pan& p) {  // panel::setGeom, CPanel/panel.cpp:33-72
        p.longSide = 0;
        for (int i = 0; i < 3; i++) {
            double l = len(p.ed[i]);
            if (l > p.longSide) p.longSide = l;
        }
        d3 p0 = P[p.nd[0]], p1 = P[p.nd[1]], p2 = P[p.nd[2]];
        d3 a = sub(p1, p0), b = sub(p2, p0);
        p.c = divs(add(add(p0, p1), p2), 3.0);
        double th = std::acos(dot(a, b) / (nrm(a) * nrm(b)));
        p.area = 0.5 * nrm(a) * nrm(b) * std::sin(th);
        p.n = unit(cross(a, b));
    }
    void geomQuad(Pan& p) {  // panel::setGeom, CPanel/panel.cpp:73-103
        p.longSide = 0;
        for (int i = 0; i < 4; i++) {
            double l = len(p.ed[i]);
            if (l > p.longSide) p.longSide = l;
        }
        d3 p0 = P[p.nd[0]], p1 = P[p.nd[1]], p2 = P[p.nd[2]], p3 = P[p.nd[3]];
        d3 a = sub(p1, p0), b = sub(p2, p1), c = sub(p3, p2);
        d3 pv = add(b, c), qv = add(a, b);
        d3 m1 = add(p1, mul(0.5, pv)), m2 = add(p0, mul(0.5, qv));
        p.c = mul(0.5, add(m1, m2));
        p.area = 0.5 * nrm(cross(pv, qv));
        p.n = unit(cross(a, b));
    }
    void addLine(Line l) {  // wake::addWakeLine, CPanel/wake.cpp:140-144
        lines.push_back(l);
        std::sort(lines.begin(), lines.end(), [](const Line& x, const Line& y) { return x.y < y.y; });
    }
    void checkTE(int ei) {  // edge::checkTE, CPanel/edge.cpp:48-109
        Edge& e = E[ei];
        if (e.body.size() != 2) return;
        if (e.wake.size() == 1) {
            e.te = true;
            Pan& W = wake[e.wake[0]];
            d3 v1 = sub(body[e.body[0]].c, W.c), v2 = sub(body[e.body[1]].c, W.c);
            double t1 = std::acos(dot(v1, W.n) / (nrm(v1) * nrm(W.n)));
            double t2 = std::acos(dot(v2, W.n) / (nrm(v2) * nrm(W.n)));
            int up = t1 < t2 ? e.body[0] : e.body[1], lo = t1 < t2 ? e.body[1] : e.body[0];
            // wakePanel::setParentPanels, CPanel/wakePanel.cpp:120-152
            if (W.upPan < 0 || body[up].c.x < W.c.x) {
                W.upPan = up;
                W.loPan = lo;
            }
            int te = -1;  // wakeLine::setDimensions: the upper panel's (last) TE edge
            for (int k = 0; k < 3; k++)
                if (E[body[W.upPan].ed[k]].te) te = body[W.upPan].ed[k];
            d3 mid = divs(add(P[E[te].n1], P[E[te].n2]), 2.0);
            addLine(Line{W.upPan, W.loPan, mid.y});
        } else {
            const Pan& b0 = body[e.body[0]];
            const Pan& b1 = body[e.body[1]];
            if (std::acos(dot(b0.n, b1.n)) > 4.7 * kPi / 6 && b0.id == b1.id) e.te = true;
        }
    }
    d3 projDir(int node) const {  // cpNode::nodeWakeProjAngle, CPanel/cpNode.cpp:95-115
        d3 avg{0, 0, 0};
        for (const Edge& e : E) {
            if (!(e.n1 == node || e.n2 == node) || !e.te) continue;
            for (int b : e.body) avg = add(avg, body[b].n);
            avg = divs(avg, 3.0);
        }
        return unit(avg);
    }
    d3 mid(int e) const { return add(P[E[e].n1], mul(0.5, sub(P[E[e].n2], P[E[e].n1]))); }
    int otherWake(int e, int self) const {  // edge::getOtherWakePan, CPanel/edge.cpp:135-146
        for (int w : E[e].wake)
            if (w != self) return w;
        return -1;
    }
};

void packTri(const Topo& T, const Pan& p, double* o) {
    for (int k = 0; k < 3; k++) {
        d3 v = T.P[p.nd[k]];
        o[3 * k] = v.x;
        o[3 * k + 1] = v.y;
        o[3 * k + 2] = v.z;
    }
    d3 l = unit(sub(T.P[p.nd[0]], p.c));  // panel::getLocalSys, CPanel/panel.cpp:156-168
    d3 m = cross(p.n, l);
    const d3 f[4] = {p.c, p.n, l, m};
    for (int q = 0; q < 4; q++) {
        o[PF_C + 3 * q] = f[q].x;
        o[PF_C + 3 * q + 1] = f[q].y;
        o[PF_C + 3 * q + 2] = f[q].z;
    }
    o[PF_AREA] = p.area;
    o[PF_LONG] = p.longSide;
    o[23] = 0;
}

void packQuad(const Topo& T, const Pan& p, double* o) {
    for (int k = 0; k < 4; k++) {
        d3 v = T.P[p.nd[k]];
        o[3 * k] = v.x;
        o[3 * k + 1] = v.y;
        o[3 * k + 2] = v.z;
    }
    d3 l = unit(sub(T.P[p.nd[0]], p.c));
    d3 m = cross(p.n, l);
    const d3 f[4] = {p.c, p.n, l, m};
    for (int q = 0; q < 4; q++) {
        o[QF_C + 3 * q] = f[q].x;
        o[QF_C + 3 * q + 1] = f[q].y;
        o[QF_C + 3 * q + 2] = f[q].z;
    }
    o[QF_AREA] = p.area;
    o[QF_LONG] = p.longSide;
    for (int k = QF_LONG + 1; k < QF_STRIDE; k++) o[k] = 0;
}

}  // namespace

void pack_quad_record(const double* v12, double* out) {
    Topo T;
    for (int k = 0; k < 4; k++) T.P.push_back({v12[3 * k], v12[3 * k + 1], v12[3 * k + 2]});
    Pan W;
    W.nv = 4;
    for (int k = 0; k < 4; k++) {
        W.nd[k] = k;
        W.ed[k] = T.edge(k, k < 3 ? k + 1 : 0);
    }
    T.geomQuad(W);
    packQuad(T, W, out);
}

std::string build_vp_geometry(const double* nodes, int64_t nn, const int64_t* tris, const int32_t* ids, int64_t nt,
                              double V, double dt, VPGeom& G) {
    if (nn <= 0 || nt <= 0) return "empty mesh";
    for (int64_t i = 0; i < nt; i++)
        if (ids[i] >= 1000) return "the vortex-particle case takes a mesh without wake panels";
    Topo T;
    T.P.resize(nn);
    for (int64_t i = 0; i < nn; i++) T.P[i] = {nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]};
    // body panels, geometry::createSurfaces, CPanel/geometry.cpp:712-747
    std::vector<std::vector<int>> surf;
    for (int64_t i = 0; i < nt; i++) {
        Pan p;
        for (int k = 0; k < 3; k++) {
            int64_t v = tris[3 * i + k] - 1;
            if (v < 0 || v >= nn) return "triangle references a node outside 1..n_nodes";
            p.nd[k] = (int)v;
        }
        if (p.nd[0] == p.nd[1] || p.nd[1] == p.nd[2] || p.nd[0] == p.nd[2]) return "degenerate triangle";
        for (int k = 0; k < 3; k++) p.ed[k] = T.edge(p.nd[k], p.nd[k < 2 ? k + 1 : 0]);
        p.id = ids[i];
        if (i == 0 || ids[i] != ids[i - 1]) surf.emplace_back();
        T.geomTri(p);
        T.body.push_back(p);
        int bi = (int)T.body.size() - 1;
        for (int k = 0; k < 3; k++) {
            T.E[p.ed[k]].body.push_back(bi);
            T.checkTE(p.ed[k]);
        }
        surf.back().push_back(bi);
    }
    std::vector<int> teEdges;
    for (size_t e = 0; e < T.E.size(); e++)
        if (T.E[e].te) teEdges.push_back((int)e);
    if (teEdges.size() < 2) return "fewer than two sharp trailing edges";
    if (dt <= 0) {  // geometry::calcTimeStep, CPanel/geometry.cpp:1289-1311
        double sum = 0;
        for (int e : teEdges) sum += T.len(e);
        dt = sum / static_cast<double>(teEdges.size()) / V;
    }
    G.dt = dt;
    // buffer wake nodes and quads, CPanel/geometry.cpp:304-393
    const double c_w = 1.3;  // cpNode.h:40
    const int nNodes = (int)nn;
    std::vector<d3> wakeNodes;
    std::vector<int> used, newIdx;
    auto project = [&](int node, int& f, int& s) {
        for (size_t j = 0; j < used.size(); j++)
            if (used[j] == node) {
                f = newIdx[2 * j] + nNodes;
                s = newIdx[2 * j + 1] + nNodes;
                return;
            }
        used.push_back(node);
        d3 bis = T.projDir(node);
        wakeNodes.push_back(add(T.P[node], mul(c_w * dt * V, bis)));
        newIdx.push_back((int)wakeNodes.size() - 1);
        f = (int)wakeNodes.size() - 1 + nNodes;
        wakeNodes.push_back(add(T.P[node], mul((c_w + 1) * dt * V, bis)));
        newIdx.push_back((int)wakeNodes.size() - 1);
        s = (int)wakeNodes.size() - 1 + nNodes;
    };
    std::vector<std::array<int, 4>> conn;
    for (int e : teEdges) {
        int n1 = T.E[e].n1, n2 = T.E[e].n2, n1f, n1s, n2f, n2s;
        project(n1, n1f, n1s);
        project(n2, n2f, n2s);
        conn.push_back({n1, n2, n2f, n1f});
        conn.push_back({n1f, n2f, n2s, n1s});
    }
    for (const d3& p : wakeNodes) T.P.push_back(p);
    // createVPWakeSurfaces, CPanel/geometry.cpp:1313-1345
    std::vector<int> w1, w2, parentW;
    for (size_t i = 0; i < conn.size(); i++) {
        Pan W;
        W.nv = 4;
        for (int k = 0; k < 4; k++) {
            W.nd[k] = conn[i][k];
            W.ed[k] = T.edge(conn[i][k], conn[i][k < 3 ? k + 1 : 0]);
        }
        W.id = 1001;
        T.geomQuad(W);
        T.wake.push_back(W);
        int wi = (int)T.wake.size() - 1;
        for (int k = 0; k < 4; k++) {
            T.E[W.ed[k]].wake.push_back(wi);
            T.checkTE(W.ed[k]);
        }
        if (i % 2 == 0) {
            w1.push_back(wi);
        } else {
            w2.push_back(wi);
            parentW.push_back((int)w1.size() - 1);
        }
    }
    if (T.lines.size() < 2) return "the buffer wake has fewer than two wake lines";
    // matrix order: surfaces in reverse file order (CPanel/geometry.cpp:452-458)
    std::vector<int> bp;
    for (size_t s = surf.size(); s-- > 0;) bp.insert(bp.end(), surf[s].begin(), surf[s].end());
    std::vector<int> index(T.body.size(), -1);
    for (size_t i = 0; i < bp.size(); i++) index[bp[i]] = (int)i;

    G.n_body = (int64_t)bp.size();
    G.n_w1 = (int64_t)w1.size();
    G.n_w2 = (int64_t)w2.size();
    G.body.assign(G.n_body * PF_STRIDE, 0.0);
    for (size_t i = 0; i < bp.size(); i++) packTri(T, T.body[bp[i]], &G.body[i * PF_STRIDE]);
    G.w1.assign(G.n_w1 * QF_STRIDE, 0.0);
    G.w2.assign(G.n_w2 * QF_STRIDE, 0.0);
    for (size_t j = 0; j < w1.size(); j++) packQuad(T, T.wake[w1[j]], &G.w1[j * QF_STRIDE]);
    for (size_t j = 0; j < w2.size(); j++) packQuad(T, T.wake[w2[j]], &G.w2[j * QF_STRIDE]);
    // wakePanel::interpPanels, CPanel/wakePanel.cpp:48-81
    G.widx.assign(4 * G.n_w1, 0);
    G.wcoef.assign(G.n_w1, 0.0);
    const std::vector<Line>& L = T.lines;
    for (size_t j = 0; j < w1.size(); j++) {
        double y = T.wake[w1[j]].c.y;
        const Line *a = nullptr, *b = nullptr;
        if (y < L[1].y) {
            a = &L[0];
            b = &L[1];
        } else if (y >= L.back().y) {
            a = &L[L.size() - 2];
            b = &L[L.size() - 1];
        } else {
            for (size_t i = 1; i + 1 < L.size(); i++)
                if (L[i].y <= y && L[i + 1].y > y) {
                    a = &L[i];
                    b = &L[i + 1];
                }
        }
        if (!a) return "a first-row wake panel lies outside its wake lines";
        G.wcoef[j] = (y - a->y) / (b->y - a->y);
        G.widx[4 * j] = index[a->up];
        G.widx[4 * j + 1] = index[a->lo];
        G.widx[4 * j + 2] = index[b->up];
        G.widx[4 * j + 3] = index[b->lo];
    }
    G.parent = parentW;
    for (const Line& l : L) {
        G.line_up.push_back(index[l.up]);
        G.line_lo.push_back(index[l.lo]);
        G.line_y.push_back(l.y);
    }
    // shedding topology of the second row
    std::vector<int> w2pos(T.wake.size(), -1);
    for (size_t k = 0; k < w2.size(); k++) w2pos[w2[k]] = (int)k;
    G.eio.assign(4 * G.n_w2, 0);
    G.pio.assign(4 * G.n_w2, 0);
    G.nbr_eio.assign(2 * G.n_w2, -1);
    G.nbr_raw.assign(2 * G.n_w2, -1);
    for (size_t k = 0; k < w2.size(); k++) {
        const Pan& W = T.wake[w2[k]];
        int e[4];  // wakePanel::edgesInOrder, CPanel/wakePanel.cpp:365-405
        e[0] = W.ed[0];
        e[2] = W.ed[2];
        d3 a = sub(T.mid(W.ed[0]), W.c);
        d3 c = cross(a, W.n);
        d3 d = add(W.c, c);
        double d1 = nrm(sub(T.mid(W.ed[1]), d)), d3_ = nrm(sub(T.mid(W.ed[3]), d));
        if (d3_ < d1) {
            e[3] = W.ed[3];
            e[1] = W.ed[1];
        } else {
            e[3] = W.ed[1];
            e[1] = W.ed[3];
        }
        auto has = [&](int ei, int node) { return T.E[ei].n1 == node || T.E[ei].n2 == node; };
        int p[4];  // wakePanel::pointsInOrder, CPanel/wakePanel.cpp:311-362
        int n1 = T.E[e[0]].n1, n2 = T.E[e[0]].n2;
        p[0] = has(e[3], n1) ? n1 : n2;
        p[1] = has(e[3], n1) ? n2 : n1;
        n1 = T.E[e[2]].n1;
        n2 = T.E[e[2]].n2;
        p[2] = has(e[1], n1) ? n1 : n2;
        p[3] = has(e[1], n1) ? n2 : n1;
        for (int q = 0; q < 4; q++) {
            G.eio[4 * k + q] = e[q];
            G.pio[4 * k + q] = p[q];
        }
        for (int s = 0; s < 2; s++) {
            int o = T.otherWake(e[1 + 2 * s], w2[k]);
            if (o >= 0 && w2pos[o] < 0) return "a second-row panel shares a side edge with a first-row panel";
            G.nbr_eio[2 * k + s] = o >= 0 ? w2pos[o] : -1;
            o = T.otherWake(W.ed[1 + 2 * s], w2[k]);
            if (o >= 0 && w2pos[o] < 0) return "a second-row panel shares a side edge with a first-row panel";
            G.nbr_raw[2 * k + s] = o >= 0 ? w2pos[o] : -1;
        }
    }
    G.nodes.resize(3 * T.P.size());
    for (size_t i = 0; i < T.P.size(); i++) {
        G.nodes[3 * i] = T.P[i].x;
        G.nodes[3 * i + 1] = T.P[i].y;
        G.nodes[3 * i + 2] = T.P[i].z;
    }
    return "";
}

}  // namespace cpg
