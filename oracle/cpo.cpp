/*
 * cpo.cpp -- CPU oracle for the CPanel steady hot path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain C++17 FP64 restatement of the reference functions named in each comment
 * (paths relative to the CPanel project root).  It exists to check the GPU library
 * (cpanel_gb300) and to time the CPU baseline; the product never links it.
 *
 * Floating-point conventions follow the reference's Eigen expressions: fixed-size
 * dot products and norms are evaluated left to right, and the file is compiled with
 * -ffp-contract=off so that no multiply-add is fused behind our back.
 */
#include "cpo.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;  // M_PI

struct V3 {
    double x = 0, y = 0, z = 0;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double sqn(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double norm(V3 a) { return std::sqrt(sqn(a)); }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalized(V3 a) {  // Eigen::MatrixBase::normalized
    double z = sqn(a);
    if (z > 0) return a / std::sqrt(z);
    return a;
}
inline double at(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
inline bool isnan3(V3 a) { return a.x != a.x || a.y != a.y || a.z != a.z; }

/* ------------------------------------------------------------------ mesh types */
struct Edge {
    int n1, n2;
    std::vector<int> body, wake;
    bool TE = false;
};
struct Tri {  // panel::setGeom state, CPanel/panel.cpp:33-72
    int node[4];  // triangles use 3; the vortex-particle buffer wake uses quads
    int edge[4];
    int nv = 3;
    V3 center, normal, bez;
    double area = 0, longSide = 0;
    int surfID = 0, fileTri = 0;
};
struct Body : Tri {
    int surf = -1;
    bool upper = false, lower = false, TEpanel = false, tip = false;
    int TSorder = 3, index = -1;
    std::vector<int> neighbors, cluster;
};
struct WakeP : Tri {
    int wake = -1;
    int upperPan = -1, lowerPan = -1;
    bool TEpanel = false;
};
struct WakeLine {  // CPanel/wakeLine.cpp:20-46
    int upper, lower;
    V3 p1, p2, pMid, normal;
    double y() const { return pMid.y; }
};
struct Wake {  // CPanel/wake.cpp:42-144
    int id;
    std::vector<int> wpanels;
    std::vector<WakeLine> lines;
    double yMin = 0, yMax = 0, x0 = 0, xf = 0, z0 = 0, zf = 0;
    V3 normal;
    bool dead = false;
};
struct Surface {
    int id;
    std::vector<int> panels;
    bool LS = false;
};

struct Mesh {
    std::vector<V3> nodes;
    std::vector<bool> nodeTE;
    std::vector<Edge> edges;
    std::unordered_map<uint64_t, int> edgeMap;
    std::vector<Body> body;    // creation order
    std::vector<WakeP> wakeP;  // creation order
    std::vector<Surface> surfaces;
    std::vector<Wake> wakes;   // after merge: live wakes in order
    std::vector<int> bPanels;  // matrix order -> body index
    std::vector<int> wPanels;  // wPanels order -> wakeP index
    std::vector<int> bodyIndex;  // body index -> matrix index
    // spanwise loads of the last post-processing, per live wake: 2y/b, Cl / PG, Cd / PG^2 at the
    // 165 Trefftz stations (cpCase::writeSpanwiseData, CPanel/cpCase.cpp:910-935)
    std::vector<std::vector<double>> span;
};

/* ------------------------------------------------------------ panel geometry */
void setGeom(Mesh& M, Tri& T) {  // CPanel/panel.cpp:33-72 (triangles)
    T.longSide = 0;
    for (int i = 0; i < 3; i++) {
        const Edge& e = M.edges[T.edge[i]];
        double l = norm(M.nodes[e.n2] - M.nodes[e.n1]);  // edge::length, edge.cpp:164
        if (l > T.longSide) T.longSide = l;
    }
    V3 p0 = M.nodes[T.node[0]], p1 = M.nodes[T.node[1]], p2 = M.nodes[T.node[2]];
    V3 a = p1 - p0, b = p2 - p0;
    T.center = ((p0 + p1) + p2) / 3.0;
    double theta = std::acos(dot(a, b) / (norm(a) * norm(b)));
    T.area = 0.5 * norm(a) * norm(b) * std::sin(theta);
    T.normal = normalized(cross(a, b));
    T.bez = T.normal;  // no normals in the .tri input
}

/* panel::getLocalSys, CPanel/panel.cpp:156-168 */
struct Local {
    V3 l, m, n;
};
Local localSys(const V3& center, const V3& normal, const V3& node0) {
    Local L;
    L.l = normalized(node0 - center);
    L.m = cross(normal, L.l);
    L.n = normal;
    return L;
}

/* panel::vortexPhi, CPanel/panel.cpp:713-735 */
double vortexPhi(double PN, double Al, V3 a, V3 b, V3 s, V3 l, V3 m) {
    const double eps = std::pow(10.0, -15.0);
    double PA = dot(a, cross(l, cross(a, s)));
    double sm = dot(s, m);
    double PB = PA - Al * sm;
    double na = norm(a), nb = norm(b);
    double num = sm * PN * (nb * PA - na * PB);
    double denom = PA * PB + std::pow(PN, 2) * na * nb * std::pow(sm, 2);
    if (denom == 0 && std::abs(PN) < eps) return PN >= 0 ? 0.5 * kPi : -0.5 * kPi;
    return std::atan2(num, denom);
}

/* bodyPanel::srcSidePhi, CPanel/bodyPanel.cpp:361-373 */
double srcSidePhi(double PN, double Al, double phiV, V3 a, V3 b, V3 s) {
    double A = norm(a), B = norm(b), S = norm(s);
    double GL = 0;
    if (std::abs(A + B - S) > 0 && S > 0) GL = 1 / S * std::log(std::abs((A + B + S) / (A + B - S)));
    return Al * GL - PN * phiV;
}

/* panel::vortexV, CPanel/panel.cpp:707-711 (core = 0.05, panel.h:67) */
V3 vortexV(V3 a, V3 b, V3 s) {
    const double core = 0.05;
    double na = norm(a), nb = norm(b);
    return (cross(a, b) * (na + nb)) / (na * nb * (na * nb + dot(a, b)) + std::pow(core * norm(s), 2));
}

/* The three vertices of a triangle plus its derived frame, for the free-panel API. */
struct Pan {
    V3 p[3];
    V3 center, normal;
    double area, longSide;
};
Pan makePan(const double* v9) {
    Pan P;
    for (int k = 0; k < 3; k++) P.p[k] = {v9[3 * k], v9[3 * k + 1], v9[3 * k + 2]};
    P.longSide = 0;
    for (int k = 0; k < 3; k++) {
        double l = norm(P.p[(k + 1) % 3] - P.p[k]);
        if (l > P.longSide) P.longSide = l;
    }
    V3 a = P.p[1] - P.p[0], b = P.p[2] - P.p[0];
    P.center = ((P.p[0] + P.p[1]) + P.p[2]) / 3.0;
    double theta = std::acos(dot(a, b) / (norm(a) * norm(b)));
    P.area = 0.5 * norm(a) * norm(b) * std::sin(theta);
    P.normal = normalized(cross(a, b));
    return P;
}

/* bodyPanel::panelPhiInf, CPanel/bodyPanel.cpp:132-190.  Accumulates in the near
 * field and assigns in the far field exactly as the reference does. */
void panelPhiInf(const V3* p, V3 center, V3 normal, double area, double longSide, V3 POI,
                 double& phiSrc, double& phiDub) {
    V3 pjk = POI - center;
    bool itself = norm(pjk) < std::pow(10.0, -10.0);
    Local L = localSys(center, normal, p[0]);
    double PN = dot(pjk, L.n);
    if (norm(pjk) / longSide > 5) {
        phiSrc = area / (4 * kPi * norm(pjk));                       // pntSrcPhi, :392-395
        phiDub = PN * area / (4 * kPi * std::pow(norm(pjk), 3));     // pntDubPhi, panel.cpp:737-740
    } else {
        double phiV = 0;
        for (int i = 0; i < 3; i++) {
            V3 p1 = p[i], p2 = p[(i + 1) % 3];
            V3 a = POI - p1, b = POI - p2, s = p2 - p1;
            double Al = dot(L.n, cross(s, a));
            if (!itself) {
                phiV = vortexPhi(PN, Al, a, b, s, L.l, L.m);
                phiDub += phiV;
            }
            phiSrc += srcSidePhi(PN, Al, phiV, a, b, s);
        }
        phiSrc /= (4 * kPi);
        if (!itself)
            phiDub /= (4 * kPi);
        else
            phiDub = -0.5;
    }
}

/* panel::dubPhiInf, CPanel/panel.cpp:208-252 */
double dubPhiInf(const V3* p, V3 center, V3 normal, double area, double longSide, V3 POI) {
    V3 pjk = POI - center;
    Local L = localSys(center, normal, p[0]);
    double PN = dot(pjk, L.n);
    if (norm(pjk) < 0.0000001) return -0.5;
    if (norm(pjk) / longSide > 5) return PN * area / (4 * kPi * std::pow(norm(pjk), 3));
    double phi = 0;
    for (int i = 0; i < 3; i++) {
        V3 p1 = p[i], p2 = p[(i + 1) % 3];
        V3 a = POI - p1, b = POI - p2, s = p2 - p1;
        double Al = dot(L.n, cross(s, a));
        phi += vortexPhi(PN, Al, a, b, s, L.l, L.m);
    }
    return phi / (4 * kPi);
}

/* bodyPanel::panelVInf, CPanel/bodyPanel.cpp:305-348 (srcSideV :375-390,
 * pntSrcV :397-400, pntDubV panel.cpp:773-776) */
void panelVInf(const V3* p, V3 center, V3 normal, double area, double longSide, V3 POI,
               V3& vSrc, V3& vDub) {
    V3 pjk = POI - center;
    Local L = localSys(center, normal, p[0]);
    double PN = dot(pjk, L.n);
    if (norm(pjk) / longSide > 5) {
        vSrc = -(area * pjk / (4 * kPi * std::pow(norm(pjk), 3)));
        vDub = area * (3 * dot(pjk, L.n) * pjk - std::pow(norm(pjk), 2) * L.n) /
               (4 * kPi * std::pow(norm(pjk), 5));
    } else {
        for (int i = 0; i < 3; i++) {
            V3 p1 = p[i], p2 = p[(i + 1) % 3];
            V3 a = POI - p1, b = POI - p2, s = a - b;
            double Al = dot(L.n, cross(s, a));
            vDub = vDub + vortexV(a, b, s);
            double A = norm(a), B = norm(b), S = norm(s);
            double GL = 0;
            if (std::abs(A + B - S) > 0 && S > 0) GL = 1 / S * std::log(std::abs((A + B + S) / (A + B - S)));
            double CJK = vortexPhi(PN, Al, a, b, s, L.l, L.m);
            vSrc = vSrc + (GL * (dot(s, L.m) * L.l - dot(s, L.l) * L.m) + CJK * L.n);
        }
        vDub = vDub / (4 * kPi);
        vSrc = vSrc / (4 * kPi);
    }
}

/* panel::dubVInf, CPanel/panel.cpp:666-704 (wake panels; s = p2 - p1 here, a - b in panelVInf) */
V3 dubVInf(const V3* p, V3 center, V3 normal, double area, double longSide, V3 POI) {
    V3 pjk = POI - center;
    Local L = localSys(center, normal, p[0]);
    if (norm(pjk) / longSide > 5)
        return area * (3 * dot(pjk, L.n) * pjk - std::pow(norm(pjk), 2) * L.n) /
               (4 * kPi * std::pow(norm(pjk), 5));  // pntDubV, panel.cpp:773-776
    V3 vel;
    for (int i = 0; i < 3; i++) {
        V3 p1 = p[i], p2 = p[(i + 1) % 3];
        V3 a = POI - p1, b = POI - p2, s = p2 - p1;
        vel = vel + vortexV(a, b, s);
    }
    return vel / (4 * kPi);
}

/* ---------------------------------------------------------------- topology */
int findEdge(Mesh& M, int n1, int n2) {  // geometry::findEdge, CPanel/geometry.cpp:771-787
    uint64_t lo = (uint64_t)std::min(n1, n2), hi = (uint64_t)std::max(n1, n2);
    uint64_t key = (lo << 32) | hi;
    auto it = M.edgeMap.find(key);
    if (it != M.edgeMap.end()) return it->second;
    Edge e;
    e.n1 = n1;
    e.n2 = n2;
    M.edges.push_back(e);
    int idx = (int)M.edges.size() - 1;
    M.edgeMap[key] = idx;
    return idx;
}

void addWakeLine(Mesh& M, Wake& W, const WakeLine& wl) {  // wake::addWakeLine, wake.cpp:140-144
    W.lines.push_back(wl);
    std::sort(W.lines.begin(), W.lines.end(),
              [](const WakeLine& a, const WakeLine& b) { return a.y() < b.y(); });
}

WakeLine makeWakeLine(Mesh& M, int upper, int lower, V3 normal) {  // wakeLine.cpp:20-46
    WakeLine wl;
    wl.upper = upper;
    wl.lower = lower;
    wl.normal = normal;
    int te = -1;
    for (int k = 0; k < 3; k++)
        if (M.edges[M.body[upper].edge[k]].TE) te = M.body[upper].edge[k];
    wl.p1 = M.nodes[M.edges[te].n1];
    wl.p2 = M.nodes[M.edges[te].n2];
    wl.pMid = (wl.p1 + wl.p2) / 2.0;
    return wl;
}

/* wakePanel::setParentPanels, CPanel/wakePanel.cpp:120-152 */
void setParentPanels(Mesh& M, int w, int upper, int lower) {
    WakeP& W = M.wakeP[w];
    M.body[upper].upper = true;
    M.body[lower].lower = true;
    if (!W.TEpanel) W.TEpanel = true;
    if (W.upperPan < 0) {
        W.upperPan = upper;
        W.lowerPan = lower;
    } else if (M.body[upper].center.x < W.center.x) {
        W.upperPan = upper;
        W.lowerPan = lower;
    }
    WakeLine wl = makeWakeLine(M, W.upperPan, W.lowerPan, W.normal);
    addWakeLine(M, M.wakes[W.wake], wl);
}

/* edge::checkTE, CPanel/edge.cpp:48-109 */
void checkTE(Mesh& M, int ei) {
    Edge& E = M.edges[ei];
    if (E.body.size() != 2) return;
    if (E.wake.size() == 1) {
        E.TE = true;
        const WakeP& W = M.wakeP[E.wake[0]];
        V3 normal = W.normal;
        V3 v1 = M.body[E.body[0]].center - W.center;
        V3 v2 = M.body[E.body[1]].center - W.center;
        double t1 = std::acos(dot(v1, normal) / (norm(v1) * norm(normal)));
        double t2 = std::acos(dot(v2, normal) / (norm(v2) * norm(normal)));
        int up, lo;
        if (t1 < t2) {
            up = E.body[0];
            lo = E.body[1];
        } else {
            up = E.body[1];
            lo = E.body[0];
        }
        int n1 = E.n1, n2 = E.n2, w = E.wake[0];
        setParentPanels(M, w, up, lo);
        M.nodeTE[n1] = true;
        M.nodeTE[n2] = true;
    } else {
        Body& b0 = M.body[E.body[0]];
        Body& b1 = M.body[E.body[1]];
        double angle = std::acos(dot(b0.normal, b1.normal));
        if (angle > 4.7 * kPi / 6 && b0.surfID == b1.surfID) {
            E.TE = true;
            M.nodeTE[E.n1] = true;
            M.nodeTE[E.n2] = true;
            b0.TEpanel = true;
            M.surfaces[b0.surf].LS = true;
            b1.TEpanel = true;
            M.surfaces[b1.surf].LS = true;
        }
    }
}

/* pow(x, e) for the small non-negative integer exponents of the CHTLS Taylor
 * monomials, evaluated as repeated products left to right.  The reference calls
 * std::pow (CPanel/chtlsnd.cpp:103,120); glibc's pow and x*x*x can differ by one
 * ulp for e = 3.  The repeated product is used here (and in the GPU library) so
 * that both sides evaluate the ill-conditioned CHTLS normal equations from
 * identical inputs. */
inline double powi(double x, int e) {
    double r = 1;
    for (int k = 0; k < e; k++) r = k == 0 ? x : r * x;
    return r;
}

int factorial(int i) {  // chtlsnd::factorial, CPanel/chtlsnd.cpp:304-321
    int out = 1;
    for (int k = 2; k <= i; k++) out *= k;
    return out;
}

/* bodyPanel::setTipFlag, CPanel/bodyPanel.cpp:58-95 */
void setTipFlag(Mesh& M, Body& P) {
    if (!M.surfaces[P.surf].LS) {
        P.tip = false;
        return;
    }
    int count = 0;
    for (int nb : P.neighbors) {
        V3 nn = M.body[nb].normal;
        double d = dot(P.normal, nn) / (norm(P.normal) * norm(nn));
        if (d > 1)
            d = 1;
        else if (d < -1)
            d = -1;
        double angle = std::acos(d);
        if (angle < std::pow(10.0, -8.0) && std::asin(nn.x) > -kPi / 12) count++;
    }
    if (count >= 2) P.tip = true;
}

/* bodyPanel::clusterTest, CPanel/bodyPanel.cpp:617-640 */
bool clusterTest(Mesh& M, int self, int other, double angle, bool upFlag, bool lowFlag) {
    Body& P = M.body[self];
    Body& O = M.body[other];
    if ((upFlag && O.lower) || (lowFlag && O.upper)) return false;
    if (P.tip != O.tip) return false;
    double d = dot(O.normal, P.normal);
    if (d > 1)
        d = 1;
    else if (d < -1)
        d = -1;
    return std::acos(d) < angle &&
           std::find(P.cluster.begin(), P.cluster.end(), other) == P.cluster.end() && other != self;
}

/* bodyPanel::setCluster, CPanel/bodyPanel.cpp:402-487 */
void setCluster(Mesh& M, int self) {
    Body& P = M.body[self];
    int dim = P.tip ? 2 : 3;
    size_t buffer = 10;
    size_t nObs = (size_t)(factorial(P.TSorder + dim) / (factorial(dim) * factorial(P.TSorder)) - 1) + buffer;
    size_t nPanels = (nObs + 1) / 2;
    size_t oldSize = P.cluster.size();
    P.cluster.push_back(self);
    bool upFlag = P.upper, lowFlag = P.lower;
    while (P.cluster.size() < nPanels) {
        std::vector<int> toAdd;
        for (size_t i = oldSize; i < P.cluster.size(); i++) {
            std::vector<int> temp = M.body[P.cluster[i]].neighbors;
            for (int t : temp) {
                if (clusterTest(M, self, t, 5 * kPi / 6, upFlag, lowFlag)) {
                    if (M.body[t].upper)
                        upFlag = true;
                    else if (M.body[t].lower)
                        lowFlag = true;
                    if (std::find(toAdd.begin(), toAdd.end(), t) == toAdd.end()) toAdd.push_back(t);
                }
            }
        }
        if (toAdd.empty() && P.cluster.size() < nPanels) {
            while (P.cluster.size() < nPanels + 1 && P.TSorder >= 1) {
                if (buffer > 0)
                    buffer -= 1;
                else
                    P.TSorder -= 1;
                nObs = (size_t)(factorial(P.TSorder + dim) / (factorial(dim) * factorial(P.TSorder))) + buffer;
                nPanels = (nObs + 1) / 2;
            }
            if (P.cluster.size() > nPanels + 1) P.cluster.erase(P.cluster.begin() + (long)(nPanels + 1), P.cluster.end());
            break;
        } else {
            oldSize = P.cluster.size();
            for (int t : toAdd) {
                P.cluster.push_back(t);
                if (P.cluster.size() == nPanels + 1) break;
            }
        }
    }
}

/* wake::addPanel, CPanel/wake.cpp:42-88 */
void wakeAddPanel(Mesh& M, Wake& W, int wi) {
    const WakeP& P = M.wakeP[wi];
    V3 pnt;
    if (W.wpanels.empty()) {
        pnt = M.nodes[P.node[0]];
        W.yMax = pnt.y;
        W.yMin = W.yMax;
        W.x0 = pnt.x;
        W.xf = W.x0;
        W.z0 = pnt.z;
        W.zf = W.z0;
        W.normal = P.normal;
    }
    for (int k = 0; k < 3; k++) {
        pnt = M.nodes[P.node[k]];
        if (pnt.y > W.yMax)
            W.yMax = pnt.y;
        else if (pnt.y < W.yMin)
            W.yMin = pnt.y;
        if (pnt.x > W.xf)
            W.xf = pnt.x;
        else if (pnt.x < W.x0)
            W.x0 = pnt.x;
        if (pnt.z > W.zf)
            W.zf = pnt.z;
        else if (pnt.z < W.z0)
            W.z0 = pnt.z;
    }
    W.wpanels.push_back(wi);
}

Mesh* buildMesh(const double* nodes, int64_t nn, const int64_t* tris, const int32_t* ids, int64_t nt) {
    Mesh* Mp = new Mesh();
    Mesh& M = *Mp;
    M.nodes.resize(nn);
    for (int64_t i = 0; i < nn; i++) M.nodes[i] = {nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]};
    M.nodeTE.assign(nn, false);
    std::vector<int64_t> conn(3 * nt);
    for (int64_t i = 0; i < 3 * nt; i++) conn[i] = tris[i] - 1;  // geometry.cpp:215

    // surface id scan, geometry.cpp:218-239
    int64_t wakeNodeStart = nn, wakeTriStart = nt;
    bool anyWake = false;
    for (int64_t i = 0; i < nt; i++) {
        if (ids[i] > 1000) anyWake = true;
        if (i > 0 && ids[i] > 1000 && ids[i - 1] < 1000) {
            wakeNodeStart = std::min(conn[3 * i], std::min(conn[3 * i + 1], conn[3 * i + 2]));
            wakeTriStart = i;
        }
    }
    if (anyWake) {  // geometry::correctWakeConnectivity, geometry.cpp:631-667
        double tol = 100000;  // shortestEdge, geometry.cpp:669-698
        for (int64_t i = 0; i < nt; i++)
            for (int j = 0; j < 3; j++) {
                V3 p1 = M.nodes[conn[3 * i + j]];
                V3 p2 = M.nodes[conn[3 * i + (j < 2 ? j + 1 : 0)]];
                double l = norm(p2 - p1);
                if (l < tol) tol = l;
            }
        std::vector<int64_t> repl(nn, -1);
        for (int64_t i = 0; i < wakeNodeStart; i++)
            for (int64_t j = wakeNodeStart; j < nn; j++) {
                V3 v = M.nodes[i] - M.nodes[j];
                double inf = std::max(std::abs(v.x), std::max(std::abs(v.y), std::abs(v.z)));
                if (inf < tol && repl[j] < 0) repl[j] = i;  // first replacement wins
            }
        for (int64_t i = wakeTriStart; i < nt; i++)
            for (int j = 0; j < 3; j++)
                if (conn[3 * i + j] < nn && repl[conn[3 * i + j]] >= 0) conn[3 * i + j] = repl[conn[3 * i + j]];
    }

    // geometry::createSurfaces, geometry.cpp:712-747
    for (int64_t i = 0; i < nt; i++) {
        int pn[3] = {(int)conn[3 * i], (int)conn[3 * i + 1], (int)conn[3 * i + 2]};
        int pe[3];
        for (int k = 0; k < 3; k++) pe[k] = findEdge(M, pn[k], pn[k < 2 ? k + 1 : 0]);
        bool newGroup = (i == 0 || ids[i] != ids[i - 1]);
        if (ids[i] <= 1000) {
            if (newGroup) {
                Surface s;
                s.id = ids[i];
                M.surfaces.push_back(s);
            }
            Body B;
            for (int k = 0; k < 3; k++) {
                B.node[k] = pn[k];
                B.edge[k] = pe[k];
            }
            B.surfID = ids[i];
            B.fileTri = (int)i;
            B.surf = (int)M.surfaces.size() - 1;
            setGeom(M, B);
            M.body.push_back(B);
            int bi = (int)M.body.size() - 1;
            for (int k = 0; k < 3; k++) {
                M.edges[pe[k]].body.push_back(bi);
                checkTE(M, pe[k]);
            }
            M.surfaces[B.surf].panels.push_back(bi);
        } else {
            if (newGroup) {
                Wake w;
                w.id = ids[i];
                M.wakes.push_back(w);
            }
            WakeP W;
            for (int k = 0; k < 3; k++) {
                W.node[k] = pn[k];
                W.edge[k] = pe[k];
            }
            W.surfID = ids[i];
            W.fileTri = (int)i;
            W.wake = (int)M.wakes.size() - 1;
            setGeom(M, W);
            M.wakeP.push_back(W);
            int wi = (int)M.wakeP.size() - 1;
            for (int k = 0; k < 3; k++) {
                M.edges[pe[k]].wake.push_back(wi);
                checkTE(M, pe[k]);
            }
            wakeAddPanel(M, M.wakes[W.wake], wi);
        }
    }

    // edge::setNeighbors, geometry.cpp:420-423 / edge.cpp:189-196
    for (auto& e : M.edges)
        if (e.body.size() == 2) {
            M.body[e.body[0]].neighbors.push_back(e.body[1]);
            M.body[e.body[1]].neighbors.push_back(e.body[0]);
        }

    // wake merge, geometry.cpp:426-447 (wake::isSameWake/mergeWake, wake.cpp:90-133)
    if (M.wakes.size() > 1) {
        std::vector<int> newWakes;
        bool merged = false;
        for (size_t i = 0; i < M.wakes.size(); i++)
            for (size_t j = i; j < M.wakes.size(); j++) {
                if (i == j || M.wakes[i].dead || M.wakes[j].dead) continue;
                Wake& a = M.wakes[i];
                Wake& b = M.wakes[j];
                double eps = std::pow(10.0, -2.0);
                if (std::abs(b.x0 - a.x0) < eps && std::abs(b.z0 - a.z0) < eps && std::abs(b.xf - a.xf) < eps &&
                    std::abs(b.zf - a.zf) < eps) {
                    for (int w : b.wpanels) {
                        a.wpanels.push_back(w);
                        M.wakeP[w].wake = (int)i;
                    }
                    for (const auto& wl : b.lines) addWakeLine(M, a, wl);
                    if (b.yMin < a.yMin) a.yMin = b.yMin;
                    if (b.yMax > a.yMax) a.yMax = b.yMax;
                    b.dead = true;
                    newWakes.push_back((int)i);
                    merged = true;
                }
            }
        if (merged) {
            std::vector<Wake> keep;
            std::vector<int> remap(M.wakes.size(), -1);
            for (int w : newWakes) {
                remap[w] = (int)keep.size();
                keep.push_back(M.wakes[w]);
            }
            for (auto& wp : M.wakeP) wp.wake = remap[wp.wake];
            M.wakes = keep;
        }
    }

    // collect panels, geometry.cpp:452-469
    for (const auto& s : M.surfaces) M.bPanels.insert(M.bPanels.begin(), s.panels.begin(), s.panels.end());
    for (const auto& w : M.wakes)
        for (int wp : w.wpanels) M.wPanels.push_back(wp);
    M.bodyIndex.assign(M.body.size(), -1);
    for (size_t i = 0; i < M.bPanels.size(); i++) {
        M.bodyIndex[M.bPanels[i]] = (int)i;
        M.body[M.bPanels[i]].index = (int)i;
    }
    // setTipFlag / setCluster, geometry.cpp:473-484
    for (int b : M.bPanels) setTipFlag(M, M.body[b]);
    for (int b : M.bPanels) setCluster(M, b);
    return Mp;
}

/* wakePanel::interpPanels, CPanel/wakePanel.cpp:48-81 */
void interpPanels(const Mesh& M, int wi, int idx[4], double& coef) {
    const WakeP& W = M.wakeP[wi];
    const std::vector<WakeLine>& wl = M.wakes[W.wake].lines;
    const WakeLine *w1 = nullptr, *w2 = nullptr;
    double y = W.center.y;
    if (y < wl[1].y()) {
        w1 = &wl[0];
        w2 = &wl[1];
    } else if (y >= wl.back().y()) {
        w1 = &wl[wl.size() - 2];
        w2 = &wl[wl.size() - 1];
    } else {
        for (size_t i = 1; i < wl.size() - 1; i++)
            if (wl[i].y() <= y && wl[i + 1].y() > y) {
                w1 = &wl[i];
                w2 = &wl[i + 1];
            }
    }
    coef = (y - w1->y()) / (w2->y() - w1->y());
    idx[0] = M.bodyIndex[w1->upper];
    idx[1] = M.bodyIndex[w1->lower];
    idx[2] = M.bodyIndex[w2->upper];
    idx[3] = M.bodyIndex[w2->lower];
}

void triVerts(const Mesh& M, const Tri& T, V3* p) {
    for (int k = 0; k < 3; k++) p[k] = M.nodes[T.node[k]];
}

/* ------------------------------------------------------------------- CHTLS */
/* chtlsnd::derivSequence / sortBySum, CPanel/chtlsnd.cpp:211-274 */
std::vector<std::vector<int>> derivSequence(int q, int N) {
    std::vector<std::vector<int>> d;
    if (q == 0) {
        d.push_back(std::vector<int>(N, 0));
        return d;
    }
    for (int i = 0; i <= q; i++) {
        if (N > 1) {
            auto sub = derivSequence(q - i, N - 1);
            for (auto& r : sub) {
                r.push_back(i);
                d.push_back(r);
            }
        } else {
            d.push_back(std::vector<int>{i});
        }
    }
    return d;
}
int rowSum(const std::vector<int>& r) {
    int s = 0;
    for (int v : r) s += v;
    return s;
}
std::vector<std::vector<int>> sortBySum(const std::vector<std::vector<int>>& m) {
    std::vector<std::vector<int>> out{m[0]};
    for (size_t i = 1; i < m.size(); i++) {
        bool flag = false;
        for (size_t j = 0; j < out.size(); j++)
            if (rowSum(m[i]) < rowSum(out[j])) {
                out.insert(out.begin() + (long)j, m[i]);
                flag = true;
                break;
            }
        if (!flag) out.push_back(m[i]);
    }
    return out;
}

/* Householder QR solve of a square system, restating the unblocked Householder QR
 * used by Eigen::HouseholderQR for small matrices (makeHouseholder /
 * applyHouseholderOnTheLeft), then Q^T b and back substitution.
 * M: t x t row-major (destroyed); R: t x ncol row-major rhs, overwritten by the solution. */
void qrSolve(std::vector<double>& Mm, int t, std::vector<double>& R, int ncol) {
    std::vector<double> tau(t);
    const double tiny = std::numeric_limits<double>::min();
    for (int k = 0; k < t; k++) {
        double c0 = Mm[k * t + k];
        double tail = 0;
        for (int i = k + 1; i < t; i++) tail += Mm[i * t + k] * Mm[i * t + k];
        double beta;
        if (tail <= tiny) {
            tau[k] = 0;
            beta = c0;
            for (int i = k + 1; i < t; i++) Mm[i * t + k] = 0;
        } else {
            beta = std::sqrt(c0 * c0 + tail);
            if (c0 >= 0) beta = -beta;
            for (int i = k + 1; i < t; i++) Mm[i * t + k] /= (c0 - beta);
            tau[k] = (beta - c0) / beta;
        }
        Mm[k * t + k] = beta;
        if (tau[k] != 0) {
            for (int j = k + 1; j < t; j++) {
                double tmp = Mm[k * t + j];
                for (int i = k + 1; i < t; i++) tmp += Mm[i * t + k] * Mm[i * t + j];
                Mm[k * t + j] -= tau[k] * tmp;
                for (int i = k + 1; i < t; i++) Mm[i * t + j] -= tau[k] * Mm[i * t + k] * tmp;
            }
        }
    }
    for (int k = 0; k < t; k++) {  // apply Q^T = H_{t-1} ... H_0
        if (tau[k] == 0) continue;
        for (int c = 0; c < ncol; c++) {
            double tmp = R[k * ncol + c];
            for (int i = k + 1; i < t; i++) tmp += Mm[i * t + k] * R[i * ncol + c];
            R[k * ncol + c] -= tau[k] * tmp;
            for (int i = k + 1; i < t; i++) R[i * ncol + c] -= tau[k] * Mm[i * t + k] * tmp;
        }
    }
    for (int c = 0; c < ncol; c++)
        for (int i = t - 1; i >= 0; i--) {
            double s = R[i * ncol + c];
            for (int j = i + 1; j < t; j++) s -= Mm[i * t + j] * R[j * ncol + c];
            R[i * ncol + c] = s / Mm[i * t + i];
        }
}

/* chtlsnd::chtlsnd (unconstrained branch), CPanel/chtlsnd.cpp:20-140,189-196.
 * Returns the first N rows of F (N x nf, row-major), already redimensionalised. */
std::vector<double> chtlsF(const std::vector<double>& X0, const std::vector<std::vector<double>>& Xf, int order,
                           const std::vector<std::vector<double>>& Xb, const std::vector<std::vector<double>>& Vb) {
    int N = (int)X0.size();
    int nf = (int)Xf.size(), nb = (int)Xb.size();
    std::vector<std::vector<double>> dXf(nf, std::vector<double>(N)), dXb(nb, std::vector<double>(N));
    double rmax = 0;
    for (int i = 0; i < nf; i++) {
        double s = 0;
        for (int k = 0; k < N; k++) {
            dXf[i][k] = Xf[i][k] - X0[k];
            s += dXf[i][k] * dXf[i][k];
        }
        double r = std::sqrt(s);
        if (r > rmax) rmax = r;
    }
    for (auto& r : dXf)
        for (auto& v : r) v /= rmax;
    for (int i = 0; i < nb; i++)
        for (int k = 0; k < N; k++) dXb[i][k] = Xb[i][k] - X0[k];
    for (auto& r : dXb)
        for (auto& v : r) v /= rmax;
    auto rnorm = [](const std::vector<double>& r) {
        double s = 0;
        for (double v : r) s += v * v;
        return std::sqrt(s);
    };
    std::vector<double> Wf(nf), Wb(nb);
    for (int i = 0; i < nf; i++) Wf[i] = 1 / rnorm(dXf[i]);
    for (int i = 0; i < nb; i++) Wb[i] = 1 / rnorm(dXb[i]);
    auto ms = sortBySum(derivSequence(order, N));
    ms.erase(ms.begin());
    int t = (int)ms.size();
    std::vector<double> A(nf * t), B(nb * t);
    for (int k = 0; k < t; k++) {
        double fact = 1;
        for (int i = 0; i < N; i++) fact /= factorial(ms[k][i]);
        for (int i = 0; i < nf; i++) {
            double prod = 1;
            for (int ii = 0; ii < N; ii++) prod *= powi(dXf[i][ii], ms[k][ii]);
            A[i * t + k] = fact * prod;
        }
        for (int i = 0; i < nb; i++) {
            double asum = 0;
            for (int a = 0; a < N; a++) {
                if (ms[k][a] != 0) {
                    std::vector<int> ps = ms[k];
                    ps[a] -= 1;
                    double prod = 1;
                    for (int ii = 0; ii < N; ii++) prod *= powi(dXb[i][ii], ps[ii]);
                    asum += Vb[i][a] * ms[k][a] * prod;
                }
            }
            B[i * t + k] = fact * asum;
        }
    }
    std::vector<double> Mm(t * t, 0.0);
    for (int r = 0; r < t; r++)
        for (int c = 0; c < t; c++) {
            double s = 0;
            for (int i = 0; i < nf; i++) s += A[i * t + r] * Wf[i] * A[i * t + c];
            double s2 = 0;
            for (int i = 0; i < nb; i++) s2 += B[i * t + r] * Wb[i] * B[i * t + c];
            Mm[r * t + c] = s + s2;
        }
    std::vector<double> R(t * nf);
    for (int r = 0; r < t; r++)
        for (int i = 0; i < nf; i++) R[r * nf + i] = A[i * t + r] * Wf[i];
    qrSolve(Mm, t, R, nf);
    std::vector<double> F(N * nf);
    for (int r = 0; r < N; r++)
        for (int i = 0; i < nf; i++) F[r * nf + i] = R[r * nf + i] / powi(rmax, rowSum(ms[r]));
    return F;
}

/* bodyPanel::velocity3D, CPanel/bodyPanel.cpp:559-589 */
V3 velocity3D(const Mesh& M, const Body& P, const std::vector<double>& phi) {
    std::vector<int> cl(P.cluster.begin() + 1, P.cluster.end());
    std::vector<std::vector<double>> Xf, Vb;
    std::vector<double> df;
    double phiP = phi[P.index];
    for (int b : cl) {
        const Body& Q = M.body[b];
        Xf.push_back({Q.center.x, Q.center.y, Q.center.z});
        Vb.push_back({Q.bez.x, Q.bez.y, Q.bez.z});
        df.push_back(phi[Q.index] - phiP);
    }
    auto F = chtlsF({P.center.x, P.center.y, P.center.z}, Xf, P.TSorder, Xf, Vb);
    int nf = (int)cl.size();
    V3 v;
    double c[3];
    for (int r = 0; r < 3; r++) {
        double s = 0;
        for (int i = 0; i < nf; i++) s += F[r * nf + i] * df[i];
        c[r] = s;
    }
    v = {c[0], c[1], c[2]};
    return v;
}

/* bodyPanel::velocity2D, CPanel/bodyPanel.cpp:524-557 */
V3 velocity2D(const Mesh& M, const Body& P, const std::vector<double>& phi) {
    std::vector<int> cl(P.cluster.begin() + 1, P.cluster.end());
    Local L = localSys(P.center, P.normal, M.nodes[P.node[0]]);
    auto g2l = [&](V3 g) {
        V3 d = g - P.center;
        return V3{dot(L.l, d), dot(L.m, d), dot(L.n, d)};
    };
    V3 x0 = g2l(P.center);
    std::vector<std::vector<double>> Xf, Xb, Vb;
    std::vector<double> df;
    double phiP = phi[P.index];
    for (int b : cl) {
        const Body& Q = M.body[b];
        V3 q = g2l(Q.center);
        Xf.push_back({q.x, q.y});
        df.push_back(phi[Q.index] - phiP);
    }
    auto F = chtlsF({x0.x, x0.y}, Xf, P.TSorder, Xb, Vb);
    int nf = (int)cl.size();
    double c[2];
    for (int r = 0; r < 2; r++) {
        double s = 0;
        for (int i = 0; i < nf; i++) s += F[r * nf + i] * df[i];
        c[r] = s;
    }
    // local2global(vLocal,false): L^T * vLocal
    V3 v = L.l * c[0] + L.m * c[1] + L.n * 0.0;
    return v;
}

/* ------------------------------------------------------------ Trefftz plane */
/* wake::wakeStrength, CPanel/wake.cpp:478-506 */
double wakeStrength(const Mesh& M, const Wake& W, const std::vector<double>& mu, double y) {
    const auto& wl = W.lines;
    const WakeLine *w1 = nullptr, *w2 = nullptr;
    if (y < wl[1].y()) {
        w1 = &wl[0];
        w2 = &wl[1];
    } else if (y >= wl.back().y()) {
        w1 = &wl[wl.size() - 2];
        w2 = &wl[wl.size() - 1];
    } else {
        for (size_t i = 1; i < wl.size() - 1; i++)
            if (wl[i].y() <= y && wl[i + 1].y() > y) {
                w1 = &wl[i];
                w2 = &wl[i + 1];
            }
    }
    double interp = (y - w1->y()) / (w2->y() - w1->y());
    double s1 = mu[M.bodyIndex[w1->upper]] - mu[M.bodyIndex[w1->lower]];
    double s2 = mu[M.bodyIndex[w2->upper]] - mu[M.bodyIndex[w2->lower]];
    return s1 + interp * (s2 - s1);
}

/* wake::pntInWake, CPanel/wake.cpp:601-640 */
V3 pntInWake(const Mesh& M, const Wake& W, double x, double y) {
    V3 yDir{0, 1, 0};
    for (int wi : W.wpanels) {
        const WakeP& P = M.wakeP[wi];
        if (!P.TEpanel) continue;
        const Body& U = M.body[P.upperPan];
        for (int k = 0; k < 3; k++) {
            const Edge& e = M.edges[U.edge[k]];
            if (!e.TE) continue;
            V3 p1 = M.nodes[e.n1], p2 = M.nodes[e.n2];
            if ((p1.y <= y && p2.y >= y) || (p1.y >= y && p2.y <= y)) {
                double t = (y - p1.y) / (p2.y - p1.y);
                V3 tvec = p2 - p1;
                V3 pnt = p1 + t * tvec;
                V3 out = -cross(P.normal, yDir);
                if (out.x < 0) out = out * -1.0;
                double scale = (x - pnt.x) / out.x;
                return pnt + scale * out;
            }
        }
    }
    return V3{0, 0, 0};
}

struct WakeEval {  // geometry::wakePotential, CPanel/geometry.cpp:1229-1237
    const Mesh& M;
    const std::vector<double>& wmu;  // per wPanels entry
    double operator()(V3 pnt) const {
        double pot = 0;
        for (size_t i = 0; i < M.wPanels.size(); i++) {
            const WakeP& P = M.wakeP[M.wPanels[i]];
            V3 p[3];
            triVerts(M, P, p);
            pot += -wmu[i] * dubPhiInf(p, P.center, P.normal, P.area, P.longSide, pnt);  // wakePanel::panelPhi
        }
        return pot;
    }
};

/* wake::Vradial, CPanel/wake.cpp:508-597 */
double Vradial(const Wake& W, const WakeEval& pot, V3 pWake) {
    double r, theta = kPi / 4, dZmax = 0.3, delZ;
    V3 POI;
    POI.x = pWake.x;
    if (pWake.y >= 0)
        r = W.yMax - pWake.y;
    else
        r = pWake.y - W.yMin;
    delZ = r * std::sin(theta);
    if (delZ > dZmax) {
        delZ = dZmax;
        theta = std::asin(dZmax / r);
    }
    if (pWake.y >= 0)
        POI.y = W.yMax - r * std::cos(theta);
    else
        POI.y = W.yMin + r * std::cos(theta);
    POI.z = pWake.z + r * std::sin(theta);
    const int nPnts = 6;
    double dz = 0.5 * delZ;
    double step = 2 * dz / (nPnts - 1);
    double phiPOI = pot(POI);
    std::vector<double> dPhiy(nPnts), dPhiz(nPnts);
    std::vector<std::vector<double>> dY(nPnts, std::vector<double>(1)), dZ(nPnts, std::vector<double>(1));
    for (int i = 0; i < nPnts; i++) {
        double delta = -dz + i * step;
        V3 pnt1 = POI + delta * V3{0, 1, 0};
        V3 pnt2 = POI + delta * V3{0, 0, 1};
        dPhiy[i] = pot(pnt1) - phiPOI;
        dPhiz[i] = pot(pnt2) - phiPOI;
        dY[i][0] = pnt1.y - POI.y;
        dZ[i][0] = pnt2.z - POI.z;
    }
    std::vector<std::vector<double>> none;
    auto Fy = chtlsF({0.0}, dY, 3, none, none);
    auto Fz = chtlsF({0.0}, dZ, 3, none, none);
    double v = 0, w = 0;
    for (int i = 0; i < nPnts; i++) v += Fy[i] * dPhiy[i];
    for (int i = 0; i < nPnts; i++) w += Fz[i] * dPhiz[i];
    return std::sqrt(std::pow(v, 2) + std::pow(w, 2));
}

/* wake::trefftzPlane, CPanel/wake.cpp:146-188 */
void trefftzPlane(const Mesh& M, const Wake& W, const WakeEval& pot, const std::vector<double>& mu, double Vinf,
                  double Sref, double& CL, double& CD, std::vector<double>& yLoc, std::vector<double>& Cl,
                  std::vector<double>& Cd) {
    const int nPnts = 164;
    yLoc.assign(nPnts + 1, 0.0);
    Cl.assign(nPnts + 1, 0.0);
    Cd.assign(nPnts + 1, 0.0);
    yLoc[0] = W.yMin;
    yLoc[nPnts] = W.yMax;
    double step = (W.yMax - W.yMin) / nPnts;
    double xT = W.x0 + 2 * (W.xf - W.x0) / 3;
    for (int i = 1; i < nPnts; i++) {
        yLoc[i] = W.yMin + i * step;
        V3 pw = pntInWake(M, W, xT, yLoc[i]);
        double w = Vradial(W, pot, pw);
        double dPhi = -wakeStrength(M, W, mu, yLoc[i]);
        Cl[i] = 2 * dPhi / (Vinf * Sref);
        Cd[i] = dPhi * w / (Vinf * Vinf * Sref);
    }
    CL = 0;
    CD = 0;
    int i = 0;
    while (i < nPnts + 1 - 2) {
        CL += 1.0 / 3 * step * (Cl[i] + 4 * Cl[i + 1] + Cl[i + 2]);
        CD += 1.0 / 3 * step * (Cd[i] + 4 * Cd[i + 1] + Cd[i + 2]);
        i += 2;
    }
}

/* ----------------------------------------------------------------- threads */
template <class F>
void parallelFor(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 2) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        int64_t a = t * chunk, b = std::min(n, a + chunk);
        if (a >= b) break;
        th.emplace_back([=] { f(a, b); });
    }
    for (auto& x : th) x.join();
}

void matvec(const double* A, int64_t n, const double* x, double* y, int nthreads) {
    parallelFor(n, nthreads, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) y[i] = 0;
        for (int64_t j = 0; j < n; j++) {
            const double* col = A + j * n;
            double xj = x[j];
            for (int64_t i = a; i < b; i++) y[i] += col[i] * xj;
        }
    });
}

/* cpCase::windToBody, CPanel/cpCase.cpp:142-165 */
void windToBody(double V, double alpha, double beta, V3& Vinf, double T[3][3]) {
    alpha *= kPi / 180;
    beta *= kPi / 180;
    T[0][0] = std::cos(alpha) * std::cos(beta);
    T[0][1] = std::cos(alpha) * std::sin(beta);
    T[0][2] = -std::sin(alpha);
    T[1][0] = -std::sin(beta);
    T[1][1] = std::cos(beta);
    T[1][2] = 0;
    T[2][0] = std::sin(alpha) * std::cos(beta);
    T[2][1] = std::sin(alpha) * std::sin(beta);
    T[2][2] = std::cos(alpha);
    Vinf = {T[0][0] * V + T[0][1] * 0 + T[0][2] * 0, T[1][0] * V + T[1][1] * 0 + T[1][2] * 0,
            T[2][0] * V + T[2][1] * 0 + T[2][2] * 0};
}

}  // namespace

/* ====================================================================== C ABI */
extern "C" {

void* cpo_mesh_new(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids, int64_t n_tris) {
    return buildMesh(nodes, n_nodes, tris, ids, n_tris);
}
void cpo_mesh_free(void* m) { delete (Mesh*)m; }
int64_t cpo_n_body(void* m) { return (int64_t)((Mesh*)m)->bPanels.size(); }
int64_t cpo_n_wake(void* m) { return (int64_t)((Mesh*)m)->wPanels.size(); }
int64_t cpo_n_wakes(void* m) { return (int64_t)((Mesh*)m)->wakes.size(); }
int64_t cpo_n_wakelines(void* m, int64_t w) { return (int64_t)((Mesh*)m)->wakes[w].lines.size(); }

void cpo_body_table(void* mp, double* out) {
    Mesh& M = *(Mesh*)mp;
    for (size_t i = 0; i < M.bPanels.size(); i++) {
        const Body& B = M.body[M.bPanels[i]];
        Local L = localSys(B.center, B.normal, M.nodes[B.node[0]]);
        double* o = out + 18 * i;
        o[0] = B.center.x; o[1] = B.center.y; o[2] = B.center.z;
        o[3] = B.normal.x; o[4] = B.normal.y; o[5] = B.normal.z;
        o[6] = L.l.x; o[7] = L.l.y; o[8] = L.l.z;
        o[9] = B.area; o[10] = B.longSide;
        o[11] = B.tip; o[12] = B.upper; o[13] = B.lower; o[14] = B.TSorder;
        o[15] = B.surfID; o[16] = (double)B.cluster.size(); o[17] = B.fileTri;
    }
}

void cpo_wake_table(void* mp, double* out, int32_t* idx4, double* coef) {
    Mesh& M = *(Mesh*)mp;
    for (size_t i = 0; i < M.wPanels.size(); i++) {
        const WakeP& W = M.wakeP[M.wPanels[i]];
        double* o = out + 8 * i;
        o[0] = W.center.x; o[1] = W.center.y; o[2] = W.center.z;
        o[3] = W.normal.x; o[4] = W.normal.y; o[5] = W.normal.z;
        o[6] = W.area; o[7] = W.longSide;
        int idx[4];
        double c;
        interpPanels(M, M.wPanels[i], idx, c);
        for (int k = 0; k < 4; k++) idx4[4 * i + k] = idx[k];
        coef[i] = c;
    }
}

void cpo_clusters(void* mp, int32_t* out) {
    Mesh& M = *(Mesh*)mp;
    for (size_t i = 0; i < M.bPanels.size(); i++) {
        const Body& B = M.body[M.bPanels[i]];
        for (int k = 0; k < 32; k++) out[32 * i + k] = k < (int)B.cluster.size() ? M.bodyIndex[B.cluster[k]] : -1;
    }
}

void cpo_body_verts(void* mp, double* out) {
    Mesh& M = *(Mesh*)mp;
    for (size_t i = 0; i < M.bPanels.size(); i++) {
        const Body& B = M.body[M.bPanels[i]];
        for (int k = 0; k < 3; k++) {
            V3 p = M.nodes[B.node[k]];
            out[9 * i + 3 * k] = p.x; out[9 * i + 3 * k + 1] = p.y; out[9 * i + 3 * k + 2] = p.z;
        }
    }
}
void cpo_wake_verts(void* mp, double* out) {
    Mesh& M = *(Mesh*)mp;
    for (size_t i = 0; i < M.wPanels.size(); i++) {
        const WakeP& W = M.wakeP[M.wPanels[i]];
        for (int k = 0; k < 3; k++) {
            V3 p = M.nodes[W.node[k]];
            out[9 * i + 3 * k] = p.x; out[9 * i + 3 * k + 1] = p.y; out[9 * i + 3 * k + 2] = p.z;
        }
    }
}

void cpo_tri_phi_inf(const double* v9, const double* poi, double* phi_src, double* phi_dub) {
    Pan P = makePan(v9);
    double s = 0, d = 0;
    panelPhiInf(P.p, P.center, P.normal, P.area, P.longSide, {poi[0], poi[1], poi[2]}, s, d);
    *phi_src = s;
    *phi_dub = d;
}
double cpo_tri_dub_phi_inf(const double* v9, const double* poi) {
    Pan P = makePan(v9);
    return dubPhiInf(P.p, P.center, P.normal, P.area, P.longSide, {poi[0], poi[1], poi[2]});
}
void cpo_tri_v_inf(const double* v9, const double* poi, double* v_src, double* v_dub) {
    Pan P = makePan(v9);
    V3 s, d;
    panelVInf(P.p, P.center, P.normal, P.area, P.longSide, {poi[0], poi[1], poi[2]}, s, d);
    v_src[0] = s.x; v_src[1] = s.y; v_src[2] = s.z;
    v_dub[0] = d.x; v_dub[1] = d.y; v_dub[2] = d.z;
}

void cpo_tri_dub_v_inf(const double* v9, const double* poi, double* v_dub) {
    Pan P = makePan(v9);
    V3 d = dubVInf(P.p, P.center, P.normal, P.area, P.longSide, {poi[0], poi[1], poi[2]});
    v_dub[0] = d.x; v_dub[1] = d.y; v_dub[2] = d.z;
}

void cpo_panels_velocity(const double* bverts, const double* sigma, const double* mu, int64_t nb,
                         const double* wverts, const double* wmu, int64_t nw, const double* pts, int64_t m,
                         double* vel, int nthreads) {
    std::vector<Pan> B(nb), W(nw);
    for (int64_t j = 0; j < nb; j++) B[j] = makePan(bverts + 9 * j);
    for (int64_t j = 0; j < nw; j++) W[j] = makePan(wverts + 9 * j);
    parallelFor(m, nthreads, [&](int64_t ia, int64_t ib) {
        for (int64_t i = ia; i < ib; i++) {
            V3 poi{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
            V3 acc;
            for (int64_t j = 0; j < nb; j++) {  // bodyPanel::panelV, bodyPanel.cpp:122-130
                V3 vs, vd;
                panelVInf(B[j].p, B[j].center, B[j].normal, B[j].area, B[j].longSide, poi, vs, vd);
                acc = acc + (sigma[j] * vs + mu[j] * vd);
            }
            for (int64_t j = 0; j < nw; j++)  // wakePanel::panelV, wakePanel.cpp:89-92
                acc = acc + wmu[j] * dubVInf(W[j].p, W[j].center, W[j].normal, W[j].area, W[j].longSide, poi);
            vel[3 * i] = acc.x; vel[3 * i + 1] = acc.y; vel[3 * i + 2] = acc.z;
        }
    });
}

void cpo_set_inf_coeff(void* mp, double* A, double* B, int64_t r0, int64_t r1, int nthreads) {
    Mesh& M = *(Mesh*)mp;
    int64_t n = (int64_t)M.bPanels.size();
    int64_t ld = r1 - r0;
    // A.setZero(); B.setZero() (rows r0..r1 only)
    for (int64_t q = 0; q < n * ld; q++) {
        A[q] = 0;
        B[q] = 0;
    }
    std::vector<V3> centers(n);
    for (int64_t i = 0; i < n; i++) centers[i] = M.body[M.bPanels[i]].center;
    // body loop: j (source) outer, i (target) inner -- geometry.cpp:827-841
    parallelFor(n, nthreads, [&](int64_t ja, int64_t jb) {
        for (int64_t j = ja; j < jb; j++) {
            const Body& S = M.body[M.bPanels[j]];
            V3 p[3];
            triVerts(M, S, p);
            for (int64_t i = r0; i < r1; i++)
                panelPhiInf(p, S.center, S.normal, S.area, S.longSide, centers[i], B[j * ld + (i - r0)],
                            A[j * ld + (i - r0)]);
        }
    });
    // wake scatter, geometry.cpp:853-873 (sequential over wake panels for each row)
    int64_t nw = (int64_t)M.wPanels.size();
    std::vector<int> idx(4 * nw);
    std::vector<double> coef(nw);
    for (int64_t j = 0; j < nw; j++) interpPanels(M, M.wPanels[j], &idx[4 * j], coef[j]);
    parallelFor(ld, nthreads, [&](int64_t a, int64_t b) {
        for (int64_t j = 0; j < nw; j++) {
            const WakeP& W = M.wakeP[M.wPanels[j]];
            V3 p[3];
            triVerts(M, W, p);
            double c = coef[j];
            for (int64_t ii = a; ii < b; ii++) {
                int64_t i = r0 + ii;
                double infl = dubPhiInf(p, W.center, W.normal, W.area, W.longSide, centers[i]);
                A[(int64_t)idx[4 * j + 0] * ld + ii] += infl * (1 - c);
                A[(int64_t)idx[4 * j + 1] * ld + ii] += infl * (c - 1);
                A[(int64_t)idx[4 * j + 2] * ld + ii] += infl * c;
                A[(int64_t)idx[4 * j + 3] * ld + ii] -= infl * c;
            }
        }
    });
}

int cpo_bicgstab(const double* A, int64_t n, const double* b, double* x, double tol, int64_t maxIters,
                 int64_t* iters_out, double* err_out, int nthreads) {
    // Eigen::BiCGSTAB with DiagonalPreconditioner and a zero initial guess.
    std::vector<double> invd(n);
    for (int64_t i = 0; i < n; i++) {
        double d = A[i * n + i];
        invd[i] = d != 0 ? 1.0 / d : 1.0;
    }
    auto dotv = [&](const std::vector<double>& u, const std::vector<double>& v) {
        double s = 0;
        for (int64_t i = 0; i < n; i++) s += u[i] * v[i];
        return s;
    };
    for (int64_t i = 0; i < n; i++) x[i] = 0;
    std::vector<double> r(b, b + n), r0 = r, v(n, 0.0), p(n, 0.0), y(n), z(n), s(n), t(n), tmp(n);
    double r0_sqnorm = dotv(r0, r0);
    double rhs_sqnorm = 0;
    for (int64_t i = 0; i < n; i++) rhs_sqnorm += b[i] * b[i];
    if (rhs_sqnorm == 0) {
        *iters_out = 0;
        *err_out = 0;
        return 1;
    }
    double rho = 1, alpha = 1, w = 1;
    double tol2 = tol * tol * rhs_sqnorm;
    double eps = std::numeric_limits<double>::epsilon();
    double eps2 = eps * eps;
    int64_t i = 0, restarts = 0;
    while (dotv(r, r) > tol2 && i < maxIters) {
        double rho_old = rho;
        rho = dotv(r0, r);
        if (std::abs(rho) < eps2 * r0_sqnorm) {
            matvec(A, n, x, tmp.data(), nthreads);
            for (int64_t k = 0; k < n; k++) r[k] = b[k] - tmp[k];
            r0 = r;
            rho = r0_sqnorm = dotv(r, r);
            if (restarts++ == 0) i = 0;
        }
        double beta = (rho / rho_old) * (alpha / w);
        for (int64_t k = 0; k < n; k++) p[k] = r[k] + beta * (p[k] - w * v[k]);
        for (int64_t k = 0; k < n; k++) y[k] = invd[k] * p[k];
        matvec(A, n, y.data(), v.data(), nthreads);
        alpha = rho / dotv(r0, v);
        for (int64_t k = 0; k < n; k++) s[k] = r[k] - alpha * v[k];
        for (int64_t k = 0; k < n; k++) z[k] = invd[k] * s[k];
        matvec(A, n, z.data(), t.data(), nthreads);
        double tt = dotv(t, t);
        w = tt > 0 ? dotv(t, s) / tt : 0;
        for (int64_t k = 0; k < n; k++) x[k] += alpha * y[k] + w * z[k];
        for (int64_t k = 0; k < n; k++) r[k] = s[k] - w * t[k];
        ++i;
    }
    *err_out = std::sqrt(dotv(r, r) / rhs_sqnorm);
    *iters_out = i;
    return 1;
}

}  // extern "C"

namespace {

/* The surface pass of cpCase::compVelocity (CPanel/cpCase.cpp:342-365) and of the steady
 * branch of cpCaseVP::compVelocity (CPanel/cpCaseVP.cpp:370-393): CHTLS velocity from the
 * panel potentials (bodyPanel::pntVelocity, bodyPanel.cpp:490-522), Cp against V, forces
 * and moments.  Fills Fbody, Fwind and CM of res. */
void surfacePost(Mesh& M, const std::vector<double>& phi, V3 Vinf, const double T[3][3], const cpo_case_params* p,
                 double PG, double* vel_out, double* cp_out, cpo_case_result* res) {
    const int64_t n = (int64_t)M.bPanels.size();
    V3 F{0, 0, 0}, CM{0, 0, 0};
    V3 cg{p->cg[0], p->cg[1], p->cg[2]};
    for (int64_t i = 0; i < n; i++) {
        const Body& B = M.body[M.bPanels[i]];
        V3 vel;
        if (B.tip) {
            vel = velocity2D(M, B, phi);
        } else {
            vel = velocity3D(M, B, phi);
            if (isnan3(vel)) vel = velocity2D(M, B, phi);
        }
        if (isnan3(vel)) vel = cross(cross(B.bez, Vinf), B.bez);
        vel.x /= PG;
        double cp = (1 - std::pow(norm(vel) / p->V, 2));  // bodyPanel::computeCp, :591-594
        if (vel_out) {
            vel_out[3 * i] = vel.x; vel_out[3 * i + 1] = vel.y; vel_out[3 * i + 2] = vel.z;
        }
        if (cp_out) cp_out[i] = cp;
        V3 f = ((-cp * B.area) * B.bez) / p->Sref;
        F = F + f;
        V3 r = B.center - cg;
        V3 Fm = ((-cp) * B.bez) * B.area;  // bodyPanel::computeMoments, :610-615
        V3 mom = cross(r, Fm);
        CM.x += mom.x / (p->Sref * p->bref);
        CM.y += mom.y / (p->Sref * p->cref);
        CM.z += mom.z / (p->Sref * p->bref);
    }
    res->Fbody[0] = F.x; res->Fbody[1] = F.y; res->Fbody[2] = F.z;
    for (int r = 0; r < 3; r++) res->Fwind[r] = T[0][r] * F.x + T[1][r] * F.y + T[2][r] * F.z;
    res->CM[0] = CM.x; res->CM[1] = CM.y; res->CM[2] = CM.z;
}

}  // namespace

extern "C" {

int cpo_spanwise(void* mp, int wake, double* y2b, double* cl, double* cdi) {
    const Mesh& M = *(const Mesh*)mp;
    if (wake < 0 || (size_t)wake >= M.span.size() || M.span[wake].empty()) return -1;
    const std::vector<double>& sp = M.span[wake];
    const size_t m = sp.size() / 3;
    for (size_t i = 0; i < m; i++) {
        y2b[i] = sp[i];
        cl[i] = sp[m + i];
        cdi[i] = sp[2 * m + i];
    }
    return (int)m;
}

int cpo_case_post(void* mp, const cpo_case_params* p, const double* mu_in, double* phi_out, double* vel_out,
                  double* cp_out, cpo_case_result* res) {
    Mesh& M = *(Mesh*)mp;
    int64_t n = (int64_t)M.bPanels.size();
    V3 Vinf;
    double T[3][3];
    windToBody(p->V, p->alpha, p->beta, Vinf, T);
    double PG = std::sqrt(1 - std::pow(p->mach, 2));
    std::vector<double> mu(mu_in, mu_in + n), phi(n);
    // setMu / setPotential, cpCase.cpp:203-212; panel.cpp:106-111
    for (int64_t i = 0; i < n; i++) phi[i] = dot(Vinf, M.body[M.bPanels[i]].center) - mu[i];
    std::vector<double> wmu(M.wPanels.size());
    for (size_t j = 0; j < M.wPanels.size(); j++) {  // wakePanel::setMu, wakePanel.cpp:94-100
        int idx[4];
        double c;
        interpPanels(M, M.wPanels[j], idx, c);
        wmu[j] = (1 - c) * mu[idx[0]] + (c - 1) * mu[idx[1]] + c * mu[idx[2]] - c * mu[idx[3]];
    }
    // compVelocity, cpCase.cpp:342-365
    surfacePost(M, phi, Vinf, T, p, PG, vel_out, cp_out, res);
    if (phi_out)
        for (int64_t i = 0; i < n; i++) phi_out[i] = phi[i];
    // trefftzPlaneAnalysis, cpCase.cpp:541-552
    WakeEval pot{M, wmu};
    double CL = 0, CD = 0;
    M.span.assign(M.wakes.size(), {});
    for (size_t w = 0; w < M.wakes.size(); w++) {
        double cl, cd;
        std::vector<double> y, Cl, Cd;
        trefftzPlane(M, M.wakes[w], pot, mu, p->V, p->Sref, cl, cd, y, Cl, Cd);
        CL += cl / PG;
        CD += cd / std::pow(PG, 2);
        // cpCase::writeSpanwiseData, CPanel/cpCase.cpp:915-917
        std::vector<double>& sp = M.span[w];
        for (double v : y) sp.push_back(2 * v / p->bref);
        for (double v : Cl) sp.push_back(v / PG);
        for (double v : Cd) sp.push_back(v / std::pow(PG, 2));
    }
    res->CL = CL;
    res->CDi = CD;
    return 0;
}

int cpo_case_run(void* mp, const double* A, const double* B, const cpo_case_params* p, double* sigma_out,
                 double* mu_out, double* phi_out, double* vel_out, double* cp_out, double* wake_mu,
                 cpo_case_result* res, int nthreads) {
    Mesh& M = *(Mesh*)mp;
    int64_t n = (int64_t)M.bPanels.size();
    V3 Vinf;
    double T[3][3];
    windToBody(p->V, p->alpha, p->beta, Vinf, T);
    std::vector<double> sigma(n), rhs(n), mu(n);
    for (int64_t i = 0; i < n; i++) sigma[i] = (-dot(Vinf, M.body[M.bPanels[i]].normal) + 0);  // bodyPanel::setSigma
    matvec(B, n, sigma.data(), rhs.data(), nthreads);
    for (int64_t i = 0; i < n; i++) rhs[i] = -rhs[i];
    int64_t iters;
    double err;
    cpo_bicgstab(A, n, rhs.data(), mu.data(), std::numeric_limits<double>::epsilon(), 2 * n, &iters, &err, nthreads);
    res->iters = iters;
    res->error = err;
    res->converged = err <= std::pow(10.0, -10.0);
    if (sigma_out) std::memcpy(sigma_out, sigma.data(), sizeof(double) * n);
    if (mu_out) std::memcpy(mu_out, mu.data(), sizeof(double) * n);
    if (wake_mu)
        for (size_t j = 0; j < M.wPanels.size(); j++) {
            int idx[4];
            double c;
            interpPanels(M, M.wPanels[j], idx, c);
            wake_mu[j] = (1 - c) * mu[idx[0]] + (c - 1) * mu[idx[1]] + c * mu[idx[2]] - c * mu[idx[3]];
        }
    return cpo_case_post(mp, p, mu.data(), phi_out, vel_out, cp_out, res);
}

}  // extern "C"

// vortex-particle case (buffer wake, shedding, panel stretching, time loop)
#include "cpo_vpcase.inc"
