// Host-side mesh ingest and topology (see mesh.h).  Compiled with
// -ffp-contract=off: every geometric quantity is evaluated in the same order as
// the reference's Eigen expressions so that branch decisions (trailing-edge side,
// tip-patch flags, cluster angles) come out identically.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>

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

struct Panel {
    int nd[3], ed[3];
    d3 c, n;
    double area, longSide;
    int id, tri;
    bool wake;
    int group;  // surface or wake index
    // body
    bool upper = false, lower = false, tip = false;
    int ts = 3, index = -1;
    int nbr[3], nnb = 0;  // body neighbours across shared edges: at most one per edge
    std::vector<int> cluster;
    // wake
    int upPan = -1, loPan = -1;
    bool teWake = false;
};

struct Edge {
    int n1, n2;
    int nb = 0, nw = 0;
    int b[3], w[3];
    bool te = false;
};

struct Line {
    int up, lo;
    double y;
};

struct Wake {
    std::vector<int> pans;
    std::vector<Line> lines;
    double yMin = 0, yMax = 0, x0 = 0, xf = 0, z0 = 0, zf = 0;
    bool live = true;
};

struct Geo {
    d3 c, n;
    double area, longSide;
};

struct Builder {
    std::vector<d3> P;
    std::vector<Edge> E;
    EdgeMap emap;
    std::vector<Panel> pan;
    std::vector<bool> surfLS;
    std::vector<Wake> wakes;

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

    // panel::setGeom, CPanel/panel.cpp:33-72.  The edges' lengths are taken from the panel's own
    // node pairs: a stored edge may run the other way round, which gives the same length.
    void geom(const int nd[3], Geo& g) const {
        g.longSide = 0;
        for (int i = 0; i < 3; i++) {
            double l = nrm(sub(P[nd[i < 2 ? i + 1 : 0]], P[nd[i]]));
            if (l > g.longSide) g.longSide = l;
        }
        d3 p0 = P[nd[0]], p1 = P[nd[1]], p2 = P[nd[2]];
        d3 a = sub(p1, p0), b = sub(p2, p0);
        g.c = divs(add(add(p0, p1), p2), 3.0);
        double th = std::acos(dot(a, b) / (nrm(a) * nrm(b)));
        g.area = 0.5 * nrm(a) * nrm(b) * std::sin(th);
        g.n = unit(cross(a, b));
    }

    void addLine(int w, Line l) {  // wake::addWakeLine, CPanel/wake.cpp:140-144
        wakes[w].lines.push_back(l);
        std::sort(wakes[w].lines.begin(), wakes[w].lines.end(), [](const Line& a, const Line& b) { return a.y < b.y; });
    }

    void parents(int wi, int up, int lo) {  // wakePanel::setParentPanels, CPanel/wakePanel.cpp:120-152
        Panel& W = pan[wi];
        pan[up].upper = true;
        pan[lo].lower = true;
        W.teWake = true;
        if (W.upPan < 0 || pan[up].c.x < W.c.x) {
            W.upPan = up;
            W.loPan = lo;
        }
        // wakeLine::setDimensions (CPanel/wakeLine.cpp:31-46): last TE edge of the upper panel
        int te = -1;
        for (int k = 0; k < 3; k++)
            if (E[pan[W.upPan].ed[k]].te) te = pan[W.upPan].ed[k];
        d3 mid = divs(add(P[E[te].n1], P[E[te].n2]), 2.0);
        addLine(W.group, Line{W.upPan, W.loPan, mid.y});
    }

    void checkTE(int ei) {  // edge::checkTE, CPanel/edge.cpp:48-109
        Edge& e = E[ei];
        if (e.nb != 2) return;
        if (e.nw == 1) {
            e.te = true;
            const Panel& W = pan[e.w[0]];
            d3 v1 = sub(pan[e.b[0]].c, W.c), v2 = sub(pan[e.b[1]].c, W.c);
            double t1 = std::acos(dot(v1, W.n) / (nrm(v1) * nrm(W.n)));
            double t2 = std::acos(dot(v2, W.n) / (nrm(v2) * nrm(W.n)));
            if (t1 < t2)
                parents(e.w[0], e.b[0], e.b[1]);
            else
                parents(e.w[0], e.b[1], e.b[0]);
        } else {
            const Panel& b0 = pan[e.b[0]];
            const Panel& b1 = pan[e.b[1]];
            // acos(d) > 4.7 pi / 6 needs d < cos(4.7 pi / 6) = -0.778: acos is evaluated only
            // below -0.7, so the outcome is the reference's test for every d
            double d = dot(b0.n, b1.n);
            if (b0.id == b1.id && d < -0.7 && std::acos(d) > 4.7 * kPi / 6) {
                e.te = true;
                surfLS[b0.group] = true;
                surfLS[b1.group] = true;
            }
        }
    }
};

int fact(int i) {
    int o = 1;
    for (int k = 2; k <= i; k++) o *= k;
    return o;
}

// Host threads for par_slices, started on first use and kept for the life of the process (they
// wait on a condition variable between calls; starting and joining 15 threads per call had cost
// up to a millisecond).  A call queues its slices and runs slices itself as well, so it finishes
// when every pool thread is busy with other calls (meshes built on several threads at once) or
// when the pool has no threads at all (a forked child).
class SlicePool {
  public:
    struct Job {
        std::function<void(unsigned, size_t, size_t)> f;
        size_t n = 0;
        unsigned nth = 1;
        std::atomic<unsigned> next{0}, left{0};
        std::mutex m;
        std::condition_variable cv;
        void work() {
            for (unsigned w; (w = next.fetch_add(1)) < nth;) {
                f(w, n * w / nth, n * (w + 1) / nth);
                if (left.fetch_sub(1) == 1) {
                    std::lock_guard<std::mutex> l(m);
                    cv.notify_all();
                }
            }
        }
    };
    static SlicePool& get() {
        static SlicePool* pool = new SlicePool();  // never destroyed: its threads outlive main
        return *pool;
    }
    void run(const std::shared_ptr<Job>& j) {
        {
            std::lock_guard<std::mutex> l(m_);
            q_.push_back(j);
        }
        cv_.notify_all();
        j->work();
        {
            std::unique_lock<std::mutex> l(j->m);
            j->cv.wait(l, [&] { return j->left.load() == 0; });
        }
        std::lock_guard<std::mutex> l(m_);
        auto it = std::find(q_.begin(), q_.end(), j);
        if (it != q_.end()) q_.erase(it);
    }

  private:
    SlicePool() {
        const unsigned k = std::max(1u, std::min(16u, std::thread::hardware_concurrency())) - 1;
        for (unsigned i = 0; i < k; i++) {
            try {
                std::thread([this] { loop(); }).detach();
            } catch (...) {
                break;
            }
        }
    }
    void loop() {
        for (;;) {
            std::shared_ptr<Job> j;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return !q_.empty(); });
                j = q_.front();
                if (j->next.load() >= j->nth) {  // every slice taken: the job leaves the queue
                    q_.pop_front();
                    continue;
                }
            }
            j->work();
        }
    }
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<std::shared_ptr<Job>> q_;
};

// Runs f(slice, lo, hi) over [0, n) in contiguous slices (at most 16, each on one thread at a
// time, so per-slice scratch indexed by the slice needs no lock); a small range runs on the
// calling thread.
template <class F>
void par_slices(size_t n, F f) {
    const unsigned nth = n < 2048 ? 1u : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (nth == 1) {
        f(0u, (size_t)0, n);
        return;
    }
    auto j = std::make_shared<SlicePool::Job>();
    j->f = [&f](unsigned w, size_t lo, size_t hi) { f(w, lo, hi); };
    j->n = n;
    j->nth = nth;
    j->left = nth;
    SlicePool::get().run(j);
}

}  // namespace

void host_parallel(size_t n, const std::function<void(unsigned, size_t, size_t)>& f) { par_slices(n, f); }

// chtlsnd::chtlsnd for N = 1, no derivative observations (used by wake::Vradial,
// CPanel/wake.cpp:587-594).  Monomials x, x^2/2, x^3/6 (orders 1..order).
void chtls_1d(const double* dx, int nf, int order, double* F) {
    double rmax = 0;
    for (int i = 0; i < nf; i++) {
        double r = std::sqrt(dx[i] * dx[i]);
        if (r > rmax) rmax = r;
    }
    const int t = order;
    std::vector<double> d(nf), W(nf), A(nf * t), M(t * t), R(t * nf);
    for (int i = 0; i < nf; i++) d[i] = dx[i] / rmax;
    for (int i = 0; i < nf; i++) W[i] = 1 / std::sqrt(d[i] * d[i]);
    for (int k = 0; k < t; k++) {
        double f = 1.0 / fact(k + 1);
        for (int i = 0; i < nf; i++) {
            double pw = d[i];  // (k+1)-th power as a left-to-right product
            for (int q = 1; q <= k; q++) pw = pw * d[i];
            A[i * t + k] = f * pw;
        }
    }
    for (int r = 0; r < t; r++)
        for (int c = 0; c < t; c++) {
            double s = 0;
            for (int i = 0; i < nf; i++) s += A[i * t + r] * W[i] * A[i * t + c];
            M[r * t + c] = s;
        }
    for (int r = 0; r < t; r++)
        for (int i = 0; i < nf; i++) R[r * nf + i] = A[i * t + r] * W[i];
    // Householder QR (no pivoting) and solve, as Eigen::HouseholderQR::solve
    std::vector<double> tau(t);
    for (int k = 0; k < t; k++) {
        double c0 = M[k * t + k], tail = 0;
        for (int i = k + 1; i < t; i++) tail += M[i * t + k] * M[i * t + k];
        double beta;
        if (tail <= std::numeric_limits<double>::min()) {
            tau[k] = 0;
            beta = c0;
            for (int i = k + 1; i < t; i++) M[i * t + k] = 0;
        } else {
            beta = std::sqrt(c0 * c0 + tail);
            if (c0 >= 0) beta = -beta;
            for (int i = k + 1; i < t; i++) M[i * t + k] /= (c0 - beta);
            tau[k] = (beta - c0) / beta;
        }
        M[k * t + k] = beta;
        if (tau[k] != 0)
            for (int j = k + 1; j < t; j++) {
                double tmp = M[k * t + j];
                for (int i = k + 1; i < t; i++) tmp += M[i * t + k] * M[i * t + j];
                M[k * t + j] -= tau[k] * tmp;
                for (int i = k + 1; i < t; i++) M[i * t + j] -= tau[k] * M[i * t + k] * tmp;
            }
    }
    for (int k = 0; k < t; k++) {
        if (tau[k] == 0) continue;
        for (int c = 0; c < nf; c++) {
            double tmp = R[k * nf + c];
            for (int i = k + 1; i < t; i++) tmp += M[i * t + k] * R[i * nf + c];
            R[k * nf + c] -= tau[k] * tmp;
            for (int i = k + 1; i < t; i++) R[i * nf + c] -= tau[k] * M[i * t + k] * tmp;
        }
    }
    for (int c = 0; c < nf; c++)
        for (int i = t - 1; i >= 0; i--) {
            double s = R[i * nf + c];
            for (int j = i + 1; j < t; j++) s -= M[i * t + j] * R[j * nf + c];
            R[i * nf + c] = s / M[i * t + i];
        }
    for (int i = 0; i < nf; i++) F[i] = R[i] / rmax;  // first-order row, / rmax^1
}

std::string build_mesh(const double* nodes, int64_t nn, const int64_t* tris, const int32_t* ids, int64_t nt,
                       HostMesh& out, const int32_t* te_upper, const int32_t* te_lower, int64_t n_te) {
    if (nn <= 0 || nt <= 0) return "empty mesh";
    Builder B;
    B.P.resize(nn);
    for (int64_t i = 0; i < nn; i++) B.P[i] = {nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]};
    std::vector<int64_t> conn(3 * nt);
    for (int64_t i = 0; i < 3 * nt; i++) {
        conn[i] = tris[i] - 1;
        if (conn[i] < 0 || conn[i] >= nn) return "triangle references a node outside 1..n_nodes";
    }
    // wake connectivity correction, CPanel/geometry.cpp:218-244,631-667
    int64_t wns = nn, wts = nt;
    bool anyWake = false;
    for (int64_t i = 0; i < nt; i++) {
        if (ids[i] > 1000) anyWake = true;
        if (i > 0 && ids[i] > 1000 && ids[i - 1] < 1000) {
            wns = std::min(conn[3 * i], std::min(conn[3 * i + 1], conn[3 * i + 2]));
            wts = i;
        }
    }
    if (anyWake) {
        double tol = 100000;
        for (int64_t i = 0; i < nt; i++)
            for (int j = 0; j < 3; j++) {
                double l = nrm(sub(B.P[conn[3 * i + (j < 2 ? j + 1 : 0)]], B.P[conn[3 * i + j]]));
                if (l < tol) tol = l;
            }
        // a wake node farther than tol from the body nodes' bounding box in some axis matches
        // none of them (rounded subtraction is monotone), so its scan is skipped
        d3 lo = B.P[0], hi = B.P[0];
        for (int64_t i = 0; i < wns; i++) {
            const d3& q = B.P[i];
            lo = {std::min(lo.x, q.x), std::min(lo.y, q.y), std::min(lo.z, q.z)};
            hi = {std::max(hi.x, q.x), std::max(hi.y, q.y), std::max(hi.z, q.z)};
        }
        std::vector<int64_t> rep(nn, -1);
        for (int64_t j = wns; j < nn; j++) {
            const d3& q = B.P[j];
            if (q.x - hi.x >= tol || lo.x - q.x >= tol || q.y - hi.y >= tol || lo.y - q.y >= tol ||
                q.z - hi.z >= tol || lo.z - q.z >= tol)
                continue;
            for (int64_t i = 0; i < wns; i++) {
                d3 v = sub(B.P[i], B.P[j]);
                if (std::max(std::fabs(v.x), std::max(std::fabs(v.y), std::fabs(v.z))) < tol) {
                    rep[j] = i;
                    break;
                }
            }
        }
        for (int64_t i = wts; i < nt; i++)
            for (int j = 0; j < 3; j++)
                if (rep[conn[3 * i + j]] >= 0) conn[3 * i + j] = rep[conn[3 * i + j]];
    }
    // panel geometry of every triangle, in parallel: it needs only the node positions
    std::vector<Geo> geo(nt);
    par_slices((size_t)nt, [&](unsigned, size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; i++) {
            int nd[3] = {(int)conn[3 * i], (int)conn[3 * i + 1], (int)conn[3 * i + 2]};
            B.geom(nd, geo[i]);
        }
    });
    // createSurfaces, CPanel/geometry.cpp:712-747
    std::vector<std::vector<int>> surfPans;
    B.pan.reserve(nt);
    B.E.reserve(2 * nt + 16);
    B.emap.reserve(2 * nt + 16);
    for (int64_t i = 0; i < nt; i++) {
        Panel p;
        for (int k = 0; k < 3; k++) p.nd[k] = (int)conn[3 * i + k];
        if (p.nd[0] == p.nd[1] || p.nd[1] == p.nd[2] || p.nd[0] == p.nd[2]) return "degenerate triangle";
        for (int k = 0; k < 3; k++) p.ed[k] = B.edge(p.nd[k], p.nd[k < 2 ? k + 1 : 0]);
        p.id = ids[i];
        p.tri = (int)i;
        p.wake = ids[i] > 1000;
        bool fresh = (i == 0 || ids[i] != ids[i - 1]);
        if (!p.wake) {
            if (fresh) {
                surfPans.emplace_back();
                B.surfLS.push_back(false);
            }
            p.group = (int)surfPans.size() - 1;
        } else {
            if (fresh) B.wakes.emplace_back();
            p.group = (int)B.wakes.size() - 1;
        }
        p.c = geo[i].c;
        p.n = geo[i].n;
        p.area = geo[i].area;
        p.longSide = geo[i].longSide;
        B.pan.push_back(p);
        int pi = (int)B.pan.size() - 1;
        for (int k = 0; k < 3; k++) {
            Edge& e = B.E[p.ed[k]];
            if (!p.wake) {
                if (e.nb < 3) e.b[e.nb] = pi;
                e.nb++;
            } else {
                if (e.nw < 3) e.w[e.nw] = pi;
                e.nw++;
            }
            B.checkTE(p.ed[k]);
        }
        if (!p.wake) {
            surfPans[p.group].push_back(pi);
        } else {  // wake::addPanel, CPanel/wake.cpp:42-88
            Wake& W = B.wakes[p.group];
            if (W.pans.empty()) {
                d3 q = B.P[p.nd[0]];
                W.yMax = W.yMin = q.y;
                W.x0 = W.xf = q.x;
                W.z0 = W.zf = q.z;
            }
            for (int k = 0; k < 3; k++) {
                d3 q = B.P[p.nd[k]];
                if (q.y > W.yMax) W.yMax = q.y;
                else if (q.y < W.yMin) W.yMin = q.y;
                if (q.x > W.xf) W.xf = q.x;
                else if (q.x < W.x0) W.x0 = q.x;
                if (q.z > W.zf) W.zf = q.z;
                else if (q.z < W.z0) W.z0 = q.z;
            }
            W.pans.push_back(pi);
        }
    }
    for (const Edge& e : B.E)  // edge::setNeighbors
        if (e.nb == 2) {
            Panel &a = B.pan[e.b[0]], &b = B.pan[e.b[1]];
            if (a.nnb < 3) a.nbr[a.nnb++] = e.b[1];
            if (b.nnb < 3) b.nbr[b.nnb++] = e.b[0];
        }
    // wake merge, CPanel/geometry.cpp:426-447
    std::vector<int> order;
    if (B.wakes.size() > 1) {
        bool merged = false;
        for (size_t i = 0; i < B.wakes.size(); i++)
            for (size_t j = i + 1; j < B.wakes.size(); j++) {
                Wake &a = B.wakes[i], &b = B.wakes[j];
                if (!a.live || !b.live) continue;
                double eps = std::pow(10.0, -2.0);
                if (std::fabs(b.x0 - a.x0) < eps && std::fabs(b.z0 - a.z0) < eps && std::fabs(b.xf - a.xf) < eps &&
                    std::fabs(b.zf - a.zf) < eps) {
                    for (int w : b.pans) {
                        a.pans.push_back(w);
                        B.pan[w].group = (int)i;
                    }
                    for (const Line& l : b.lines) B.addLine((int)i, l);
                    if (b.yMin < a.yMin) a.yMin = b.yMin;
                    if (b.yMax > a.yMax) a.yMax = b.yMax;
                    b.live = false;
                    order.push_back((int)i);
                    merged = true;
                }
            }
        if (!merged) {
            order.clear();
            for (size_t i = 0; i < B.wakes.size(); i++) order.push_back((int)i);
        }
    } else {
        for (size_t i = 0; i < B.wakes.size(); i++) order.push_back((int)i);
    }
    // bPanels: surfaces in reverse file order; wPanels: wakes in order
    std::vector<int> bp, wp;
    for (size_t s = surfPans.size(); s-- > 0;) bp.insert(bp.end(), surfPans[s].begin(), surfPans[s].end());
    for (int w : order)
        for (int p : B.wakes[w].pans) wp.push_back(p);
    for (size_t i = 0; i < bp.size(); i++) B.pan[bp[i]].index = (int)i;
    // trailing-edge parents given by the caller (matrix indices): a wake built outside the
    // .tri file, such as the vortex-particle buffer wake, flags them as
    // wakePanel::setParentPanels does (CPanel/wakePanel.cpp:120-152) before the clusters
    for (int64_t q = 0; q < n_te; q++) {
        if (te_upper[q] < 0 || te_upper[q] >= (int64_t)bp.size() || te_lower[q] < 0 ||
            te_lower[q] >= (int64_t)bp.size())
            return "trailing-edge parent outside the body panels";
        B.pan[bp[te_upper[q]]].upper = true;
        B.pan[bp[te_lower[q]]].lower = true;
    }
    for (int w : order)
        if (B.wakes[w].lines.size() < 2) return "a wake has fewer than two trailing-edge wake lines";

    // bodyPanel::setTipFlag, CPanel/bodyPanel.cpp:58-95
    const double tipTol = std::pow(10.0, -8.0);
    for (int b : bp) {
        Panel& p = B.pan[b];
        if (!B.surfLS[p.group]) continue;
        int count = 0;
        for (int t = 0; t < p.nnb; t++) {
            d3 nn2 = B.pan[p.nbr[t]].n;
            double d = dot(p.n, nn2) / (nrm(p.n) * nrm(nn2));
            d = d > 1 ? 1 : (d < -1 ? -1 : d);
            // acos(d) < 1e-8 needs d > 1 - 1e-12 (below it acos(d) > 1.4e-6), so acos is
            // evaluated only there
            if (d > 1 - 1e-12 && std::acos(d) < tipTol && std::asin(nn2.x) > -kPi / 12) count++;
        }
        p.tip = count >= 2;
    }
    // bodyPanel::setCluster / clusterTest, CPanel/bodyPanel.cpp:402-487,617-640.  Each panel's
    // cluster depends only on the (fixed) panel data, so the panels are split over host
    // threads; the first failing panel in matrix order is reported, as a sequential loop would.
    // Membership of the growing cluster and of the candidate list is kept in two per-thread
    // stamp arrays over all panels (inC stamped with self + 1, inA with a per-pass counter) in
    // place of linear searches; the order in which panels join is unchanged.
    struct Marks {
        std::vector<uint32_t> inC, inA;
        uint32_t pass = 0;
    };
    auto cluster_of = [&](int self, Marks& mk) -> int {  // 0 ok, 1 no neighbourhood, 2 too large
        Panel& p = B.pan[self];
        int dim = p.tip ? 2 : 3;
        size_t buffer = 10;
        size_t nObs = (size_t)(fact(p.ts + dim) / (fact(dim) * fact(p.ts)) - 1) + buffer;
        size_t nP = (nObs + 1) / 2;
        size_t old = 0;
        const uint32_t me = (uint32_t)self + 1;
        p.cluster.reserve(nP + 1);
        p.cluster.push_back(self);
        mk.inC[self] = me;
        bool upF = p.upper, loF = p.lower;
        std::vector<int> add;
        while (p.cluster.size() < nP) {
            add.clear();
            const uint32_t pass = ++mk.pass;
            for (size_t i = old; i < p.cluster.size(); i++) {
                const Panel& c = B.pan[p.cluster[i]];
                for (int t = 0; t < c.nnb; t++) {
                    int q = c.nbr[t];
                    const Panel& o = B.pan[q];
                    bool ok = !((upF && o.lower) || (loF && o.upper)) && p.tip == o.tip;
                    if (ok) {
                        double d = dot(o.n, p.n);
                        d = d > 1 ? 1 : (d < -1 ? -1 : d);
                        // acos(d) < 5 pi / 6 holds for d > -0.8 and fails for d < -0.9; acos is
                        // evaluated only between, so the outcome is the reference's test
                        bool turn = d > -0.8 ? true : (d < -0.9 ? false : std::acos(d) < 5 * kPi / 6);
                        ok = turn && mk.inC[q] != me && q != self;
                    }
                    if (ok) {
                        if (o.upper) upF = true;
                        else if (o.lower) loF = true;
                        if (mk.inA[q] != pass) {
                            mk.inA[q] = pass;
                            add.push_back(q);
                        }
                    }
                }
            }
            if (add.empty() && p.cluster.size() < nP) {
                while (p.cluster.size() < nP + 1 && p.ts >= 1) {
                    if (buffer > 0) buffer -= 1;
                    else p.ts -= 1;
                    nObs = (size_t)(fact(p.ts + dim) / (fact(dim) * fact(p.ts))) + buffer;
                    nP = (nObs + 1) / 2;
                }
                if (p.cluster.size() > nP + 1) p.cluster.resize(nP + 1);
                break;
            }
            old = p.cluster.size();
            for (int q : add) {
                p.cluster.push_back(q);
                mk.inC[q] = me;
                if (p.cluster.size() == nP + 1) break;
            }
        }
        if (p.ts < 1 || p.cluster.size() < 2) return 1;
        if (p.cluster.size() > 32) return 2;
        return 0;
    };
    {
        const size_t np = bp.size();
        std::vector<int> status(np, 0);
        par_slices(np, [&](unsigned, size_t lo, size_t hi) {
            Marks mk;
            mk.inC.assign(B.pan.size(), 0);
            mk.inA.assign(B.pan.size(), 0);
            for (size_t i = lo; i < hi; i++) status[i] = cluster_of(bp[i], mk);
        });
        for (size_t i = 0; i < np; i++) {
            if (status[i] == 1) return "a body panel has no usable CHTLS neighbourhood";
            if (status[i] == 2) return "CHTLS cluster larger than 32 panels";
        }
    }

    // ---- flatten ----
    HostMesh& H = out;
    H.n_nodes = nn;
    H.n_body = (int64_t)bp.size();
    H.n_wake = (int64_t)wp.size();
    H.body.assign(H.n_body * PF_STRIDE, 0.0);
    H.bez.assign(H.n_body * 3, 0.0);
    H.tip.resize(H.n_body);
    H.upper.resize(H.n_body);
    H.lower.resize(H.n_body);
    H.tsorder.resize(H.n_body);
    H.surf_id.resize(H.n_body);
    H.file_tri.resize(H.n_body);
    H.cl_ptr.assign(H.n_body + 1, 0);
    for (int64_t i = 0; i < H.n_body; i++)
        H.cl_ptr[i + 1] = H.cl_ptr[i] + (int32_t)B.pan[bp[i]].cluster.size();
    H.cl_idx.assign(H.cl_ptr[H.n_body], 0);
    H.n_tip = 0;
    auto pack = [&](const Panel& p, double* o) {
        for (int k = 0; k < 3; k++) {
            d3 v = B.P[p.nd[k]];
            o[3 * k] = v.x;
            o[3 * k + 1] = v.y;
            o[3 * k + 2] = v.z;
        }
        d3 l = unit(sub(B.P[p.nd[0]], p.c));  // panel::getLocalSys, CPanel/panel.cpp:156-168
        d3 m = cross(p.n, l);
        const d3 f[4] = {p.c, p.n, l, m};
        for (int q = 0; q < 4; q++) {
            o[PF_C + 3 * q] = f[q].x;
            o[PF_C + 3 * q + 1] = f[q].y;
            o[PF_C + 3 * q + 2] = f[q].z;
        }
        o[PF_AREA] = p.area;
        o[PF_LONG] = p.longSide;
    };
    par_slices((size_t)H.n_body, [&](unsigned, size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; i++) {
            const Panel& p = B.pan[bp[i]];
            pack(p, &H.body[i * PF_STRIDE]);
            H.bez[3 * i] = p.n.x;
            H.bez[3 * i + 1] = p.n.y;
            H.bez[3 * i + 2] = p.n.z;
            H.tip[i] = p.tip;
            H.upper[i] = p.upper;
            H.lower[i] = p.lower;
            H.tsorder[i] = p.ts;
            H.surf_id[i] = p.id;
            H.file_tri[i] = p.tri;
            int32_t o = H.cl_ptr[i];
            for (int q : p.cluster) H.cl_idx[o++] = B.pan[q].index;
        }
    });
    for (int64_t i = 0; i < H.n_body; i++) H.n_tip += H.tip[i];
    H.wake.assign(H.n_wake * PF_STRIDE, 0.0);
    H.widx.resize(H.n_wake * 4);
    H.wcoef.resize(H.n_wake);
    // wakePanel::interpPanels, CPanel/wakePanel.cpp:48-81
    auto bracket = [](const std::vector<Line>& L, double y, const Line*& a, const Line*& b) {
        if (y < L[1].y) {
            a = &L[0];
            b = &L[1];
        } else if (y >= L.back().y) {
            a = &L[L.size() - 2];
            b = &L[L.size() - 1];
        } else {
            a = b = nullptr;
            for (size_t i = 1; i + 1 < L.size(); i++)
                if (L[i].y <= y && L[i + 1].y > y) {
                    a = &L[i];
                    b = &L[i + 1];
                }
        }
    };
    H.wake_file_tri.resize(H.n_wake);
    for (int64_t j = 0; j < H.n_wake; j++) {
        const Panel& w = B.pan[wp[j]];
        pack(w, &H.wake[j * PF_STRIDE]);
        H.wake_file_tri[j] = w.tri;
        const Line *a, *b;
        bracket(B.wakes[w.group].lines, w.c.y, a, b);
        if (!a) return "wake panel outside its wake lines";
        H.wcoef[j] = (w.c.y - a->y) / (b->y - a->y);
        H.widx[4 * j] = B.pan[a->up].index;
        H.widx[4 * j + 1] = B.pan[a->lo].index;
        H.widx[4 * j + 2] = B.pan[b->up].index;
        H.widx[4 * j + 3] = B.pan[b->lo].index;
    }
    H.n_lines = 0;
    // Trefftz plane geometry, CPanel/wake.cpp:146-188,508-640
    H.trefftz.clear();
    H.tz_pts.clear();
    for (int wi : order) {
        const Wake& W = B.wakes[wi];
        H.n_lines += (int64_t)W.lines.size();
        TrefftzWake T;
        const int nP2 = 164;
        T.step = (W.yMax - W.yMin) / nP2;
        T.y0 = W.yMin;
        T.y1 = W.yMax;
        double xT = W.x0 + 2 * (W.xf - W.x0) / 3;
        for (int i = 1; i < nP2; i++) {
            TrefftzStation S;
            S.y = W.yMin + i * T.step;
            // wake::pntInWake
            d3 pw{0, 0, 0};
            bool found = false;
            for (int q : W.pans) {
                const Panel& w = B.pan[q];
                if (!w.teWake || found) continue;
                const Panel& U = B.pan[w.upPan];
                for (int k = 0; k < 3 && !found; k++) {
                    const Edge& e = B.E[U.ed[k]];
                    if (!e.te) continue;
                    d3 p1 = B.P[e.n1], p2 = B.P[e.n2];
                    if ((p1.y <= S.y && p2.y >= S.y) || (p1.y >= S.y && p2.y <= S.y)) {
                        double t = (S.y - p1.y) / (p2.y - p1.y);
                        d3 pnt = add(p1, mul(t, sub(p2, p1)));
                        d3 c = cross(w.n, d3{0, 1, 0});
                        d3 o{-c.x, -c.y, -c.z};
                        if (o.x < 0) o = mul(-1.0, o);
                        double sc = (xT - pnt.x) / o.x;
                        pw = add(pnt, mul(sc, o));
                        found = true;
                    }
                }
            }
            // wake::Vradial sample points
            double r, th = kPi / 4, dZmax = 0.3, delZ;
            d3 POI;
            POI.x = pw.x;
            r = pw.y >= 0 ? W.yMax - pw.y : pw.y - W.yMin;
            delZ = r * std::sin(th);
            if (delZ > dZmax) {
                delZ = dZmax;
                th = std::asin(dZmax / r);
            }
            POI.y = pw.y >= 0 ? W.yMax - r * std::cos(th) : W.yMin + r * std::cos(th);
            POI.z = pw.z + r * std::sin(th);
            double dz = 0.5 * delZ, stp = 2 * dz / (6 - 1);
            double dY[6], dZ[6];
            S.pt0 = (int32_t)(H.tz_pts.size() / 3);
            H.tz_pts.push_back(POI.x);
            H.tz_pts.push_back(POI.y);
            H.tz_pts.push_back(POI.z);
            d3 ys[6], zs[6];
            for (int q = 0; q < 6; q++) {
                double delta = -dz + q * stp;
                ys[q] = add(POI, mul(delta, d3{0, 1, 0}));
                zs[q] = add(POI, mul(delta, d3{0, 0, 1}));
                dY[q] = ys[q].y - POI.y;
                dZ[q] = zs[q].z - POI.z;
            }
            for (int q = 0; q < 6; q++) {
                H.tz_pts.push_back(ys[q].x);
                H.tz_pts.push_back(ys[q].y);
                H.tz_pts.push_back(ys[q].z);
            }
            for (int q = 0; q < 6; q++) {
                H.tz_pts.push_back(zs[q].x);
                H.tz_pts.push_back(zs[q].y);
                H.tz_pts.push_back(zs[q].z);
            }
            chtls_1d(dY, 6, 3, S.Fy);
            chtls_1d(dZ, 6, 3, S.Fz);
            // wake::wakeStrength bracketing
            const Line *a, *b;
            bracket(W.lines, S.y, a, b);
            if (!a) return "Trefftz station outside the wake lines";
            S.interp = (S.y - a->y) / (b->y - a->y);
            S.line_up1 = B.pan[a->up].index;
            S.line_lo1 = B.pan[a->lo].index;
            S.line_up2 = B.pan[b->up].index;
            S.line_lo2 = B.pan[b->lo].index;
            T.st.push_back(S);
        }
        H.trefftz.push_back(std::move(T));
    }
    return "";
}

}  // namespace cpg
