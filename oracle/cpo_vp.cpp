/*
 * cpo_vp.cpp -- CPU oracle for the vortex-particle operators (TEST INFRASTRUCTURE ONLY).
 * See cpo_vp.h for the reference functions restated here.  Compiled with
 * -ffp-contract=off; expressions keep the reference's evaluation order.
 */
#include "cpo_vp.h"
#include "cpo_pair.h"

#include <cmath>
#include <vector>

namespace {
using namespace cpo_pair;

std::vector<Part> load(const double* pos, const double* str, const double* rad, int64_t n) {
    std::vector<Part> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {ld(pos, i), ld(str, i), rad[i]};
    return P;
}

/* ---------------------------------------------------------------- octree */
struct Node {
    P3 origin, half;
    int level = 1;
    int child[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    std::vector<int> members;
    Part exp;
    bool hasExp = false;
    bool leaf() const {
        for (int c : child)
            if (c >= 0) return false;
        return true;
    }
};

struct Tree {
    std::vector<Part> P;
    std::vector<Node> nodes;  // index 0 = root
    int64_t maxMembers = 10;
    double theta = 0.5;
    std::vector<int> order;   // pre-order node list
    int levels = 0;

    int childFor(int nd, P3 p) const {  // node::getChildContainingPnt, node.h:429-446
        const Node& N = nodes[nd];
        int c = 0;
        if (p.x > N.origin.x) c |= 4;
        if (p.y > N.origin.y) c |= 2;
        if (p.z > N.origin.z) c |= 1;
        return c;
    }
    int createChild(int nd, int c) {  // node::createChild, node.h:46-62
        Node ch;
        P3 o = nodes[nd].origin, h = nodes[nd].half;
        o.x += h.x * (c & 4 ? 0.5 : -0.5);
        o.y += h.y * (c & 2 ? 0.5 : -0.5);
        o.z += h.z * (c & 1 ? 0.5 : -0.5);
        ch.origin = o;
        ch.half = {0.5 * h.x, 0.5 * h.y, 0.5 * h.z};
        ch.level = nodes[nd].level + 1;
        nodes.push_back(ch);
        int id = (int)nodes.size() - 1;
        nodes[nd].child[c] = id;
        return id;
    }
    void pushMember(int nd, int m) {  // node::pushMember, node.h:64-77
        int c = childFor(nd, P[m].pos);
        int id = nodes[nd].child[c];
        if (id < 0) id = createChild(nd, c);
        addMember(id, m);
    }
    void addMember(int nd, int m) {  // node::addMember, node.h:196-214
        if (nodes[nd].leaf()) {
            nodes[nd].members.push_back(m);
            // depth guard: more than maxMembers coincident particles would make the
            // reference split without end; here a node at kMaxLevel stays a leaf
            if ((int64_t)nodes[nd].members.size() > maxMembers && nodes[nd].level < kMaxLevel) {
                std::vector<int> ms = nodes[nd].members;
                for (int q : ms) pushMember(nd, q);
                nodes[nd].members.clear();
            }
        } else {
            pushMember(nd, m);
        }
    }
    void preorder(int nd) {  // node::getSubNodes, node.h:466-487
        order.push_back(nd);
        for (int c = 0; c < 8; c++)
            if (nodes[nd].child[c] >= 0) preorder(nodes[nd].child[c]);
    }
    void membersOf(int nd, std::vector<int>& out) const {  // node::getMembers, node.h:448-464
        if (nodes[nd].leaf()) {
            out.insert(out.end(), nodes[nd].members.begin(), nodes[nd].members.end());
        } else {
            for (int c = 0; c < 8; c++)
                if (nodes[nd].child[c] >= 0) membersOf(nodes[nd].child[c], out);
        }
    }
    void build() {  // octree::addData (fresh tree), octree.h:151-195,39-73
        P3 mn = P[0].pos, mx = P[0].pos;
        for (const Part& p : P) {
            if (p.pos.x < mn.x) mn.x = p.pos.x;
            if (p.pos.x > mx.x) mx.x = p.pos.x;
            if (p.pos.y < mn.y) mn.y = p.pos.y;
            if (p.pos.y > mx.y) mx.y = p.pos.y;
            if (p.pos.z < mn.z) mn.z = p.pos.z;
            if (p.pos.z > mx.z) mx.z = p.pos.z;
        }
        Node root;
        root.origin = scl(0.5, add(mn, mx));
        P3 ext = sub(mx, mn);
        double maxD = std::max(ext.x, std::max(ext.y, ext.z));
        root.half = {1 * (0.51 * maxD), 1 * (0.51 * maxD), 1 * (0.51 * maxD)};
        root.level = 1;
        nodes.clear();
        nodes.push_back(root);
        for (int m = 0; m < (int)P.size(); m++) addMember(0, m);
        order.clear();
        preorder(0);
        levels = 0;  // octree::numTreeLevels, octree.h:263-275
        for (int nd : order)
            if (nodes[nd].level > levels) levels++;
        computeMultExp();
    }
    void computeMultExp() {  // particleFMM::computeMultExp, particleFMM.cpp:30-62
        for (int lv = levels + 1; lv > 1; lv--)
            for (int nd : order) {
                Node& N = nodes[nd];
                if (N.level != lv) continue;
                std::vector<Part> src;
                if (N.leaf()) {
                    std::vector<int> ms;
                    membersOf(nd, ms);
                    for (int m : ms) src.push_back(P[m]);
                } else {
                    for (int c = 0; c < 8; c++)
                        if (N.child[c] >= 0) src.push_back(nodes[N.child[c]].exp);
                }
                P3 wp{0, 0, 0}, st{0, 0, 0};
                double tot = 0;
                for (const Part& q : src) {  // findExpPos / findExpStrength, particleFMM.cpp:121-175
                    wp = add(wp, scl(nrm(q.str), q.pos));
                    tot += nrm(q.str);
                }
                for (const Part& q : src) st = add(st, q.str);
                N.exp.pos = {wp.x / tot, wp.y / tot, wp.z / tot};
                N.exp.str = st;
                N.exp.rad = nrm(N.half) * 2 * 1.5;
                N.hasExp = true;
            }
    }
    bool far(int nd, P3 p) const {  // node::isFarField(POI), node.h:404-421
        double s = 2 * nodes[nd].half.x;
        double d = nrm(sub(nodes[nd].exp.pos, p));
        return s / d < theta;
    }
    // node::calcVel / calcStretch / calcDiff, node.h:236-364 (kind: 0 alg point, 1 Gauss particle,
    // 2 stretch, 3 diffusion); target particle index ti (or -1 for a point)
    P3 calc(int nd, int kind, P3 pt, int ti) const {
        const Node& N = nodes[nd];
        P3 acc{0, 0, 0};
        if (N.leaf()) {
            std::vector<int> ms;
            membersOf(nd, ms);
            for (int m : ms) {
                if (kind == 0)
                    acc = add(acc, velAlg(P[m], pt));
                else if (m != ti) {
                    if (kind == 1) acc = add(acc, velGaussPart(P[m], P[ti]));
                    if (kind == 2) acc = add(acc, stretch(P[m], P[ti]));
                    if (kind == 3) acc = add(acc, diffusion(P[m], P[ti]));
                }
            }
        } else if (far(nd, pt)) {
            if (kind == 0) acc = velAlg(N.exp, pt);
            if (kind == 1) acc = velGaussPart(N.exp, P[ti]);
            if (kind == 2) acc = stretch(N.exp, P[ti]);
            if (kind == 3) acc = diffusion(N.exp, P[ti]);
        } else {
            for (int c = 0; c < 8; c++)
                if (N.child[c] >= 0) acc = add(acc, calc(N.child[c], kind, pt, ti));
        }
        return acc;
    }
    P3 query(int kind, P3 pt, int ti) const {  // particleFMM::barnesHut*, particleFMM.cpp:65-116
        P3 acc{0, 0, 0};
        for (int c = 0; c < 8; c++)
            if (nodes[0].child[c] >= 0) acc = add(acc, calc(nodes[0].child[c], kind, pt, ti));
        return acc;
    }
};

void put(double* out, int64_t i, P3 v) {
    out[3 * i] = v.x;
    out[3 * i + 1] = v.y;
    out[3 * i + 2] = v.z;
}

}  // namespace

extern "C" {

void cpo_vp_direct_velocity(const double* pos, const double* str, const double* rad, int64_t n, const double* pts,
                            int64_t m, int mode, double* vel) {
    std::vector<Part> P = load(pos, str, rad, n);
    int64_t nt = mode == 0 ? n : m;
    for (int64_t i = 0; i < nt; i++) {
        P3 acc{0, 0, 0};
        for (int64_t j = 0; j < n; j++) {
            if (mode == 0) {
                if (j != i) acc = add(acc, velGaussPart(P[j], P[i]));
            } else if (mode == 1) {
                acc = add(acc, velGaussPoint(P[j], ld(pts, i)));
            } else {
                acc = add(acc, velAlg(P[j], ld(pts, i)));
            }
        }
        put(vel, i, acc);
    }
}

void cpo_vp_direct_stretch(const double* pos, const double* str, const double* rad, int64_t n, double* out) {
    std::vector<Part> P = load(pos, str, rad, n);
    for (int64_t i = 0; i < n; i++) {
        P3 acc{0, 0, 0};
        for (int64_t j = 0; j < n; j++)
            if (j != i) acc = add(acc, stretch(P[i], P[j]));  // particles[i]->vortexStretching(particles[j])
        put(out, i, acc);
    }
}

void cpo_vp_direct_diffusion(const double* pos, const double* str, const double* rad, int64_t n, double* out) {
    std::vector<Part> P = load(pos, str, rad, n);
    for (int64_t i = 0; i < n; i++) {
        P3 acc{0, 0, 0};
        for (int64_t j = 0; j < n; j++)
            if (j != i) acc = add(acc, diffusion(P[i], P[j]));  // particles[i]->viscousDiffusion(particles[j])
        put(out, i, acc);
    }
}

void* cpo_bh_build(const double* pos, const double* str, const double* rad, int64_t n, int64_t max_members,
                   double theta) {
    Tree* T = new Tree();
    T->P = load(pos, str, rad, n);
    T->maxMembers = max_members;
    T->theta = theta;
    T->build();
    return T;
}
void cpo_bh_free(void* t) { delete (Tree*)t; }
int64_t cpo_bh_num_nodes(void* t) { return (int64_t)((Tree*)t)->nodes.size(); }
int64_t cpo_bh_num_levels(void* t) { return ((Tree*)t)->levels; }

void cpo_bh_nodes(void* t, double* out) {
    Tree& T = *(Tree*)t;
    std::vector<int> pos(T.nodes.size());
    for (size_t q = 0; q < T.order.size(); q++) pos[T.order[q]] = (int)q;
    for (size_t q = 0; q < T.order.size(); q++) {
        const Node& N = T.nodes[T.order[q]];
        double* o = out + 24 * q;
        o[0] = N.origin.x; o[1] = N.origin.y; o[2] = N.origin.z;
        o[3] = N.half.x; o[4] = N.half.y; o[5] = N.half.z;
        o[6] = N.level; o[7] = N.leaf(); o[8] = (double)N.members.size();
        o[9] = N.exp.pos.x; o[10] = N.exp.pos.y; o[11] = N.exp.pos.z;
        o[12] = N.exp.str.x; o[13] = N.exp.str.y; o[14] = N.exp.str.z;
        o[15] = N.hasExp ? N.exp.rad : 0;
        for (int c = 0; c < 8; c++) o[16 + c] = N.child[c] >= 0 ? pos[N.child[c]] : -1;
    }
}

void cpo_bh_leaf_members(void* t, int64_t* out) {
    Tree& T = *(Tree*)t;
    int64_t k = 0;
    for (int nd : T.order)
        if (T.nodes[nd].leaf())
            for (int m : T.nodes[nd].members) out[k++] = m;
}

void cpo_bh_velocity(void* t, const double* pts, int64_t m, int mode, double* vel) {
    Tree& T = *(Tree*)t;
    int64_t nt = mode == 0 ? m : (int64_t)T.P.size();
    for (int64_t i = 0; i < nt; i++) {
        P3 p = mode == 0 ? ld(pts, i) : T.P[i].pos;
        put(vel, i, T.query(mode == 0 ? 0 : 1, p, mode == 0 ? -1 : (int)i));
    }
}

void cpo_bh_stretch(void* t, double* out) {
    Tree& T = *(Tree*)t;
    for (int64_t i = 0; i < (int64_t)T.P.size(); i++) put(out, i, T.query(2, T.P[i].pos, (int)i));
}

void cpo_bh_diffusion(void* t, double* out) {
    Tree& T = *(Tree*)t;
    for (int64_t i = 0; i < (int64_t)T.P.size(); i++) put(out, i, T.query(3, T.P[i].pos, (int)i));
}

}  // extern "C"
