// Particle octree build (host): see octree.h for the rules and their reference.
// Compiled with -ffp-contract=off: origins, expansions and widths are rounded
// exactly as the reference's expressions, so the device far-field tests
// (2 half.x / |x_exp - x| < theta) take the same branches as the reference.
#include "octree.h"

#include <cmath>

namespace cpg {
namespace {

struct Builder {
    const double *pos, *str, *rad;
    ParticleTree& T;
    std::vector<int64_t> scratch;

    int octant(const double* o, int64_t p) const {  // node::getChildContainingPnt, node.h:429-446
        int c = 0;
        if (pos[3 * p] > o[0]) c |= 4;
        if (pos[3 * p + 1] > o[1]) c |= 2;
        if (pos[3 * p + 2] > o[2]) c |= 1;
        return c;
    }

    int new_node(const double* o, const double* h, int lvl) {
        int id = (int)T.level.size();
        for (int k = 0; k < 3; k++) {
            T.origin.push_back(o[k]);
            T.half.push_back(h[k]);
        }
        T.level.push_back(lvl);
        for (int c = 0; c < 8; c++) T.child.push_back(-1);
        T.nodes.push_back(BHNode{});
        return id;
    }

    // Members idx[b, e) (increasing particle index) fall in node `id`.
    void split(int id, int64_t b, int64_t e) {
        int lvl = T.level[id];
        int64_t cnt = e - b;
        if (cnt <= T.max_members || lvl >= kBHMaxLevel) {  // node::addMember, node.h:196-214
            BHNode& nd = T.nodes[id];
            nd.leaf = 1;
            nd.first = (int32_t)b;
            nd.count = (int32_t)cnt;
            nd.skip = id + 1;
            return;
        }
        double o[3] = {T.origin[3 * id], T.origin[3 * id + 1], T.origin[3 * id + 2]};
        double h[3] = {T.half[3 * id], T.half[3 * id + 1], T.half[3 * id + 2]};
        // stable partition by octant (counting sort keeps index order inside octants)
        int64_t counts[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int64_t q = b; q < e; q++) counts[octant(o, T.perm[q])]++;
        int64_t start[9];
        start[0] = b;
        for (int c = 0; c < 8; c++) start[c + 1] = start[c] + counts[c];
        int64_t fill[8];
        for (int c = 0; c < 8; c++) fill[c] = start[c];
        for (int64_t q = b; q < e; q++) scratch[fill[octant(o, T.perm[q])]++] = T.perm[q];
        for (int64_t q = b; q < e; q++) T.perm[q] = scratch[q];
        for (int c = 0; c < 8; c++) {
            if (counts[c] == 0) continue;
            double co[3] = {o[0], o[1], o[2]}, ch[3];  // node::createChild, node.h:46-62
            co[0] += h[0] * (c & 4 ? 0.5 : -0.5);
            co[1] += h[1] * (c & 2 ? 0.5 : -0.5);
            co[2] += h[2] * (c & 1 ? 0.5 : -0.5);
            for (int k = 0; k < 3; k++) ch[k] = 0.5 * h[k];
            int cid = new_node(co, ch, lvl + 1);
            T.child[8 * id + c] = cid;
            split(cid, start[c], start[c + 1]);
        }
        BHNode& nd = T.nodes[id];
        nd.leaf = 0;
        nd.first = (int32_t)b;
        nd.count = 0;
        nd.skip = (int32_t)T.nodes.size();
    }
};

inline double norm3(double x, double y, double z) { return std::sqrt(x * x + y * y + z * z); }

}  // namespace

void build_particle_tree(const double* pos, const double* str, const double* rad, int64_t n, int64_t max_members,
                         double theta, ParticleTree& T) {
    T = ParticleTree();
    T.n = n;
    T.max_members = max_members;
    T.theta = theta;
    if (n <= 0) return;
    // octree::setDimensions / boundingBox, octree.h:39-73
    double mn[3] = {pos[0], pos[1], pos[2]}, mx[3] = {pos[0], pos[1], pos[2]};
    for (int64_t p = 0; p < n; p++)
        for (int k = 0; k < 3; k++) {
            double v = pos[3 * p + k];
            if (v < mn[k]) mn[k] = v;
            if (v > mx[k]) mx[k] = v;
        }
    double o[3], h[3];
    for (int k = 0; k < 3; k++) o[k] = 0.5 * (mn[k] + mx[k]);
    double ext[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    double maxD = ext[0];
    if (ext[1] > maxD) maxD = ext[1];
    if (ext[2] > maxD) maxD = ext[2];
    for (int k = 0; k < 3; k++) h[k] = 1 * (0.51 * maxD);

    T.perm.resize(n);
    for (int64_t p = 0; p < n; p++) T.perm[p] = p;
    Builder B{pos, str, rad, T, std::vector<int64_t>(n)};
    B.new_node(o, h, 1);  // root: level 1 (node constructor with parent level 0)
    B.split(0, 0, n);

    const int nn = (int)T.nodes.size();
    T.levels = 0;
    for (int i = 0; i < nn; i++)
        if (T.level[i] > T.levels) T.levels++;

    // particle records in slot order
    T.parts.resize(n);
    for (int64_t q = 0; q < n; q++) {
        int64_t p = T.perm[q];
        T.parts[q] = BHPart{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2], rad[p],
                            str[3 * p], str[3 * p + 1], str[3 * p + 2], (double)p};
    }

    // particleFMM::computeMultExp: children before parents.  In pre-order every child
    // follows its parent, so a reverse sweep visits children first; each expansion is
    // a function of its own node's members or children only, so the reverse sweep gives
    // the same values as the reference's level-by-level order.
    for (int i = nn - 1; i >= 1; i--) {
        BHNode& nd = T.nodes[i];
        double wx = 0, wy = 0, wz = 0, tot = 0, sx = 0, sy = 0, sz = 0;
        if (nd.leaf) {  // findExpPos / findExpStrength over members, particleFMM.cpp:121-164
            for (int32_t q = nd.first; q < nd.first + nd.count; q++) {
                const BHPart& P = T.parts[q];
                double a = norm3(P.ax, P.ay, P.az);
                wx = wx + P.x * a;
                wy = wy + P.y * a;
                wz = wz + P.z * a;
                tot += a;
            }
            for (int32_t q = nd.first; q < nd.first + nd.count; q++) {
                sx = sx + T.parts[q].ax;
                sy = sy + T.parts[q].ay;
                sz = sz + T.parts[q].az;
            }
        } else {  // from child expansions, particleFMM.cpp:138-175
            for (int c = 0; c < 8; c++) {
                int ci = T.child[8 * i + c];
                if (ci < 0) continue;
                const BHNode& C = T.nodes[ci];
                double a = norm3(C.ax, C.ay, C.az);
                wx = wx + C.ex * a;
                wy = wy + C.ey * a;
                wz = wz + C.ez * a;
                tot += a;
            }
            for (int c = 0; c < 8; c++) {
                int ci = T.child[8 * i + c];
                if (ci < 0) continue;
                sx = sx + T.nodes[ci].ax;
                sy = sy + T.nodes[ci].ay;
                sz = sz + T.nodes[ci].az;
            }
        }
        nd.ex = wx / tot;
        nd.ey = wy / tot;
        nd.ez = wz / tot;
        nd.ax = sx;
        nd.ay = sy;
        nd.az = sz;
        const double* hh = &T.half[3 * i];
        nd.erad = norm3(hh[0], hh[1], hh[2]) * 2 * 1.5;
        nd.width = 2 * hh[0];
    }
    T.nodes[0].width = 2 * T.half[0];
    T.fnodes.resize(T.nodes.size());
    for (size_t i = 0; i < T.nodes.size(); i++) {
        const BHNode& nd = T.nodes[i];
        BHNodeF& f = T.fnodes[i];
        f.hx = (float)nd.ex;
        f.hy = (float)nd.ey;
        f.hz = (float)nd.ez;
        f.lx = (float)(nd.ex - (double)f.hx);
        f.ly = (float)(nd.ey - (double)f.hy);
        f.lz = (float)(nd.ez - (double)f.hz);
        f.ax = (float)nd.ax;
        f.ay = (float)nd.ay;
        f.az = (float)nd.az;
        f.erad = (float)nd.erad;
        const double fr = nd.width / theta, ct = 5 * nd.erad;
        f.far2 = (float)(fr * fr);
        f.cut2 = (float)(ct * ct);
    }
}

void particle_tree_table(const ParticleTree& T, double* out) {
    const int nn = (int)T.nodes.size();
    for (int i = 0; i < nn; i++) {
        const BHNode& nd = T.nodes[i];
        double* o = out + (int64_t)kBHNodeFields * i;
        for (int k = 0; k < 3; k++) {
            o[k] = T.origin[3 * i + k];
            o[3 + k] = T.half[3 * i + k];
        }
        o[6] = T.level[i];
        o[7] = nd.leaf;
        o[8] = nd.leaf ? nd.count : 0;
        bool has = i > 0;
        o[9] = has ? nd.ex : 0;
        o[10] = has ? nd.ey : 0;
        o[11] = has ? nd.ez : 0;
        o[12] = has ? nd.ax : 0;
        o[13] = has ? nd.ay : 0;
        o[14] = has ? nd.az : 0;
        o[15] = has ? nd.erad : 0;
        for (int c = 0; c < 8; c++) o[16 + c] = T.child[8 * i + c];
    }
}

}  // namespace cpg
