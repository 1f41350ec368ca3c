// Particle octree for the Barnes-Hut operators (host build, device-ready layout).
//
// The tree is the one the reference's octree<particle> builds by inserting the
// particles in index order (octree/include/octree.h:39-195, node.h:46-214):
//   - root cube: centre of the bounding box, half-width 0.51 x the largest extent;
//   - a node holding more than max_members members splits, pushing them to the
//     octants x>o -> 4, y>o -> 2, z>o -> 1; children exist only where members fall.
// That insertion process ends in a state that depends only on the point set: a node
// is internal iff more than max_members particles fall in it, a child exists iff its
// octant is non-empty, and a leaf lists its members in increasing particle index.  The
// builder here partitions recursively to that state directly, emitting nodes in the
// reference's pre-order (node::getSubNodes, node.h:473-498).
//
// Expansions follow particleFMM::computeMultExp (CPanel/particleFMM.cpp:30-62):
// leaves from members, internal nodes from child expansions (in child order);
// position = sum |alpha| x / sum |alpha|, strength = sum alpha, radius = |half|*2*1.5.
// The root has none (the queries start at the root's children).
#pragma once
#include <cstdint>
#include <vector>

namespace cpg {

// Device node record, pre-order.  80 bytes.
struct BHNode {
    double ex, ey, ez;  // expansion position
    double ax, ay, az;  // expansion strength
    double erad;        // expansion radius |half| * 2 * 1.5
    double width;       // 2 * half.x (node::isFarField, node.h:404-421)
    int32_t first;      // leaf: first member slot in the permuted particle array
    int32_t count;      // leaf: member count; internal: 0
    int32_t skip;       // pre-order index of the first node after this subtree
    int32_t leaf;       // 1 for a leaf
};

// Particle record in leaf-member order.  64 bytes.
struct BHPart {
    double x, y, z, r;
    double ax, ay, az;
    double idx;  // original particle index (exact in a double)
};

// Single-precision view of a node's far-field data, for traversals that evaluate far
// nodes in FP32 (48 bytes): expansion centre split into a high and a low float (the
// difference to a target is then accurate to float rounding of the difference itself),
// strength and radius, and the squared distances beyond which the node is far
// ((width / theta)^2) and within which its stretching acts ((5 erad)^2).  The
// traversal compares squared distances against these with a relative margin and falls
// back to the exact FP64 test inside the margin, so every decision equals the FP64 one.
struct BHNodeF {
    float hx, hy, hz, lx;
    float ly, lz, ax, ay;
    float az, erad, far2, cut2;
};

constexpr int kBHMaxLevel = 32;  // a node at this level stays a leaf (reference: unbounded)
constexpr int kBHNodeFields = 24;

struct ParticleTree {
    int64_t n = 0;
    int64_t max_members = 10;
    double theta = 0.5;
    int levels = 0;  // octree::numTreeLevels (octree.h:252-264)
    // pre-order node data (host)
    std::vector<double> origin, half;  // 3 per node
    std::vector<int32_t> level, child;  // child: 8 per node (pre-order index or -1)
    std::vector<BHNode> nodes;
    std::vector<BHNodeF> fnodes;  // FP32 view of nodes (same order)
    std::vector<int64_t> perm;  // slot -> particle index (leaves in pre-order)
    std::vector<BHPart> parts;  // slot order
};

// pos, str: n x 3 row-major; rad: n.  max_members >= 1.
void build_particle_tree(const double* pos, const double* str, const double* rad, int64_t n, int64_t max_members,
                         double theta, ParticleTree& T);

// Node table in the layout of 24 doubles per node: origin(3) half(3) level leaf
// n_members exp_pos(3) exp_str(3) exp_radius child0..7.
void particle_tree_table(const ParticleTree& T, double* out);

}  // namespace cpg
