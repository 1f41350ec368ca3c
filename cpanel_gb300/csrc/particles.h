// Launchers for the vortex-particle kernels (particles.cu) and the panel-velocity
// kernel (assemble.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "octree.h"

namespace cpg {

struct VPConst {
    double four_pi, inv_four_pi, sqrt2, two_pi_15, c15, four_pi_3, nu;
};
VPConst vp_constants();

cudaError_t launch_pack_parts(const double* pos, const double* str, const double* rad, int64_t n, BHPart* out,
                              cudaStream_t s);
// Barnes-Hut traversals.  fnodes (the tree's BHNodeF view on the device) selects far
// nodes in FP32 with the near field in FP64; null: everything in FP64.
// any of vel/str/dif may be null; outputs indexed by original particle index
cudaError_t launch_bh_particles(const BHNode* nodes, const BHNodeF* fnodes, int nn, const BHPart* parts, int64_t n,
                                double theta, const VPConst& c, double* vel, double* str, double* dif,
                                cudaStream_t s);
// traversal for explicit targets (original order; outputs by target position); vel / str+dif / all
cudaError_t launch_bh_targets(const BHNode* nodes, const BHNodeF* fnodes, int nn, const BHPart* slots, double theta,
                              const BHPart* tgt, int64_t m, const VPConst& c, double* vel, double* str, double* dif,
                              cudaStream_t s);
// slots[q] <- current state of particle perm[q]
cudaError_t launch_refresh_slots(const int64_t* perm, int64_t ns, const double* pos, const double* str,
                                 const double* rad, BHPart* slots, cudaStream_t s);
cudaError_t launch_bh_points(const BHNode* nodes, const BHNodeF* fnodes, int nn, const BHPart* parts, double theta,
                             const double* pts, int64_t m, const VPConst& c, double* vel, cudaStream_t s);
// vk: 0 none, 1 symmetrised Gaussian (particle targets), 2 Gaussian at points, 3 algebraic.
// With scratch of at least direct_scratch_doubles(n, m) doubles, few targets over many
// sources split the sources into ranges summed by separate blocks and added in range order
// (the same sum in a different association); without it one block row takes all sources.
cudaError_t launch_direct(int vk, bool S, bool D, const BHPart* src, int64_t n, const BHPart* tgt, const double* pts,
                          int64_t m, const VPConst& c, double* vel, double* str, double* dif, cudaStream_t s,
                          double* scratch = nullptr, int64_t scratch_doubles = 0);
int64_t direct_scratch_doubles(int64_t n, int64_t m);
// panel records (24 doubles) of m free triangles (vertices m x 9)
cudaError_t launch_pack_records(const double* verts, int64_t m, double* rec, cudaStream_t s);
// Panel-induced velocity at points: body records (sigma, mu) and wake records (mu_w)
cudaError_t launch_panels_velocity(const double* body_verts, const double* sigma, const double* mu, int64_t nb,
                                   const double* wake_verts, const double* wmu, int64_t nw, const double* pts,
                                   int64_t m, double* rec_scratch, double* vel, cudaStream_t s);

}  // namespace cpg
