/*
 * cpo_vp.h -- CPU oracle for the vortex-particle operators (TEST INFRASTRUCTURE ONLY).
 *
 * Restates, in FP64 and in the reference's own evaluation order:
 *   particle::velInflAlgSmooth / velInfl / vortexStretching / viscousDiffusion
 *     (CPanel/particle.cpp:31-140, coreOverlap 1.5 at CPanel/particle.h:32);
 *   the octree build of octree::addData / node::addMember / pushMember / createChild
 *     (octree/include/octree.h:39-195, octree/include/node.h:46-214);
 *   particleFMM::computeMultExp and the Barnes-Hut queries barnesHutVel/Stretch/Diff
 *     (CPanel/particleFMM.cpp:30-175, octree/include/node.h:236-421).
 * Particles are SoA arrays: pos n x 3, strength n x 3, radius n.
 */
#pragma once
#include <cstdint>

extern "C" {

/* direct sums over all particles j
 * mode 0: velocity at particle i from all j != i, Gaussian symmetrised core (velInfl(particle*))
 * mode 1: velocity at points, Gaussian core 1.5 r_j (velInfl(POI)); this is the direct
 *         branch of cpCaseVP::velocityInflFromEverything, CPanel/cpCaseVP.cpp:651-655,697-703,
 *         with the particle positions as the points (the self term is zero there)
 * mode 2: velocity at points, high-order algebraic core (velInflAlgSmooth) */
void cpo_vp_direct_velocity(const double* pos, const double* str, const double* rad, int64_t n,
                            const double* pts, int64_t m, int mode, double* vel);
/* the direct branch of cpCaseVP::particleStrengthUpdate, CPanel/cpCaseVP.cpp:504-516:
 * sum over j != i of particles[i]->vortexStretching(particles[j]) (resp. viscousDiffusion).
 * Note the roles: here `this` is the target i; in the Barnes-Hut leaves (node.h:299-364)
 * `this` is the source member, which flips the diffusion sign and changes the stretching
 * cut-off radius.  Both forms are restated as the reference has them. */
void cpo_vp_direct_stretch(const double* pos, const double* str, const double* rad, int64_t n, double* out);
void cpo_vp_direct_diffusion(const double* pos, const double* str, const double* rad, int64_t n, double* out);

/* Barnes-Hut octree (fresh build, particles inserted in order) */
void*   cpo_bh_build(const double* pos, const double* str, const double* rad, int64_t n, int64_t max_members,
                     double theta);
void    cpo_bh_free(void* t);
int64_t cpo_bh_num_nodes(void* t);
int64_t cpo_bh_num_levels(void* t);
/* per node in pre-order (root first): [origin(3) half(3) level leaf n_members exp_pos(3)
 * exp_str(3) exp_radius child0..7] (child = pre-order node index or -1; 24 doubles).
 * The root has no expansion (zeros).  A node at level 32 is never split (the reference
 * has no limit and recurses without end on more than max_members coincident points). */
void    cpo_bh_nodes(void* t, double* out);
/* particle indices of every leaf, leaves in pre-order, members in insertion order */
void    cpo_bh_leaf_members(void* t, int64_t* out);
/* queries: mode 0 points (algebraic leaves), 1 particles (Gaussian leaves, self skipped) */
void    cpo_bh_velocity(void* t, const double* pts, int64_t m, int mode, double* vel);
void    cpo_bh_stretch(void* t, double* out);
void    cpo_bh_diffusion(void* t, double* out);

}
