/*
 * cpanel_vp.h -- C ABI of the GB300 vortex-particle operators (sm_103a).
 *
 * Particle arrays are device pointers in structure-of-arrays form: positions and
 * strengths n x 3 (row-major), radii n.  Outputs are device arrays of the same
 * layout.  Every call is ordered on the context's stream and returns when its
 * results are ready.  Status codes and cpg_last_error() as in cpanel_gpu.h.
 *
 * Reference interfaces replaced (paths relative to the CPanel project root):
 *   cpg_ptree_build            particleOctree::addData on a fresh tree + particleFMM::build,
 *                              octree/include/octree.h:151-195, CPanel/particleFMM.cpp:22-62
 *   cpg_ptree_table            octree::getNodes / node getters, octree/include/node.h:448-577
 *   cpg_bh_velocity_points     particleFMM::barnesHutVel(POI), CPanel/particleFMM.cpp:65-77
 *   cpg_bh_particles           particleFMM::barnesHutVel(particle*), barnesHutStretch,
 *                              barnesHutDiff, CPanel/particleFMM.cpp:79-116
 *   cpg_particles_velocity     the direct sums of particle::velInfl(POI) / velInfl(particle*)
 *                              / velInflAlgSmooth, CPanel/particle.cpp:31-77, as called at
 *                              CPanel/cpCaseVP.cpp:609-612,651-655,697-703
 *   cpg_particles_stretch_diff the direct branch of cpCaseVP::particleStrengthUpdate,
 *                              CPanel/cpCaseVP.cpp:504-516 (particle.cpp:80-140)
 *   cpg_panels_velocity        bodyPanel::panelV + wakePanel::panelV summed over panels,
 *                              CPanel/bodyPanel.cpp:122-130, CPanel/wakePanel.cpp:89-92,
 *                              as called at CPanel/cpCaseVP.cpp:713-731
 *   cpg_panels_stretching      bodyPanel::partStretching + wakePanel::partStretching summed
 *                              over panels, CPanel/bodyPanel.cpp:697-1063,
 *                              CPanel/wakePanel.cpp:266-289, CPanel/panel.cpp:113-153,813-966
 *   cpg_vpcase_*               cpCaseVP on a body-only mesh: the buffer wake of
 *                              CPanel/geometry.cpp:261-400,1313-1345, and cpCaseVP::run,
 *                              CPanel/cpCaseVP.cpp:26-117 (convection, shedding, strength
 *                              update, octree rebuild, source strengths, solve) one step
 *                              at a time, with the Trefftz-plane early stop
 *                              (cpCaseVP::solutionConvergence, CPanel/cpCaseVP.cpp:204-229;
 *                              wake::trefftzPlaneVP, CPanel/wake.cpp:191-361)
 *   cpg_vpcase_surface         cpCaseVP::compVelocity, CPanel/cpCaseVP.cpp:370-393
 */
#ifndef CPANEL_VP_H
#define CPANEL_VP_H

#include <stdint.h>

#include "cpanel_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cpg_ptree cpg_ptree;

typedef struct {
    int64_t n_particles;
    int64_t n_nodes;
    int64_t n_leaves;
    int64_t n_levels; /* octree::numTreeLevels (root = level 1) */
} cpg_ptree_info;

/* Velocity kernels of cpg_particles_velocity */
typedef enum {
    CPG_VEL_GAUSS_SYM = 1, /* particle::velInfl(particle*): targets are the particles, self skipped */
    CPG_VEL_GAUSS = 2,     /* particle::velInfl(POI): Gaussian core 1.5 r, zero at distance 0     */
    CPG_VEL_ALG = 3        /* particle::velInflAlgSmooth                                         */
} cpg_vel_kernel;

/* Builds the particle octree with the reference's rules (root cube 0.51 x largest
 * extent about the box centre; leaves split above max_members; octant x>o:4, y>o:2,
 * z>o:1) and the lumped expansions.  theta is the far-field ratio (0.5 in the
 * reference).  Nodes deeper than level 32 are not split (the reference has no limit
 * and recurses without end on more than max_members coincident particles). */
int  cpg_ptree_build(cpg_ctx* ctx, const double* pos, const double* strength, const double* radius, int64_t n,
                     int64_t max_members, double theta, cpg_ptree** out);
void cpg_ptree_destroy(cpg_ptree* t);
int  cpg_ptree_info_get(const cpg_ptree* t, cpg_ptree_info* info);
/* Host copy of the tree, nodes in the reference's pre-order (node::getSubNodes): 24
 * doubles per node [origin(3) half(3) level leaf n_members exp_pos(3) exp_strength(3)
 * exp_radius child0..7 (pre-order index or -1)]; the root carries no expansion (zeros).
 * leaf_members (n, may be null): particle indices of the leaves in pre-order. */
int  cpg_ptree_table(const cpg_ptree* t, double* nodes, int64_t* leaf_members);
/* Host-only build of the same tree from host arrays (no device use; for checking and
 * for hosts that want the tree itself).  Fills info; writes the node table only when
 * cap_nodes >= info->n_nodes (else returns CPG_E_INVALID with info filled). */
int  cpg_ptree_host_table(const double* pos, const double* strength, const double* radius, int64_t n,
                          int64_t max_members, double* nodes, int64_t cap_nodes, int64_t* leaf_members,
                          cpg_ptree_info* info);
/* Precision of this tree's traversals: CPG_PLAIN_FP64 (default; every interaction in
 * FP64) or CPG_MIXED (far nodes in FP32 from a float view of their expansions, leaf
 * members -- the direct near field -- in FP64; far/near and cut-off decisions equal the
 * FP64 ones, so the same nodes are visited). */
int  cpg_ptree_set_precision(cpg_ptree* t, int precision);
/* barnesHutVel(POI) at m points (device pts m x 3 -> vel m x 3) */
int  cpg_bh_velocity_points(cpg_ptree* t, const double* pts, int64_t m, double* vel);
/* barnesHutVel(particle*), barnesHutStretch, barnesHutDiff for every particle of the
 * tree in one traversal; any output may be null.  Outputs by particle index. */
int  cpg_bh_particles(cpg_ptree* t, double* vel, double* stretch, double* diff);

/* Direct velocity sums over n particles at m points (kernel CPG_VEL_GAUSS or
 * CPG_VEL_ALG), or at the particles themselves (pts = NULL, m = n; any kernel). */
int  cpg_particles_velocity(cpg_ctx* ctx, const double* pos, const double* strength, const double* radius,
                            int64_t n, const double* pts, int64_t m, int kernel, double* vel);
/* Direct stretching and diffusion on every particle: sum over j != i of
 * particles[i]->vortexStretching(particles[j]) (resp. viscousDiffusion); either
 * output may be null. */
int  cpg_particles_stretch_diff(cpg_ctx* ctx, const double* pos, const double* strength, const double* radius,
                                int64_t n, double* stretch, double* diff);

/* Precision of this context's panel-particle operators (cpg_panels_velocity,
 * cpg_panels_stretching): CPG_PLAIN_FP64 (default) or CPG_MIXED (body-panel pairs
 * beyond five panel lengths -- the point-source/point-doublet branch -- in FP32, the
 * rest in FP64, the same near/far split). */
int  cpg_set_particle_precision(cpg_ctx* ctx, int precision);

/* Panel-induced velocity at m points: sum over nb body triangles (vertices nb x 9)
 * of sigma_j vSrc + mu_j vDub, then over nw wake triangles of mu_w dubVInf.
 * All arrays on the device; wake arrays may be null when nw = 0. */
int  cpg_panels_velocity(cpg_ctx* ctx, const double* body_verts, const double* sigma, const double* mu,
                         int64_t nb, const double* wake_verts, const double* wake_mu, int64_t nw,
                         const double* pts, int64_t m, double* vel);

/* Panel-induced stretching on m particles (pos, strength m x 3): sum over nb body
 * triangles (vertices nb x 9, sigma, mu) of bodyPanel::partStretching and over nw wake
 * quadrilaterals (vertices nw x 12, mu) of wakePanel::partStretching.  Device arrays. */
int  cpg_panels_stretching(cpg_ctx* ctx, const double* body_verts, const double* sigma, const double* mu,
                           int64_t nb, const double* wake_verts, const double* wake_mu, int64_t nw,
                           const double* pos, const double* strength, int64_t m, double* out);

/* ---- the vortex-particle case ---- */
typedef struct cpg_vpcase cpg_vpcase;
typedef struct {
    double V, alpha, beta; /* free stream (degrees)                                       */
    double dt;             /* time step; <= 0: mean trailing-edge length / V (calcTimeStep) */
    double cref;           /* reference chord of the far-field cut-offs (12 c, 20 c)       */
    int accelerate;        /* Barnes-Hut (inputParams::accelerateCode) or direct sums      */
    double Sref;           /* reference area of the Trefftz-plane coefficients (> 0)       */
    double mach;           /* Prandtl-Glauert factor sqrt(1 - M^2) of those coefficients   */
    int precision;         /* CPG_PLAIN_FP64: the reference method in FP64.  CPG_MIXED:
                              particle-node and panel far fields in FP32 (near fields, and
                              every near/far decision, as in FP64) and refinement against
                              FP64 A to 1e-12 each step with an FP32 inverse of A formed
                              once from its LU (BiCGSTAB for a step whose refinement
                              stalls)                                                  */
    int run_all_steps;     /* 0: the reference's loop, which stops once the Trefftz-plane
                              check fires (CPanel/cpCaseVP.cpp:94-100); nonzero: keep
                              stepping (a benchmark of the full step count; the check
                              still runs and cpg_vpcase_trefftz reports that it fired)   */
} cpg_vp_params;
typedef struct {
    int64_t n_body, n_w1, n_w2;   /* body panels, first and second buffer rows           */
    int64_t n_particles;
    int64_t timestep;             /* completed steps (the reference's timestep counter)   */
    int64_t solver_iters;         /* BiCGSTAB iterations (CPG_MIXED: refinement steps) of
                                     the last solve                                      */
    double dt;
    int64_t n_tree_nodes;         /* octree of the last rebuild                          */
    int64_t solve_fallbacks;      /* CPG_MIXED: steps whose refinement stalled            */
} cpg_vp_info;
/* Host-only build of the buffer wake (no device use): counts[3] = n_body, n_w1, n_w2 and
 * *dt_out always; the other outputs (w1/w2 vertices n x 12, first-row interpolation
 * columns n_w1 x 4 and coefficients, second-row parents) when non-null. */
int  cpg_vp_topology(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                     int64_t n_tris, double V, double dt, int64_t* counts, double* dt_out, double* w1_verts,
                     double* w2_verts, int32_t* w1_idx4, double* w1_coef, int32_t* w2_parent);
/* Mesh as in cpg_geometry_create (host arrays, 1-based triangles); no wake panels. */
int  cpg_vpcase_create(cpg_ctx* ctx, const double* nodes, int64_t n_nodes, const int64_t* tris,
                       const int32_t* ids, int64_t n_tris, const cpg_vp_params* params, cpg_vpcase** out);
void cpg_vpcase_destroy(cpg_vpcase* c);
int  cpg_vpcase_info_get(const cpg_vpcase* c, cpg_vp_info* info);
/* advance nsteps time steps (step 1: steady solve; 2: first buffer convection; then the
 * loop).  From step 5 on every step ends with the Trefftz-plane convergence check of
 * cpCaseVP::solutionConvergence (CPanel/cpCaseVP.cpp:204-229): once CL and CD both change
 * by less than 0.01 % the case is converged and further steps do nothing, as the
 * reference leaves its time loop (CPanel/cpCaseVP.cpp:94-100), unless run_all_steps. */
int  cpg_vpcase_step(cpg_vpcase* c, int nsteps);
/* Trefftz-plane CL and CD of the current state (cpCaseVP::trefftzPlaneAnalysisVP,
 * CPanel/cpCaseVP.cpp:418-429; wake::trefftzPlaneVP, CPanel/wake.cpp:191-320) and whether
 * the convergence check has fired.  Any pointer may be null. */
int  cpg_vpcase_trefftz(cpg_vpcase* c, double* CL, double* CD, int* converged);
/* Convective velocity of every particle at the current state (host vel n_particles x 3):
 * Vinf + particle term + panel/filament term (the latter zero beyond 12 cref), as the
 * next step's convection evaluates it (cpCaseVP::convectParticles, CPanel/cpCaseVP.cpp:
 * 370-391).  precision CPG_PLAIN_FP64 or CPG_MIXED; direct != 0 replaces the octree by
 * the FP64 direct sum over all particles (symmetrised Gaussian core, self excluded). */
int  cpg_vpcase_velocities(cpg_vpcase* c, int precision, int direct, double* vel);
/* host copies: particles in shedding order (pos, strength n x 3, radius, shed step, index
 * of the shedding second-row panel); any pointer may be null */
int  cpg_vpcase_particles(cpg_vpcase* c, double* pos, double* strength, double* radius, int32_t* shed_time,
                          int32_t* parent);
int  cpg_vpcase_strengths(cpg_vpcase* c, double* sigma, double* mu, double* mu_w1, double* mu_w2);
/* cpCaseVP::compVelocity of a steady case (CPanel/cpCaseVP.cpp:370-393) on the current state:
 * the panel potentials solveVPmatrixEq sets, (Vinf + particle + filament velocity at the
 * centre) . centre - mu (cpCaseVP::VinfPlusVecPot, :601-623), give the CHTLS surface velocity
 * (x divided by the Prandtl-Glauert factor), Cp = 1 - (|V| / V)^2 and the surface-integrated
 * coefficients.  The clusters are those readTri grows after the buffer wake exists
 * (CPanel/geometry.cpp:473-484).  Host outputs, any may be null: phi (n), vel (n x 3), cp (n),
 * forces (9: Fbody, Fwind, CM about cg with bref, cref; Sref of the case).  At least one step
 * must have been taken. */
int  cpg_vpcase_surface(cpg_vpcase* c, const double* cg, double bref, double cref, double* phi, double* vel,
                        double* cp, double* forces);
/* buffer-wake quadrilaterals (n_w1 x 12, n_w2 x 12 doubles) */
int  cpg_vpcase_wake(const cpg_vpcase* c, double* w1_verts, double* w2_verts);
/* A, B (n x n) and C (n x n_w2), column-major, host */
int  cpg_vpcase_matrices(cpg_vpcase* c, double* A, double* B, double* C);

#ifdef __cplusplus
}
#endif

#endif /* CPANEL_VP_H */
