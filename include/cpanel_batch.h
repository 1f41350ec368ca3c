/*
 * cpanel_batch.h -- many meshes at once on one GB300 (sm_103a): the grouped, persistent
 * mixed-precision influence assembly, its work-shape autotuner, and a batch solve of
 * uneven meshes with several flow conditions each.
 *
 * Reference interfaces replaced (paths relative to the CPanel project root):
 *   cpg_set_inf_coeff_grouped  geometry::setInfCoeff, CPanel/geometry.cpp:809-891, which
 *                              geometry::readTri calls once per geometry
 *                              (CPanel/geometry.cpp:607-621); here m geometries share one
 *                              launch
 *   cpg_batch_solve            cpCase::run minus file output, CPanel/cpCase.cpp:31-139,
 *                              once per flow condition as CPanelMgr::run drives it
 *                              (CPanel/CPanelMgr.cpp:90-167), for m meshes at once
 *   cpg_lu_factor_grouped      the LU of the mixed path's cpCase::solveMatrixEq replacement
 *                              (CPanel/cpCase.cpp:185-214) for m geometries in lockstep
 *   cpg_group_schedule         no counterpart (host-only view of the grouped launch's
 *                              work queue, for checking and tuning)
 *
 * Results do not depend on the work shape: every work item writes its own partial sums
 * with the chunk length of the single-mesh assembly, so the grouped launch gives the
 * same bits as cpg_set_inf_coeff(g, CPG_MIXED) for every shape the tuner may pick.
 */
#ifndef CPANEL_BATCH_H
#define CPANEL_BATCH_H

#include <stdint.h>

#include "cpanel_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Work shape of the grouped assembly.  A work item is one block of 128 target rows
 * times a range of source chunks of one mesh. */
typedef struct {
    int chunks_per_item;  /* source chunks in one far item (1..16)                         */
    int near_band;        /* an item is near when its row and source index ranges lie within
                             near_band chunk lengths of each other (0..64); near items hold
                             one chunk each and are queued first (they carry the FP64 near
                             field)                                                         */
    int blocks_per_sm;    /* resident blocks of the persistent kernel per SM; 0 or more
                             than the occupancy limit = the occupancy limit (the grid is
                             this times the SM count)                                       */
} cpg_group_shape;

typedef enum {
    CPG_TUNE_OFF = 0,   /* the given shape, or the default one                          */
    CPG_TUNE_AUTO = 1,  /* the cached shape of this device and size class, else tune now */
    CPG_TUNE_FORCE = 2  /* time the candidate shapes on this group and cache the fastest */
} cpg_tune_mode;

typedef struct {
    cpg_group_shape shape;  /* the shape the final launch used                           */
    int tuned;              /* 0 given/default, 1 timed in this call, 2 from the cache    */
    int candidates;         /* shapes timed in this call                                  */
    int64_t items;          /* work items in the queue                                    */
    int64_t pairs;          /* (target, source) pairs over all meshes                     */
    int64_t near_pairs;     /* pairs evaluated in FP64                                    */
    double ms;              /* device time of the final launch: assembly, partial-sum
                               reduction and wake columns                                  */
} cpg_group_report;

/* Default shape: 2 chunks per far item, near band 1, blocks_per_sm 0 (occupancy limit). */
int  cpg_group_default_shape(cpg_group_shape* shape);

/* Mixed-precision assembly (CPG_MIXED) of m geometries in one grouped, persistent launch.
 * All geometries must live on one device; the launch runs on the stream of gs[0]'s
 * context after the work already queued on every geometry's context stream, and every
 * one of those streams waits for it.  Afterwards each geometry holds its CPG_MIXED matrix
 * exactly as cpg_set_inf_coeff(g, CPG_MIXED) would have left it.  tune: cpg_tune_mode;
 * shape: used with CPG_TUNE_OFF (null = default).  Tuning times each candidate shape
 * with one launch of the assembly kernel over this group (the kernel only overwrites, so
 * repeating it is harmless) and caches the fastest per device, group size and pair count
 * class for the rest of the process. */
int  cpg_set_inf_coeff_grouped(cpg_geometry* const* gs, int m, int tune, const cpg_group_shape* shape,
                               cpg_group_report* report);

/* FP32 LU factorizations (the CPG_MIXED solve's) of m geometries at once, each holding its
 * CPG_MIXED matrix.  The blocked LU of cpg_solve_cases taken in lockstep: every 128-column
 * block step is one launch of the diagonal-block kernel for all geometries, then one launch
 * each of the batched panel solves and updates; the rank-1024 trailing updates stay per
 * geometry.  Runs on gs[0]'s context stream like cpg_set_inf_coeff_grouped, and the
 * following cpg_solve_cases calls reuse the factors.  ms: device time (may be null).
 * The factors agree with the per-geometry factorization to FP32 rounding (different
 * summation orders), so the refined solutions agree within the refinement tolerance, not
 * bit for bit. */
int  cpg_lu_factor_grouped(cpg_geometry* const* gs, int m, double* ms);

/* Host only (no device needed): the grouped launch's work queue for meshes of n_body
 * panels.  items: cap x 4 ints (mesh, row block of 128 rows, first source chunk, chunk
 * count), costliest first; *count = number of items (items may be null to count only).
 * chunk_len: m ints, the source chunk length of each mesh (may be null). */
int  cpg_group_schedule(const int64_t* n_body, int m, const cpg_group_shape* shape, int32_t* items, int64_t cap,
                        int64_t* count, int64_t* chunk_len);

/* One mesh of a batch: .tri arrays as cpg_geometry_create takes them, k flow conditions
 * and the reference quantities; outputs in caller memory (any may be null). */
typedef struct {
    const double* nodes;
    int64_t n_nodes;
    const int64_t* tris;
    const int32_t* ids;
    int64_t n_tris;
    const cpg_flow* flows;
    int k;
    cpg_refs refs;
    double* cp;      /* k x n_body                                                     */
    double* mu;      /* k x n_body                                                     */
    double* CL;      /* k                                                              */
    double* CDi;     /* k                                                              */
    int status;      /* out: cpg_status of this mesh                                   */
    int64_t n_body;  /* out                                                            */
} cpg_batch_mesh;

typedef struct {
    int workers;          /* contexts (stream and cuBLAS handle each) that build, factor
                             and solve the meshes side by side; 0 = 8                      */
    int tune;             /* cpg_tune_mode of the grouped assembly                         */
    double budget_bytes;  /* device memory the meshes of one wave may hold together;
                             0 = three quarters of the free memory                         */
    int lockstep;         /* 0: each mesh's LU, refined solves and post on its worker;
                             1: the wave's LU factorizations in lockstep
                             (cpg_lu_factor_grouped), then its refined solves in lockstep
                             (one launch per substitution block step for every mesh)       */
} cpg_batch_params;

typedef struct {
    double ms_total;          /* host clock, whole call                                  */
    double ms_topology;       /* host clock: readTri topology and uploads (in parallel)  */
    double ms_assembly;       /* device time of the grouped launches                     */
    double ms_factor;         /* device time of the lockstep factorizations             */
    double ms_solve;          /* host clock: factorizations, refined solves and post     */
    int waves;                /* grouped launches (meshes split by the memory budget)    */
    int64_t solves;           /* (mesh, flow condition) pairs solved                     */
    int failed;               /* meshes whose status is not CPG_OK                       */
    cpg_group_report group;   /* the last wave's grouped launch                          */
} cpg_batch_stats;

/* Steady mixed-precision solves of m meshes: topology, uploads and post-processing tables
 * in parallel on the workers, one grouped assembly per wave, then either (lockstep = 0)
 * each mesh's FP32 LU, refined solves to relative residual 1e-12 and post-processing on
 * its worker's stream, the workers side by side, or (lockstep = 1) the wave's
 * factorizations and refined solves in lockstep and each mesh's post-processing on one
 * stream.  With lockstep = 0 the results equal cpg_solve_cases(g, ..., CPG_MIXED, ...) on
 * the same mesh bit for bit; with lockstep = 1 they agree within the refinement tolerance
 * (relative residual 1e-12).  Returns CPG_OK when every mesh succeeded, else the first failing
 * mesh's status (each mesh's own status is in meshes[i].status). */
int  cpg_batch_solve(cpg_ctx* ctx, cpg_batch_mesh* meshes, int m, const cpg_batch_params* params,
                     cpg_batch_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* CPANEL_BATCH_H */
