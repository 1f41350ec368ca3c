/*
 * cpanel_gpu.h -- C ABI of the GB300 (sm_103a) CPanel steady panel path.
 *
 * Plain pointers and sizes only.  Every call returns a cpg_status; the message of
 * the last failure on a context is returned by cpg_last_error().  Nothing here
 * exits, prompts or prints.
 *
 * Reference interfaces replaced (paths relative to the CPanel project root):
 *   cpg_geometry_create   geometry::readTri topology, CPanel/geometry.cpp:132-484
 *   cpg_set_inf_coeff     geometry::setInfCoeff, CPanel/geometry.cpp:809-891
 *   cpg_get_A / cpg_get_B geometry::getA / getB, CPanel/geometry.h:310-311
 *   cpg_solve_cases       cpCase::run minus file output, CPanel/cpCase.cpp:31-139
 *                         (setSourceStrengths :174-183, solveMatrixEq :185-214,
 *                          compVelocity :342-365, trefftzPlaneAnalysis :541-552)
 *   cpg_stability_derivatives  cpCase::stabilityDerivatives, CPanel/cpCase.cpp:635-665
 *   cpg_volume_velocity   cpCase::velocityAtPoint, CPanel/cpCase.cpp:1007-1021
 *   cpg_spanwise_loads    wake::getSpanwisePnts/Cl/Cd as cpCase::writeSpanwiseData scales them,
 *                         CPanel/cpCase.cpp:910-935, wake.cpp:146-188
 *   cpg_streamlines       streamline::streamline / rkf, CPanel/streamline.cpp:20-78, through
 *                         geometry::pntVelocity, CPanel/geometry.cpp:1239-1253
 *   cpg_panel_phi_inf     bodyPanel::panelPhiInf, CPanel/bodyPanel.cpp:132-190
 *   cpg_dub_phi_inf       panel::dubPhiInf, CPanel/panel.cpp:208-252
 *   cpg_panel_v_inf       bodyPanel::panelVInf, CPanel/bodyPanel.cpp:305-348
 */
#ifndef CPANEL_GPU_H
#define CPANEL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CPG_OK = 0,
    CPG_E_INVALID = 1,        /* bad argument or size                           */
    CPG_E_OOM = 2,            /* device or host allocation refused              */
    CPG_E_CUDA = 3,           /* a CUDA runtime call failed                     */
    CPG_E_BAD_MESH = 4,       /* topology the reference would reject or crash on */
    CPG_E_NOT_CONVERGED = 5,  /* solver finished above its tolerance (results valid) */
    CPG_E_TIMEOUT = 6,        /* a bounded device wait ran out                  */
    CPG_E_NO_DEVICE = 7       /* no CUDA device / extension not usable          */
} cpg_status;

typedef enum {
    CPG_PLAIN_FP64 = 0,  /* the reference method in FP64: explicit A, B; BiCGSTAB to eps */
    CPG_MIXED = 1        /* double-float far field + FP64 near field, matrix kept as an
                            FP32 hi + lo pair; FP32 LU + refinement with an exact-
                            product residual to relative residual 1e-12              */
} cpg_precision;

typedef struct cpg_ctx cpg_ctx;
typedef struct cpg_geometry cpg_geometry;

typedef struct {
    int64_t n_body;      /* body panels = matrix order                         */
    int64_t n_wake;      /* wake panels (wPanels)                              */
    int64_t n_wakes;     /* wakes after merging                                */
    int64_t n_wakelines; /* trailing-edge wake lines, summed over wakes        */
    int64_t n_tip;       /* panels flagged as tip patch                        */
    int64_t n_nodes;
    int64_t h2d_bytes;   /* bytes copied host->device by cpg_geometry_create      */
} cpg_geometry_info;

typedef struct {
    double V, alpha, beta, mach; /* one flow condition (degrees)                */
} cpg_flow;

typedef struct {
    double Sref, bref, cref, cg[3];
} cpg_refs;

/* Host output buffers of cpg_solve_cases; any pointer may be null (not returned).
 * Per-panel arrays are k x n_body row-major (case-major). */
typedef struct {
    double* mu;      /* doublet strengths                                        */
    double* sigma;   /* source strengths                                         */
    double* phi;     /* panel potential                                          */
    double* vel;     /* k x n x 3                                                */
    double* cp;
    double* CL;      /* k: Trefftz plane                                         */
    double* CDi;     /* k                                                        */
    double* Fbody;   /* k x 3 */
    double* Fwind;   /* k x 3 */
    double* CM;      /* k x 3 */
} cpg_case_out;

typedef struct {
    int64_t iters_max;      /* most Krylov iterations over the k cases          */
    int64_t iters_total;
    int64_t refinements;    /* outer refinement steps (CPG_MIXED)                */
    double  residual_max;   /* largest final relative residual                   */
    int64_t n_near;         /* near-field pairs found by the last assembly       */
    int64_t n_far;
    double  ms_assemble, ms_solve, ms_post; /* device time of the last calls      */
} cpg_solve_stats;

/* ---- context ---- */
int         cpg_create(cpg_ctx** out, int device);
void        cpg_destroy(cpg_ctx* ctx);
const char* cpg_last_error(const cpg_ctx* ctx);
/* All work of a context is issued on this stream (cudaStream_t; 0 = the context's
 * own non-blocking stream). */
int         cpg_set_stream(cpg_ctx* ctx, void* stream);
int         cpg_synchronize(cpg_ctx* ctx);

/* ---- geometry: readTri topology + device-resident panel tables ----
 * nodes n_nodes x 3, tris n_tris x 3 (1-based, Cart3D order), ids per tri (>1000: wake). */
int  cpg_geometry_create(cpg_ctx* ctx, const double* nodes, int64_t n_nodes, const int64_t* tris,
                         const int32_t* ids, int64_t n_tris, cpg_geometry** out);
/* Destroy a geometry before its context: its matrix buffers go to the context's spares
 * (at most 6 buffers and 16 GB), taken by the next geometry of a similar size. */
void cpg_geometry_destroy(cpg_geometry* g);
/* Free the context's spare matrix buffers now (for callers that account for device memory
 * themselves; the request loop and the batch solve call it after each request and wave). */
int  cpg_release_spares(cpg_ctx* ctx);
int  cpg_geometry_info_get(const cpg_geometry* g, cpg_geometry_info* out);
/* Host copies of the topology for checking (same layouts as the CPU oracle):
 * body: n_body x 18 [c(3) n(3) l(3) area longSide tip upper lower TSorder surfID
 * cluster_size file_tri]; wake: n_wake x 8 [c(3) n(3) area longSide] + idx4 + coef;
 * clusters: n_body x 32 (matrix indices, -1 padded, self first). */
int  cpg_geometry_tables(const cpg_geometry* g, double* body, double* wake, int32_t* idx4, double* coef,
                         int32_t* clusters);

/* Host-only topology (no device needed): the same tables as cpg_geometry_tables
 * straight from .tri arrays.  Call with null table pointers to fill *info only. */
int  cpg_topology(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids, int64_t n_tris,
                  cpg_geometry_info* info, double* body, double* wake, int32_t* idx4, double* coef,
                  int32_t* clusters);

/* Host-only (no device needed): the .tri triangle (zero-based) of each wake panel in wPanels
 * order (n_wake values), for writing wake results against the input mesh. */
int  cpg_topology_wake_tris(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                            int64_t n_tris, int64_t* wake_tris);

/* ---- assembly (geometry::setInfCoeff) ----
 * CPG_PLAIN_FP64 builds A and B (n x n FP64, column-major, A(i,j) = A[j*n+i]).
 * CPG_MIXED builds A in FP32 plus the FP64 near-field correction and the three
 * source right-hand-side basis vectors (B is never stored). */
int  cpg_set_inf_coeff(cpg_geometry* g, int precision);
/* Copy the assembled matrices to host column-major buffers (n*n doubles).
 * cpg_get_A works for both precisions (CPG_MIXED: the float pair hi + lo as FP64, the
 * matrix its refinement solves with). */
int  cpg_get_A(cpg_geometry* g, double* host);
int  cpg_get_B(cpg_geometry* g, double* host);

/* Allocation-free FP64 assembly.  No counterpart in the reference: it exists for
 * callers that may not allocate device memory while the path runs (a host that
 * records the assembly into a CUDA graph, a plug-in confined to another solver's
 * memory pool, a real-time loop that forbids allocation after start-up).
 * Inputs and outputs are caller-owned DEVICE arrays in matrix order: body_verts
 * n x 9, wake_verts nw x 9 (wPanels order), wake_idx4 nw x 4 and wake_coef nw (the
 * tables cpg_geometry_tables / cpg_topology return), A and B n x n column-major.
 * Every wake_idx4 entry must lie in [0, n): the kernels index columns of A with them
 * unchecked, as the geometry's own tables always satisfy.
 * A CUDA error already pending on the calling thread when the call starts is returned as
 * CPG_E_CUDA before anything is queued, and left pending for the caller to read.
 * The packed panel records live in a fixed per-device array of 16,384 panels
 * (n + nw <= 16384; larger sizes return CPG_E_INVALID, about 3 MB held by every GPU
 * that loads the library).  The first call on a device looks the array's address
 * up (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the one array, so calls whose work overlaps on the GPU race:
 * serialize them (one stream, or events).  stream: cudaStream_t, 0 = default. */
int  cpg_set_inf_coeff_noalloc(const double* body_verts, int64_t n, const double* wake_verts,
                               const int32_t* wake_idx4, const double* wake_coef, int64_t nw, double* A,
                               double* B, void* stream);

/* ---- steady cases (cpCase::run) over k flow conditions on one geometry ----
 * Assembles first if the geometry holds no matrix of that precision. */
int  cpg_solve_cases(cpg_geometry* g, const cpg_flow* flows, int k, const cpg_refs* refs, int precision,
                     const cpg_case_out* out, cpg_solve_stats* stats);

/* ---- stability derivatives (cpCase::stabilityDerivatives, CPanel/cpCase.cpp:635-665) ----
 * The base case and the reference's two sub-cases (alpha + 0.5 deg, beta + 0.5 deg) solved as
 * three right-hand sides of one cpg_solve_cases call, then the reference's forward differences
 * over 0.5 deg: F = (CDi, CY wind, CL) with the Trefftz-plane CL and CDi, M = (roll, pitch, yaw).
 * base (may be null): the base case's outputs as cpg_solve_cases would give them for k = 1.
 * Unlike the reference, the base case's panel state is what base receives (the reference's
 * sub-cases overwrite the panel state before its files are written). */
typedef struct {
    double dF_dAlpha[3], dF_dBeta[3];  /* per radian: (CD, CY, CL)    */
    double dM_dAlpha[3], dM_dBeta[3];  /* per radian: (roll, pitch, yaw) */
} cpg_stability;
int  cpg_stability_derivatives(cpg_geometry* g, const cpg_flow* flow, const cpg_refs* refs, int precision,
                               const cpg_case_out* base, cpg_stability* out);

/* ---- velocity anywhere in the flow (cpCase::velocityAtPoint, CPanel/cpCase.cpp:1007-1021) ----
 * The velocity that all body and wake panels of g induce at m points (host arrays pts m x 3 ->
 * vel m x 3), for one case's source and doublet strengths (host arrays sigma, mu: n_body).  The
 * wake doublets follow from mu through the trailing-edge interpolation of the assembly.  V_inf
 * is not included (the reference adds it in populateVolMesh, CPanel/cpCase.cpp:1105-1122). */
/* ---- spanwise Trefftz-plane loads (cpCase::writeSpanwiseData, CPanel/cpCase.cpp:910-935) ----
 * cpg_trefftz_wakes: the number of wakes with a Trefftz plane, in the order CL sums them (the
 * reference's spanwiseData_Wake<i + 1>.csv).  cpg_spanwise_loads: for case c of the last
 * cpg_solve_cases call on g and wake `wake`, the reference's 165 stations (wake::trefftzPlane,
 * wake.cpp:146-188): 2y/b, Cl / PG and Cdi / PG^2 (PG = sqrt(1 - M^2); the end stations carry zero
 * loads).  *n: in, the length of each buffer; out, the stations (165).  CPG_E_INVALID if no steady
 * case was solved on g, if c or wake is out of range or the buffers are too short (*n then holds
 * the length needed). */
int  cpg_trefftz_wakes(const cpg_geometry* g);
int  cpg_spanwise_loads(cpg_geometry* g, int c, int wake, double* y2b, double* cl, double* cdi, int* n);

int  cpg_volume_velocity(cpg_geometry* g, const double* sigma, const double* mu, const double* pts, int64_t m,
                         double* vel);

/* ---- off-body streamlines (streamline::streamline / rkf, CPanel/streamline.cpp:20-78) ----
 * Integrates n_lines streamlines from starts (n_lines x 3) with the reference's adaptive
 * Runge-Kutta-Fehlberg 4(5) step: the first step is 0.1 / |V_inf|; after each step whose error
 * estimate err (the distance between the fifth- and fourth-order steps) is positive,
 * dt <- dt (tol dt / (2 err))^(1/4); a line stops once a step ends at x >= x_max.  The velocity is
 * geometry::pntVelocity's (CPanel/geometry.cpp:1239-1253): the panels' velocity for the case's
 * strengths (as cpg_volume_velocity) plus V_inf, its x component divided by sqrt(1 - M^2).
 * Every step start is recorded with its velocity: pts and vel are n_lines x max_points x 3, line i's
 * points first; counts[i] is the number recorded; ended[i] is 1 where the line stopped as the
 * reference's loop stops (x >= x_max, or x no longer a number) and 0 where max_points cut it short.
 * Treat a line with ended 0 as truncated: its last point starts a step that was not taken.  The
 * reference has no such cap (a line that never reaches x_max, at a stagnation point for one, keeps
 * stepping there).  All lines advance together: each of the six stages evaluates every live line's stage point in
 * one batched panel-velocity launch. */
int  cpg_streamlines(cpg_geometry* g, const double* sigma, const double* mu, const cpg_flow* flow,
                     const double* starts, int n_lines, double x_max, double tol, int max_points, double* pts,
                     double* vel, int32_t* counts, int32_t* ended);

/* The same integrator through a caller's velocity field (host only): fn(user, p, m, v) writes into v
 * (m x 3) the velocity at the points p (m x 3), free stream and compressibility included, and returns
 * 0; a non-zero return stops the integration and is returned.  The first step is 0.1 / speed. */
typedef int (*cpg_velocity_fn)(void* user, const double* p, int64_t m, double* v);
int  cpg_streamlines_field(cpg_velocity_fn fn, void* user, double speed, const double* starts, int n_lines,
                           double x_max, double tol, int max_points, double* pts, double* vel, int32_t* counts,
                           int32_t* ended);

/* ---- single-evaluation influence operators on DEVICE arrays (batched) ----
 * verts m x 9 (three vertices), poi m x 3; outputs m (phi) or m x 3 (velocity). */
int  cpg_panel_phi_inf(cpg_ctx* ctx, const double* verts, const double* poi, int64_t m, double* phi_src,
                       double* phi_dub);
int  cpg_dub_phi_inf(cpg_ctx* ctx, const double* verts, const double* poi, int64_t m, double* phi_dub);
int  cpg_panel_v_inf(cpg_ctx* ctx, const double* verts, const double* poi, int64_t m, double* v_src,
                     double* v_dub);

/* ---- optional device-time accounting (CUDA events on the context's stream) ----
 * Classes: 0 assembly, 1 wake columns, 2 FP32 matvec, 3 FP64 matvec, 4 refinement
 * residual, 5 LU factorization (one graph launch), 6 particle and panel-velocity
 * operators (cpanel_vp.h), 7 CHTLS weights,
 * 8 velocity/Cp/forces, 9 LU triangular solves (one graph launch per solve), 10 tensor-core
 * GEMM launches (cpg_gemm_f32_tc and the factorizations' GEMMs; nested in class 5 there). */
#define CPG_PROF_NCLS 11
typedef struct {
    long long launches[CPG_PROF_NCLS];
    double ms[CPG_PROF_NCLS];
} cpg_prof;
int  cpg_prof_enable(cpg_ctx* ctx, int on);           /* on != 0 starts (and clears) */
int  cpg_prof_read(cpg_ctx* ctx, cpg_prof* out);      /* totals since enable        */

/* FP64 FMA throughput of the context's GPU in TFLOP/s (a short probe kernel), the
 * denominator for FP64-issue-bound kernels. */
int  cpg_measure_fp64_peak(cpg_ctx* ctx, double* tflops);

/* The tensor-core GEMM of the mixed path's factorizations, on caller-owned FP32 DEVICE matrices
 * (column-major): C = alpha A B + beta C with A m x k (lda), B k x n (ldb), C m x n (ldc); beta = 0
 * does not read C.  No counterpart in the reference (its solves are Eigen's BiCGSTAB): it is the
 * sm_103a kernel the mixed LU runs (tcgen05 MMAs in tensor memory, operands by TMA), exposed so
 * hosts and tests can call it.  Each operand row is scaled by a power of two and split into two
 * FP16 halves; the three leading products are accumulated in FP32, which gives about 22
 * significant bits per product.  sm_budget: SMs the persistent grid may take (0: all).
 * Allocates its split operands for the call.  CPG_E_TIMEOUT when a wait of the kernel ran out. */
int  cpg_gemm_f32_tc(cpg_ctx* ctx, int64_t m, int64_t n, int64_t k, float alpha, const float* A, int64_t lda,
                     const float* B, int64_t ldb, float beta, float* C, int64_t ldc, int sm_budget);

/* A (n x n, column-major FP32 device matrix) <- its unpivoted LU factors (unit lower L below the
 * diagonal, U on and above it); X (n x k, ld n, device) <- A^{-1} X by the blocked forward and
 * backward substitutions.  The factorization and substitutions of the mixed precision, without
 * the refinement.  No counterpart in the reference (its solves are Eigen's BiCGSTAB,
 * CPanel/cpCase.cpp:192); exposed so hosts and tests can call the kernels directly.  Allocates
 * its inverses and scratch for the call.  CPG_E_INVALID on a zero pivot or non-finite entry. */
int  cpg_lu_solve_f32(cpg_ctx* ctx, int64_t n, float* A, int64_t k, float* X);

/* Build identification: the sm architecture the kernels were compiled for. */
int  cpg_compiled_arch(void);

#ifdef __cplusplus
}
#endif
#endif /* CPANEL_GPU_H */
