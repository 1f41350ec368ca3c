/*
 * cpo.h -- CPU oracle for the CPanel steady hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain C++17 FP64 restatement of the reference algorithms, written to
 * check the GPU library.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs may load it.  The product path never calls
 * into it.
 *
 * Every function cites the reference file:line it restates (paths relative to the
 * CPanel project root).  Parity is pinned against the reference's own fixtures:
 *   - CPanelTests/influenceTests.cpp:598-643 (single-triangle phi known answers)
 *   - Connor Cases/4412 (4412.tri, 4412.CPout CL/CDi/forces, surfaceData-0.vtu)
 * See tests/test_oracle_pin.py.
 */
#pragma once
#include <cstdint>

extern "C" {

/* ---- mesh ingest + topology (geometry::readTri, CPanel/geometry.cpp:132-629) ---- */
/* nodes: n_nodes x 3 (row-major); tris: n_tris x 3, 1-based as in a Cart3D .tri
 * file; ids: surface id per tri (>1000 means wake).  Returns an opaque handle. */
void*   cpo_mesh_new(const double* nodes, int64_t n_nodes, const int64_t* tris,
                     const int32_t* ids, int64_t n_tris);
void    cpo_mesh_free(void* m);
int64_t cpo_n_body(void* m);
int64_t cpo_n_wake(void* m);
int64_t cpo_n_wakes(void* m);
int64_t cpo_n_wakelines(void* m, int64_t wake);

/* body panel table in matrix order (bPanels): per panel 18 doubles
 * [c(3) n(3) l(3) area longSide tip upper lower TSorder surfID cluster_size file_tri] */
void    cpo_body_table(void* m, double* out);
/* wake panel table in wPanels order: per panel 8 doubles
 * [c(3) n(3) area longSide] and interp data idx(4, matrix columns), coeff */
void    cpo_wake_table(void* m, double* out, int32_t* idx4, double* coef);
/* cluster lists: out_idx n_body x 32 (matrix indices, -1 padded, self first) */
void    cpo_clusters(void* m, int32_t* out_idx);
/* triangle vertex coordinates per body panel (n_body x 9) and wake panel (n_wake x 9) */
void    cpo_body_verts(void* m, double* out);
void    cpo_wake_verts(void* m, double* out);

/* ---- influence kernels (single evaluation) ---- */
/* bodyPanel::panelPhiInf, CPanel/bodyPanel.cpp:132-190 for a free triangle */
void    cpo_tri_phi_inf(const double* verts9, const double* poi, double* phi_src,
                        double* phi_dub);
/* panel::dubPhiInf, CPanel/panel.cpp:208-252 */
double  cpo_tri_dub_phi_inf(const double* verts9, const double* poi);
/* bodyPanel::panelVInf, CPanel/bodyPanel.cpp:305-348 */
void    cpo_tri_v_inf(const double* verts9, const double* poi, double* v_src, double* v_dub);

/* panel::dubVInf, CPanel/panel.cpp:666-704 (doublet-only velocity of a wake triangle) */
void    cpo_tri_dub_v_inf(const double* verts9, const double* poi, double* v_dub);
/* Panel-induced velocity at m points (the panel terms of cpCaseVP::velocityInflFromEverything,
 * CPanel/cpCaseVP.cpp:713-731): sum over body triangles of sigma*vSrc + mu*vDub
 * (bodyPanel::panelV) then over wake triangles of mu_w*dubVInf (wakePanel::panelV). */
void    cpo_panels_velocity(const double* bverts, const double* sigma, const double* mu, int64_t nb,
                            const double* wverts, const double* wmu, int64_t nw, const double* pts,
                            int64_t m, double* vel, int nthreads);

/* ---- assembly: geometry::setInfCoeff, CPanel/geometry.cpp:809-891 ----
 * Rows [r0, r1) of A and B (full matrix: r0 = 0, r1 = n), stored column-major with
 * leading dimension r1 - r0: A(i,j) = A[j*(r1-r0) + (i-r0)].  nthreads >= 1. */
void    cpo_set_inf_coeff(void* m, double* A, double* B, int64_t r0, int64_t r1, int nthreads);

/* ---- steady case: cpCase::run minus I/O, CPanel/cpCase.cpp:31-139 ---- */
typedef struct {
    double V, alpha, beta, mach, Sref, bref, cref, cg[3];
} cpo_case_params;
typedef struct {
    double CL, CDi;            /* Trefftz plane, CPanel/cpCase.cpp:541-552 */
    double Fbody[3], Fwind[3], CM[3];
    int64_t iters;             /* BiCGSTAB iterations */
    double  error;             /* BiCGSTAB relative residual */
    int     converged;
} cpo_case_result;

/* sigma = -Vinf.n ; rhs = -B sigma ; BiCGSTAB (Eigen semantics) ; mu, phi ;
 * velocity by CHTLS ; Cp ; forces ; Trefftz.  Any output pointer may be null. */
int     cpo_case_run(void* m, const double* A, const double* B, const cpo_case_params* p,
                     double* sigma, double* mu, double* phi, double* vel, double* cp,
                     double* wake_mu, cpo_case_result* res, int nthreads);
/* The spanwise Trefftz-plane loads of the last cpo_case_run / cpo_case_post on m, for live wake
 * `wake`: 2y/b, Cl / PG and Cdi / PG^2 at the reference's 165 stations (cpCase::writeSpanwiseData,
 * CPanel/cpCase.cpp:910-935; wake::trefftzPlane, wake.cpp:146-188).  Returns the station count or -1. */
int     cpo_spanwise(void* m, int wake, double* y2b, double* cl, double* cdi);
/* Post-processing only, from a given mu (used to isolate solver differences). */
int     cpo_case_post(void* m, const cpo_case_params* p, const double* mu,
                      double* phi, double* vel, double* cp, cpo_case_result* res);

/* Dense BiCGSTAB with Jacobi preconditioner, Eigen 3.3 semantics
 * (Eigen/src/IterativeLinearSolvers/BiCGSTAB.h; called at CPanel/cpCase.cpp:196-201). */
int     cpo_bicgstab(const double* A, int64_t n, const double* b, double* x, double tol,
                     int64_t max_iters, int64_t* iters, double* err, int nthreads);

}  /* extern "C" */
