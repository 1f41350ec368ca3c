/*
 * cpanel_io.h -- CPanel's result files from this library's results (host only, no device).
 *
 * Reference interfaces replaced (paths relative to the CPanel project root):
 *   cpg_write_cpout         caseMgr::writeSummary / writeCase, CPanel/CPanelMgr.cpp:89-180, with the
 *                           input echo of inputParams::print, CPanel/inputParams.cpp:227-318
 *   cpg_write_surface_vtu   cpCase::writeBodyData, CPanel/cpCase.cpp:711-763, through
 *                           VTUfile::write, CPanel/VTUfile.cpp:20-147
 *   cpg_write_wake_vtu      cpCase::writeWakeData, CPanel/cpCase.cpp:883-907
 *   cpg_write_volume_vtu    cpCase::writeVolMeshData, CPanel/cpCase.cpp:979-1004
 *   cpg_write_streamlines_vtu  cpCase::writeBodyStreamlines, CPanel/cpCase.cpp:937-977
 *   cpg_write_spanwise_csv  cpCase::writeSpanwiseData, CPanel/cpCase.cpp:910-935
 *
 * The text follows the reference's layout and stream formatting (the same column widths,
 * precisions and array names), so the files diff against CPanel's own.  One difference is
 * unavoidable: the reference numbers nodes after sorting node pointers (geometry.cpp:405-406),
 * which varies from run to run; here nodes keep their .tri file order.
 */
#ifndef CPANEL_IO_H
#define CPANEL_IO_H

#include <stdint.h>

#include "cpanel_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The input echo of a .CPout file (what the reference reads from its .CPin). */
typedef struct {
    const char* geom_file;
    double Sref, bref, cref, cg[3];
    const double* velocities;
    int n_velocities;
    const double* alphas;
    int n_alphas;
    const double* betas;
    int n_betas;
    const double* machs;
    int n_machs;
    int subsonic_hom, surface_streamlines, stability_derivatives, write_inf_coeff, vortex_particles,
        accelerate_code, unsteady; /* printed ON (non-zero) or OFF */
} cpg_cpout_inputs;

/* One case of a .CPout file: the coefficient vectors as cpCase returns them. */
typedef struct {
    cpg_flow flow;    /* V, alpha, beta, mach                                           */
    double CL, CDi;   /* Trefftz plane                                                  */
    double Fbody[3];  /* body-axis force coefficients (x, y, z): printed CN, CA, CY     */
    double Fwind[3];  /* wind-axis force coefficients (x, y, z): printed CL, CD, CY     */
    double CM[3];     /* moment coefficients (roll, pitch, yaw): printed Cm, Cl, Cn     */
    int has_stability;          /* non-zero: print the stability derivatives block       */
    cpg_stability stability;    /* as cpg_stability_derivatives gives them               */
} cpg_cpout_case;

/* Write the .CPout summary of n_cases cases. */
int cpg_write_cpout(const char* path, const cpg_cpout_inputs* inputs, const cpg_cpout_case* cases, int n_cases);

/* Write surfaceData.vtu for one case: nodes n_nodes x 3; tris n x 3 zero-based node indices of
 * the body panels in matrix order; per body panel mu, sigma, phi, cp (n), vel, bez, centers
 * (n x 3).  Cell arrays as the reference names them ("Doublet Strengths", "Source Strengths",
 * "Velocity Potential", "Velocity", "Cp", "bezNormals", "xPosition", "yPosition",
 * "zPostition"). */
int cpg_write_surface_vtu(const char* path, const double* nodes, int64_t n_nodes, const int64_t* tris, int64_t n,
                          const double* mu, const double* sigma, const double* phi, const double* vel,
                          const double* cp, const double* bez, const double* centers);

/* Write wakeData.vtu (cpCase::writeWakeData, CPanel/cpCase.cpp:883-907): tris n_wake x 3 zero-based
 * node indices of the wake panels in wPanels order; per wake panel mu and phi (the reference's
 * "Doublet Strengths" and "Velocity Potential"). */
int cpg_write_wake_vtu(const char* path, const double* nodes, int64_t n_nodes, const int64_t* tris, int64_t n_wake,
                       const double* mu, const double* phi);

/* Write volumeMesh.vtu (cpCase::writeVolMeshData, CPanel/cpCase.cpp:979-1004): points n_points x 3,
 * cells n_cells x 8 zero-based point indices (VTK voxels, the order cpCase::createVolMesh uses),
 * per cell vel (n_cells x 3) and cp (n_cells). */
int cpg_write_volume_vtu(const char* path, const double* points, int64_t n_points, const int64_t* cells,
                         int64_t n_cells, const double* vel, const double* cp);

/* Write streamlines.vtu (cpCase::writeBodyStreamlines, CPanel/cpCase.cpp:937-977; the same layout as the
 * reference's commented-out off-body writer): one piece per line, its points with point data "Velocity"
 * and line cells (j, j + 1).  pts, vel, counts are cpg_streamlines' outputs (n_lines x max_points x 3;
 * the first counts[i] rows of line i are written). */
int cpg_write_streamlines_vtu(const char* path, const double* pts, const double* vel, const int32_t* counts,
                              int n_lines, int max_points);

/* Write spanwiseData_Wake<i>.csv (cpCase::writeSpanwiseData, CPanel/cpCase.cpp:910-935): the header
 * "2y/b,Cl,Cdi", then n rows "y2b,cl,cdi" in the stream's default format; the columns are
 * cpg_spanwise_loads' outputs. */
int cpg_write_spanwise_csv(const char* path, const double* y2b, const double* cl, const double* cdi, int n);

#ifdef __cplusplus
}
#endif
#endif /* CPANEL_IO_H */
