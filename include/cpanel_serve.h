/*
 * cpanel_serve.h -- request loop of the GB300 panel path: steady solves and unsteady
 * vortex-particle runs of different meshes admitted by device-memory footprint and run
 * concurrently (sm_103a).
 *
 * No counterpart in the reference, which runs one case at a time from its CLI
 * (CPanel/cpanel.cpp, CPanel/CPanelMgr.cpp:90-167).  Each request is what
 * cpCase::run does for one mesh and a list of flow conditions (cpg_solve_cases).
 *
 * Continuous batching: a request that arrives while others are on the GPU starts as
 * soon as a slot and enough of the memory budget are free; it does not wait for the
 * running ones to finish.  Each slot owns a context (stream, cuBLAS handle), so the
 * assembly, factorization and solves of different requests overlap on the device.
 * Results do not depend on what else runs: every kernel's reduction order is fixed.
 */
#ifndef CPANEL_SERVE_H
#define CPANEL_SERVE_H

#include <stdint.h>

#include "cpanel_gpu.h"
#include "cpanel_vp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cpg_server cpg_server;

typedef struct {
    int device;
    int slots;            /* requests in flight at once (one context and stream each)    */
    double budget_bytes;  /* device memory the admitted requests may hold together       */
    int precision;        /* CPG_MIXED or CPG_PLAIN_FP64                                 */
} cpg_server_params;

typedef struct {
    int status;              /* cpg_status of the request                              */
    int64_t n_body;
    int k;                   /* flow conditions (unsteady: 0)                          */
    int64_t footprint_bytes; /* admission estimate                                     */
    double queue_ms;         /* submit -> start (host clock)                           */
    double run_ms;           /* start -> done                                          */
    double total_ms;         /* submit -> done                                         */
    int running_at_start;    /* requests on the GPU when this one started, itself included */
    char message[160];       /* error text when status != CPG_OK                        */
} cpg_request_info;

int  cpg_server_create(const cpg_server_params* params, cpg_server** out);
/* Waits for the running requests; queued ones are dropped. */
void cpg_server_destroy(cpg_server* s);
/* Copies the inputs and queues the request; *ticket identifies it.  A request whose
 * footprint exceeds the whole budget is refused (CPG_E_OOM) at once. */
int  cpg_server_submit(cpg_server* s, const double* nodes, int64_t n_nodes, const int64_t* tris,
                       const int32_t* ids, int64_t n_tris, const cpg_flow* flows, int k, const cpg_refs* refs,
                       int64_t* ticket);
/* Blocks until the request is done, copies its results (cp: k x n_body, CL, CDi: k; any
 * may be null) and releases the ticket.  Returns the request's status. */
int  cpg_server_wait(cpg_server* s, int64_t ticket, double* cp, double* CL, double* CDi, cpg_request_info* info);
/* Device-memory estimate of one request (the admission rule). */
int64_t cpg_server_footprint(int64_t n_body, int k, int precision);

/* Unsteady request: the vortex-particle case of cpg_vpcase_create on this mesh (body
 * panels only), advanced nsteps time steps or until its Trefftz-plane check converges. */
typedef struct {
    double CL, CD;        /* Trefftz plane of the final state                          */
    int64_t steps;        /* time steps taken                                           */
    int64_t n_particles;
    int converged;
} cpg_vp_result;
int  cpg_server_submit_vp(cpg_server* s, const double* nodes, int64_t n_nodes, const int64_t* tris,
                          const int32_t* ids, int64_t n_tris, const cpg_vp_params* params, int nsteps,
                          int64_t* ticket);
/* Blocks until the unsteady request is done; mu (n_body, may be null): the final body
 * doublet strengths.  Returns the request's status. */
int  cpg_server_wait_vp(cpg_server* s, int64_t ticket, cpg_vp_result* result, double* mu, cpg_request_info* info);
/* Device-memory estimate of an unsteady request: n_w2 second-row buffer panels (one
 * particle each per step), nsteps steps. */
int64_t cpg_server_footprint_vp(int64_t n_body, int64_t n_w2, int nsteps, int precision);

#ifdef __cplusplus
}
#endif

#endif /* CPANEL_SERVE_H */
