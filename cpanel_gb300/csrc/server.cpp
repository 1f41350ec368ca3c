// Request loop (include/cpanel_serve.h): steady and unsteady (vortex-particle) requests
// on a pool of slots, each with its own context,
// taking queued requests in arrival order whenever a slot is idle and the request fits
// in the free memory budget (a later, smaller request may start ahead of an earlier one
// that does not fit yet).
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cpanel_gpu.h"
#include "../../include/cpanel_serve.h"
#include "../../include/cpanel_vp.h"
#include "assemble.h"
#include "vpgeom.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    std::vector<double> nodes;
    std::vector<int64_t> tris;
    std::vector<int32_t> ids;
    std::vector<cpg_flow> flows;
    cpg_refs refs{};
    int64_t n_body = 0;
    int64_t footprint = 0;
    Clock::time_point t_submit, t_start, t_done;
    int running_at_start = 0;
    bool done = false;
    int status = CPG_OK;
    std::string message;
    std::vector<double> cp, CL, CDi;
    // unsteady request
    bool vp = false;
    cpg_vp_params vprm{};
    int nsteps = 0;
    cpg_vp_result vres{};
    std::vector<double> mu;
};

double ms(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct cpg_server {
    cpg_server_params p{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<int64_t, std::shared_ptr<Request>> all;
    std::vector<std::thread> workers;
    int64_t next_id = 1;
    double used = 0;
    int running = 0;
    bool stop = false;
    int init_status = CPG_OK;
    int ready = 0;
};

namespace {

void run_request(cpg_ctx* ctx, int precision, Request& r) {
    cpg_geometry* g = nullptr;
    int rc = cpg_geometry_create(ctx, r.nodes.data(), (int64_t)r.nodes.size() / 3, r.tris.data(), r.ids.data(),
                                 (int64_t)r.ids.size(), &g);
    if (rc == CPG_OK) rc = cpg_set_inf_coeff(g, precision);
    if (rc == CPG_OK) {
        cpg_geometry_info gi;
        cpg_geometry_info_get(g, &gi);
        const int k = (int)r.flows.size();
        r.n_body = gi.n_body;
        r.cp.assign((size_t)k * gi.n_body, 0.0);
        r.CL.assign(k, 0.0);
        r.CDi.assign(k, 0.0);
        cpg_case_out out{};
        out.cp = r.cp.data();
        out.CL = r.CL.data();
        out.CDi = r.CDi.data();
        cpg_solve_stats st;
        std::vector<cpg_refs> refs(k, r.refs);
        rc = cpg_solve_cases(g, r.flows.data(), k, refs.data(), precision, &out, &st);
    }
    if (rc != CPG_OK) r.message = cpg_last_error(ctx);
    r.status = rc;
    if (g) cpg_geometry_destroy(g);
    cpg_release_spares(ctx);  // admission counts only the running requests' memory
}

void run_request_vp(cpg_ctx* ctx, Request& r) {
    cpg_vpcase* c = nullptr;
    int rc = cpg_vpcase_create(ctx, r.nodes.data(), (int64_t)r.nodes.size() / 3, r.tris.data(), r.ids.data(),
                               (int64_t)r.ids.size(), &r.vprm, &c);
    if (rc == CPG_OK) rc = cpg_vpcase_step(c, r.nsteps);
    if (rc == CPG_OK) rc = cpg_vpcase_trefftz(c, &r.vres.CL, &r.vres.CD, &r.vres.converged);
    if (rc == CPG_OK) {
        cpg_vp_info vi;
        cpg_vpcase_info_get(c, &vi);
        r.vres.steps = vi.timestep;
        r.vres.n_particles = vi.n_particles;
        r.n_body = vi.n_body;
        r.mu.assign(vi.n_body, 0.0);
        rc = cpg_vpcase_strengths(c, nullptr, r.mu.data(), nullptr, nullptr);
    }
    if (rc != CPG_OK) r.message = cpg_last_error(ctx);
    r.status = rc;
    if (c) cpg_vpcase_destroy(c);
}

void worker(cpg_server* S) {
    cpg_ctx* ctx = nullptr;
    int rc = cpg_create(&ctx, S->p.device);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (rc != CPG_OK) S->init_status = rc;
        S->ready++;
    }
    S->cv_done.notify_all();
    if (rc != CPG_OK) return;
    for (;;) {
        std::shared_ptr<Request> r;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                if (S->stop) break;
                for (auto it = S->queue.begin(); it != S->queue.end(); ++it)
                    if ((*it)->footprint <= S->p.budget_bytes - S->used) {
                        r = *it;
                        S->queue.erase(it);
                        break;
                    }
                if (r) break;
                S->cv_work.wait(lk);
            }
            if (!r) break;
            S->used += (double)r->footprint;
            S->running++;
            r->running_at_start = S->running;
            r->t_start = Clock::now();
        }
        if (r->vp)
            run_request_vp(ctx, *r);
        else
            run_request(ctx, S->p.precision, *r);
        {
            std::lock_guard<std::mutex> lk(S->mu);
            r->t_done = Clock::now();
            r->done = true;
            S->used -= (double)r->footprint;
            S->running--;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
    cpg_destroy(ctx);
}

}  // namespace

namespace {
// blocks until request `ticket` is done and takes it out of the table
std::shared_ptr<Request> take_done(cpg_server* S, int64_t ticket) {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) return nullptr;
    std::shared_ptr<Request> r = it->second;
    S->cv_done.wait(lk, [&] { return r->done || S->stop; });
    if (!r->done) return nullptr;
    S->all.erase(ticket);
    return r;
}

void fill_info(const Request& r, cpg_request_info* info) {
    if (!info) return;
    info->status = r.status;
    info->n_body = r.n_body;
    info->k = (int)r.flows.size();
    info->footprint_bytes = r.footprint;
    info->queue_ms = ms(r.t_submit, r.t_start);
    info->run_ms = ms(r.t_start, r.t_done);
    info->total_ms = ms(r.t_submit, r.t_done);
    info->running_at_start = r.running_at_start;
    std::snprintf(info->message, sizeof(info->message), "%s", r.message.c_str());
}
}  // namespace

extern "C" {

int64_t cpg_server_footprint(int64_t n, int k, int precision) {
    // matrices and factors, per-case vectors, the CHTLS/Trefftz tables, the factorization's
    // diagonal-block inverses, split tensor-core operands and scratch (lu_factor_bytes), with a
    // fixed margin
    const int64_t nn = n * n;
    // (mixed: also the assembly's per-chunk partial sums of the right-hand-side basis)
    int64_t mats = precision == CPG_PLAIN_FP64
                       ? 16 * nn
                       : 12 * nn + (int64_t)cpg::lu_factor_bytes(n) + 8 * (3 * n + cpg::mixed_rb_part_doubles(n, 0));
    return mats + (int64_t)n * (int64_t)(2000 + 64 * k) + ((int64_t)64 << 20);
}

int64_t cpg_server_footprint_vp(int64_t n, int64_t n2, int nsteps, int precision) {
    // A and B (FP64), C; for CPG_MIXED the float pair of A, its LU, inverse and the inversion's
    // n x n scratch, and the factorization's own buffers (lu_factor_bytes); per particle its
    // state, tree slot, step scratch and the panel kernels' partial sums
    const int64_t nn = n * n;
    int64_t mats = 16 * nn + 8 * n * n2;
    if (precision == CPG_MIXED) mats += 20 * nn + (int64_t)cpg::lu_factor_bytes(n);
    const int64_t np = n2 * (int64_t)(nsteps > 0 ? nsteps : 0);
    return mats + n * 4000 + np * 4096 + ((int64_t)64 << 20);
}

int cpg_server_create(const cpg_server_params* p, cpg_server** out) {
    if (!p || !out || p->slots < 1 || p->slots > 64 || !(p->budget_bytes > 0)) return CPG_E_INVALID;
    if (p->precision != CPG_MIXED && p->precision != CPG_PLAIN_FP64) return CPG_E_INVALID;
    *out = nullptr;
    cpg_server* S = new (std::nothrow) cpg_server();
    if (!S) return CPG_E_OOM;
    S->p = *p;
    for (int i = 0; i < p->slots; i++) S->workers.emplace_back(worker, S);
    {
        std::unique_lock<std::mutex> lk(S->mu);
        S->cv_done.wait(lk, [&] { return S->ready == p->slots; });
    }
    if (S->init_status != CPG_OK) {
        int rc = S->init_status;
        cpg_server_destroy(S);
        return rc;
    }
    *out = S;
    return CPG_OK;
}

void cpg_server_destroy(cpg_server* S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->queue.clear();
    }
    S->cv_work.notify_all();
    for (auto& t : S->workers) t.join();
    delete S;
}

int cpg_server_submit(cpg_server* S, const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                      int64_t n_tris, const cpg_flow* flows, int k, const cpg_refs* refs, int64_t* ticket) {
    if (!S || !nodes || !tris || !ids || !flows || !refs || !ticket || n_nodes <= 0 || n_tris <= 0 || k < 1)
        return CPG_E_INVALID;
    auto r = std::make_shared<Request>();
    r->nodes.assign(nodes, nodes + 3 * n_nodes);
    r->tris.assign(tris, tris + 3 * n_tris);
    r->ids.assign(ids, ids + n_tris);
    r->flows.assign(flows, flows + k);
    r->refs = *refs;
    int64_t nb = 0;
    for (int64_t i = 0; i < n_tris; i++) nb += ids[i] <= 1000 ? 1 : 0;
    r->n_body = nb;
    r->footprint = cpg_server_footprint(nb, k, S->p.precision);
    if ((double)r->footprint > S->p.budget_bytes) return CPG_E_OOM;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->id = S->next_id++;
        S->all[r->id] = r;
        S->queue.push_back(r);
        *ticket = r->id;
    }
    S->cv_work.notify_one();
    return CPG_OK;
}

int cpg_server_submit_vp(cpg_server* S, const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                         int64_t n_tris, const cpg_vp_params* prm, int nsteps, int64_t* ticket) {
    if (!S || !nodes || !tris || !ids || !prm || !ticket || n_nodes <= 0 || n_tris <= 0 || nsteps < 0)
        return CPG_E_INVALID;
    // the buffer wake's size sets the particle count: build it on the host now (this also
    // rejects a mesh the case cannot take before it is queued)
    cpg::VPGeom G;
    if (!cpg::build_vp_geometry(nodes, n_nodes, tris, ids, n_tris, prm->V, prm->dt, G).empty()) return CPG_E_BAD_MESH;
    auto r = std::make_shared<Request>();
    r->vp = true;
    r->nodes.assign(nodes, nodes + 3 * n_nodes);
    r->tris.assign(tris, tris + 3 * n_tris);
    r->ids.assign(ids, ids + n_tris);
    r->vprm = *prm;
    r->nsteps = nsteps;
    r->n_body = G.n_body;
    r->footprint = cpg_server_footprint_vp(G.n_body, G.n_w2, nsteps, prm->precision);
    if ((double)r->footprint > S->p.budget_bytes) return CPG_E_OOM;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->id = S->next_id++;
        S->all[r->id] = r;
        S->queue.push_back(r);
        *ticket = r->id;
    }
    S->cv_work.notify_one();
    return CPG_OK;
}


int cpg_server_wait_vp(cpg_server* S, int64_t ticket, cpg_vp_result* res, double* mu, cpg_request_info* info) {
    if (!S) return CPG_E_INVALID;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->all.find(ticket);
        if (it == S->all.end() || !it->second->vp) return CPG_E_INVALID;
    }
    std::shared_ptr<Request> r = take_done(S, ticket);
    if (!r) return CPG_E_INVALID;
    if (res) *res = r->vres;
    if (mu && !r->mu.empty()) std::memcpy(mu, r->mu.data(), sizeof(double) * r->mu.size());
    fill_info(*r, info);
    return r->status;
}

int cpg_server_wait(cpg_server* S, int64_t ticket, double* cp, double* CL, double* CDi, cpg_request_info* info) {
    if (!S) return CPG_E_INVALID;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->all.find(ticket);
        if (it == S->all.end() || it->second->vp) return CPG_E_INVALID;
    }
    std::shared_ptr<Request> r = take_done(S, ticket);
    if (!r) return CPG_E_INVALID;
    if (cp && !r->cp.empty()) std::memcpy(cp, r->cp.data(), sizeof(double) * r->cp.size());
    if (CL && !r->CL.empty()) std::memcpy(CL, r->CL.data(), sizeof(double) * r->CL.size());
    if (CDi && !r->CDi.empty()) std::memcpy(CDi, r->CDi.data(), sizeof(double) * r->CDi.size());
    fill_info(*r, info);
    return r->status;
}

}  // extern "C"
