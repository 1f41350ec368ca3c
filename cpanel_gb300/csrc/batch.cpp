// Batch solve of many uneven meshes (include/cpanel_batch.h).
//
// The reference solves one mesh per process: geometry::readTri builds the topology and
// calls setInfCoeff (CPanel/geometry.cpp:607-621), then CPanelMgr::run runs cpCase::run
// once per flow condition (CPanel/CPanelMgr.cpp:90-167, CPanel/cpCase.cpp:31-139).
// Here m meshes run together on one GPU:
//   1. topology, uploads and the post-processing tables (CHTLS weights, Trefftz operator)
//      on worker threads, one context (stream, cuBLAS handle) each, the meshes dealt out
//      costliest first to the least loaded worker;
//   2. one grouped, persistent mixed-precision assembly per wave of meshes that fits the
//      memory budget (cpg_set_inf_coeff_grouped);
//   3. either each mesh's FP32 LU, refined solves and post-processing (cpg_solve_cases) on
//      its worker's stream, the workers side by side; or (lockstep) the wave's
//      factorizations together (cpg_lu_factor_grouped: one diagonal-block launch per block
//      step for every mesh), then the wave's refined solves together (one launch per
//      substitution block step for every mesh) and each mesh's post-processing;
//   4. the wave's device memory released once every worker of the wave is done (a
//      cudaFree synchronizes the device, so none runs while other workers compute).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <new>
#include <stdexcept>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cpanel_batch.h"
#include "../../include/cpanel_serve.h"

namespace cpg {
int ctx_workers(cpg_ctx* ctx, int w, std::vector<cpg_ctx*>& out);
int geometry_prepare_post(cpg_geometry* g);
int solve_cases_grouped(cpg_geometry* const* gs, int m, const cpg_flow* const* flows, const int* ks,
                        const cpg_refs* refs, const cpg_case_out* outs, int* status);
int ctx_device(cpg_ctx* ctx);
void ctx_set_error(cpg_ctx* ctx, const std::string& msg);
}  // namespace cpg

namespace {

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// runs fn(w) on one host thread per worker, each with the device current; if a thread
// cannot be started, the started ones are joined and the error is passed on
template <typename F>
void on_workers(int W, int device, F fn) {
    std::vector<std::thread> th;
    th.reserve(W);
    try {
        for (int w = 0; w < W; w++)
            th.emplace_back([&, w] {
                cudaSetDevice(device);
                fn(w);
            });
    } catch (...) {
        for (auto& t : th) t.join();
        throw;
    }
    for (auto& t : th) t.join();
}

}  // namespace

static int batch_solve_impl(cpg_ctx* ctx, cpg_batch_mesh* M, int m, const cpg_batch_params* p,
                            cpg_batch_stats* st) {
    if (!ctx || !M || m <= 0) return CPG_E_INVALID;
    const auto T0 = std::chrono::steady_clock::now();
    int W = (p && p->workers > 0) ? p->workers : 8;
    W = std::max(1, std::min({W, m, 64}));
    const int tune = p ? p->tune : CPG_TUNE_AUTO;
    const bool lockstep = p && p->lockstep != 0;
    if (tune < CPG_TUNE_OFF || tune > CPG_TUNE_FORCE) {
        cpg::ctx_set_error(ctx, "unknown tune mode");
        return CPG_E_INVALID;
    }
    for (int i = 0; i < m; i++) {
        M[i].status = CPG_OK;
        M[i].n_body = 0;
        if (!M[i].nodes || !M[i].tris || !M[i].ids || !M[i].flows || M[i].k < 1 || M[i].k > 4096) {
            cpg::ctx_set_error(ctx, "batch mesh " + std::to_string(i) + ": bad argument");
            return CPG_E_INVALID;
        }
    }
    const int device = cpg::ctx_device(ctx);
    std::vector<cpg_ctx*> wk;
    int rc = cpg::ctx_workers(ctx, W, wk);
    if (rc != CPG_OK) {
        cpg::ctx_set_error(ctx, "worker contexts could not be created");
        return rc;
    }
    // costliest first (assembly and LU grow with n^2 and n^3; n_tris stands in for n)
    std::vector<int> order(m);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return M[a].n_tris > M[b].n_tris; });
    std::vector<int> owner(m, 0);
    std::vector<double> load(W, 0.0);
    for (int i : order) {
        int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        owner[i] = w;
        const double n = (double)M[i].n_tris;
        load[w] += n * n * (1.0 + n / 4000.0);
    }
    // 1. topology and uploads
    std::vector<cpg_geometry*> g(m, nullptr);
    on_workers(W, device, [&](int w) {
        for (int i : order) {
            if (owner[i] != w) continue;
            cpg_geometry* gi = nullptr;
            int r = cpg_geometry_create(wk[w], M[i].nodes, M[i].n_nodes, M[i].tris, M[i].ids, M[i].n_tris, &gi);
            M[i].status = r;
            if (r == CPG_OK) {
                cpg_geometry_info info;
                cpg_geometry_info_get(gi, &info);
                M[i].n_body = info.n_body;
                g[i] = gi;
                // CHTLS weights and the Trefftz operator on the worker's second stream,
                // beside the grouped assembly
                M[i].status = r = cpg::geometry_prepare_post(gi);
                if (r != CPG_OK) {
                    cpg_geometry_destroy(gi);
                    g[i] = nullptr;
                }
            }
        }
    });
    const double ms_topology = ms_since(T0);
    // 2. waves by the memory budget (the request loop's footprint rule)
    double budget = p ? p->budget_bytes : 0.0;
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        cudaSetDevice(device);
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            for (int i = 0; i < m; i++) cpg_geometry_destroy(g[i]);
            cpg::ctx_set_error(ctx, "cudaMemGetInfo failed");
            return CPG_E_CUDA;
        }
        budget = 0.75 * (double)fr;
    }
    std::vector<std::vector<int>> waves;
    double used = 0;
    for (int i : order) {
        if (!g[i]) continue;
        const double fp = (double)cpg_server_footprint(M[i].n_body, M[i].k, CPG_MIXED);
        if (waves.empty() || (used + fp > budget && !waves.back().empty())) {
            waves.emplace_back();
            used = 0;
        }
        waves.back().push_back(i);
        used += fp;
    }
    double ms_assembly = 0, ms_factor = 0, ms_solve = 0;
    cpg_group_report last{};
    for (const std::vector<int>& wave : waves) {
        if (&wave != &waves.front())  // the previous wave's matrices: this wave was sized by the budget
            for (cpg_ctx* w : wk) cpg_release_spares(w);
        std::vector<cpg_geometry*> gs;
        for (int i : wave) gs.push_back(g[i]);
        cpg_group_report rep{};
        int r = cpg_set_inf_coeff_grouped(gs.data(), (int)gs.size(), tune, nullptr, &rep);
        if (r != CPG_OK) {
            for (int i : wave) M[i].status = r;
        } else {
            ms_assembly += rep.ms;
            last = rep;
            if (lockstep) {  // the wave's factorizations and refined solves in lockstep
                double fms = 0;
                r = cpg_lu_factor_grouped(gs.data(), (int)gs.size(), &fms);
                ms_factor += fms;
                if (r != CPG_OK)
                    for (int i : wave) M[i].status = r;
            }
        }
        if (r == CPG_OK && lockstep) {
            const auto T1 = std::chrono::steady_clock::now();
            std::vector<const cpg_flow*> fl;
            std::vector<int> ks, stv(wave.size(), CPG_OK);
            std::vector<cpg_refs> rf;
            std::vector<cpg_case_out> outs(wave.size());
            for (size_t j = 0; j < wave.size(); j++) {
                const cpg_batch_mesh& b = M[wave[j]];
                fl.push_back(b.flows);
                ks.push_back(b.k);
                rf.push_back(b.refs);
                outs[j] = cpg_case_out{};
                outs[j].mu = b.mu;
                outs[j].cp = b.cp;
                outs[j].CL = b.CL;
                outs[j].CDi = b.CDi;
            }
            const int rs = cpg::solve_cases_grouped(gs.data(), (int)gs.size(), fl.data(), ks.data(), rf.data(),
                                                    outs.data(), stv.data());
            for (size_t j = 0; j < wave.size(); j++)
                M[wave[j]].status = (rs != CPG_OK && rs != CPG_E_NOT_CONVERGED) ? rs : stv[j];
            ms_solve += ms_since(T1);
        } else if (r == CPG_OK) {
            // 3. factorizations, refined solves and post on the workers
            const auto T1 = std::chrono::steady_clock::now();
            on_workers(W, device, [&](int w) {
                for (int i : wave) {
                    if (owner[i] != w) continue;
                    cpg_case_out out{};
                    out.mu = M[i].mu;
                    out.cp = M[i].cp;
                    out.CL = M[i].CL;
                    out.CDi = M[i].CDi;
                    M[i].status = cpg_solve_cases(g[i], M[i].flows, M[i].k, &M[i].refs, CPG_MIXED, &out, nullptr);
                }
            });
            ms_solve += ms_since(T1);
        }
        // 4. release the wave (every worker has joined)
        for (int i : wave) {
            cpg_geometry_destroy(g[i]);
            g[i] = nullptr;
        }
    }
    int first_bad = CPG_OK, failed = 0;
    int64_t solves = 0;
    for (int i = 0; i < m; i++) {
        if (M[i].status != CPG_OK) {
            failed++;
            if (first_bad == CPG_OK) {
                first_bad = M[i].status;
                cpg::ctx_set_error(ctx, "batch mesh " + std::to_string(i) + " failed with status " +
                                            std::to_string(M[i].status));
            }
        } else {
            solves += M[i].k;
        }
    }
    if (st) {
        st->ms_total = ms_since(T0);
        st->ms_topology = ms_topology;
        st->ms_assembly = ms_assembly;
        st->ms_factor = ms_factor;
        st->ms_solve = ms_solve;
        st->waves = (int)waves.size();
        st->solves = solves;
        st->failed = failed;
        st->group = last;
    }
    return first_bad;
}

extern "C" int cpg_batch_solve(cpg_ctx* ctx, cpg_batch_mesh* M, int m, const cpg_batch_params* p,
                               cpg_batch_stats* st) {
    try {
        return batch_solve_impl(ctx, M, m, p, st);
    } catch (const std::bad_alloc&) {
        cpg::ctx_set_error(ctx, "host allocation failed");
        return CPG_E_OOM;
    } catch (const std::exception& e) {
        cpg::ctx_set_error(ctx, e.what());
        return CPG_E_INVALID;
    }
}
