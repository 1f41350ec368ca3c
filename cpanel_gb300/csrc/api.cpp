// C ABI of the GB300 panel path (include/cpanel_gpu.h).
//
// A cpg_geometry owns its device tables; matrices are assembled lazily per
// precision and kept resident, so further cases on the same mesh reuse them
// (the reference assembles once per geometry too, CPanel/geometry.cpp:607-621).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <map>
#include <mutex>
#include <new>
#include <stdexcept>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/cpanel_batch.h"
#include "../../include/cpanel_gpu.h"
#include "../../include/cpanel_vp.h"
#include "assemble.h"
#include "mesh.h"
#include "streamline.h"
#include "octree.h"
#include "particles.h"
#include "vpkern.h"
#include "post.h"
#include "tc_gemm.h"

struct cpg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaStream_t aux = nullptr;  // per-geometry tables built beside the solve
    std::string err;
    cpg::Prof* prof = nullptr;  // device-time accounting, when enabled
    int particle_precision = CPG_PLAIN_FP64;  // cpg_panels_velocity / cpg_panels_stretching
    std::vector<cpg_ctx*> workers;  // contexts of cpg_batch_solve, created on first use
    // matrix buffers of destroyed geometries, kept for the next geometry of a similar size
    // (no cudaMalloc for it, no device-wide synchronization in cudaFree); ev: recorded on
    // the context's stream when the buffer was parked
    struct Spare {
        void* p;
        size_t bytes;
        cudaEvent_t ev;
    };
    std::vector<Spare> spare;
    // the FP32 factorization state (inverses, split operands, scratch, streams, events) of the last
    // destroyed geometry, taken over by the next geometry's mixed solve instead of allocated again
    cpg::LuGraphs* lu_pool = nullptr;
};

namespace {
// Streams of a context: its own stream one priority level above the lowest, the aux stream (the
// per-geometry post tables, queued beside a solve) at the lowest, so the solve's kernels take the
// SMs first and the tables fill what they leave free.  The LU's own side streams are at the
// highest level.
cudaError_t make_stream(cudaStream_t* s, bool background) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
    const int prio = (background || greatest >= least) ? least : least - 1;
    return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, prio);
}

// installs the context's profiler for the calling thread during one API call
struct ProfInstall {
    cpg::Prof* saved;
    explicit ProfInstall(cpg_ctx* c) : saved(cpg::g_prof) { cpg::g_prof = c ? c->prof : nullptr; }
    ~ProfInstall() { cpg::g_prof = saved; }
};
}  // namespace

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const {
        return (T*)p;
    }
};

// Spare matrix buffers of a context: at most kSpareMax buffers and kSpareBytes bytes.
constexpr size_t kSpareMax = 6;
constexpr size_t kSpareBytes = size_t(16) << 30;

void spare_free_oldest(cpg_ctx* c) {
    auto sp = c->spare.front();
    c->spare.erase(c->spare.begin());
    cudaEventSynchronize(sp.ev);
    cudaEventDestroy(sp.ev);
    cudaFree(sp.p);
}

// hand b's memory to the context's spares (or free it)
void park(cpg_ctx* c, DevBuf& b) {
    if (!b.p) return;
    cudaEvent_t ev = nullptr;
    if (c && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
        cudaEventRecord(ev, c->stream) == cudaSuccess) {
        c->spare.push_back(cpg_ctx::Spare{b.p, b.bytes, ev});
        b.p = nullptr;
        b.bytes = 0;
        size_t tot = 0;
        for (const auto& sp : c->spare) tot += sp.bytes;
        while (!c->spare.empty() && (c->spare.size() > kSpareMax || tot > kSpareBytes)) {
            tot -= c->spare.front().bytes;
            spare_free_oldest(c);
        }
        return;
    }
    if (ev) cudaEventDestroy(ev);
    b.release();
}

// DevBuf::ensure for the matrices: a spare of at least `bytes` (and at most twice that) is
// taken once its last use has finished; otherwise cudaMalloc, after freeing the spares if
// the device is out of memory
cudaError_t ensure_big(cpg_ctx* c, DevBuf& b, size_t bytes) {
    if (bytes <= b.bytes) return cudaSuccess;
    park(c, b);
    int best = -1;
    for (size_t i = 0; i < c->spare.size(); i++) {
        const auto& sp = c->spare[i];
        if (sp.bytes >= bytes && sp.bytes <= 2 * bytes && (best < 0 || sp.bytes < c->spare[best].bytes)) best = (int)i;
    }
    if (best >= 0) {
        auto sp = c->spare[best];
        c->spare.erase(c->spare.begin() + best);
        cudaError_t e = cudaEventSynchronize(sp.ev);
        cudaEventDestroy(sp.ev);
        b.p = sp.p;
        b.bytes = sp.bytes;
        return e;
    }
    cudaError_t e = b.ensure(bytes);
    if (e == cudaErrorMemoryAllocation && !c->spare.empty()) {
        cudaGetLastError();
        while (!c->spare.empty()) spare_free_oldest(c);
        e = b.ensure(bytes);
    }
    return e;
}

constexpr double kPi = 3.14159265358979323846;
// Relative residual at which the mixed path's refinement stops (per right-hand side).
// 1e-10 (two passes) measured Cp errors of 4.9e-6 against the plain path on the 19k
// wing: CHTLS weights of order 1/h amplify the remaining doublet error.  Three passes
// (1e-12) give 3.6e-9.
constexpr double kMixedRefineTol = 1e-12;
constexpr int F_STRIDE_HOST = 64;  // double-float record of the mixed assembly, F_STRIDE in common.cuh

}  // namespace

#ifndef CPG_COMPILED_ARCH
#define CPG_COMPILED_ARCH 103
#endif

struct cpg_geometry {
    cpg_ctx* ctx = nullptr;
    cpg::HostMesh H;
    DevBuf rec, frec, bez, clp, cli, tip, ts, wrec, widx, wcoef, tzst, tzln, tzpts, G, F3, F2, mode;
    DevBuf order;  // block schedule of the mixed assembly
    DevBuf erec;   // FP64 edge constants of the mixed near field
    int64_t order_n = -1;
    DevBuf A64, B64, A32, Alo, rb, count;
    DevBuf LU, bad;
    cpg::LuGraphs graphs;
    bool lu_ready = false;
    DevBuf work, post_work, cases, outs;
    bool have64 = false, have32 = false, post_ready = false;
    cudaEvent_t post_ev = nullptr;  // recorded on the aux stream when the post tables are built
    // the CHTLS weights computed on the host threads while the device assembles (cpg_set_inf_coeff
    // starts it; prepare_post uploads its result, or launches the device kernel when there is none)
    std::future<void> chtls;
    std::vector<double> hF3, hF2;
    std::vector<int32_t> hmode;
    int64_t h2d_bytes = 0;
    int64_t n_near64 = 0, n_near32 = 0;
    cpg::PostTables T;
    float ms_asm = 0;
    // the last cpg_solve_cases whose post-processing left its Trefftz station loads in post_work:
    // its case count, each case's Prandtl-Glauert factor and bref (0 cases: none yet)
    int post_k = 0;
    std::vector<double> post_pg;
    double post_bref = 0;
};

struct cpg_ptree {
    cpg_ctx* ctx = nullptr;
    cpg::ParticleTree T;
    DevBuf nodes, parts, fnodes;
    int precision = CPG_PLAIN_FP64;
};

namespace cpg {
void ctx_set_error(cpg_ctx* ctx, const std::string& msg) {
    if (ctx) ctx->err = msg;
}
cudaStream_t ctx_stream(cpg_ctx* ctx) { return ctx ? ctx->stream : nullptr; }
int ctx_particle_precision(cpg_ctx* ctx) { return ctx ? ctx->particle_precision : CPG_PLAIN_FP64; }
int ctx_device(cpg_ctx* ctx) { return ctx ? ctx->device : 0; }
// the first w worker contexts of ctx (created on first use, destroyed with ctx)
int ctx_workers(cpg_ctx* ctx, int w, std::vector<cpg_ctx*>& out) {
    while ((int)ctx->workers.size() < w) {
        cpg_ctx* c = nullptr;
        int rc = cpg_create(&c, ctx->device);
        if (rc != CPG_OK) return rc;
        ctx->workers.push_back(c);
    }
    out.assign(ctx->workers.begin(), ctx->workers.begin() + w);
    return CPG_OK;
}
}  // namespace cpg

namespace {

int fail(cpg_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(cpg_ctx* c, cudaError_t e, const char* where) {
    return fail(c, e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA,
                std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(expr, where)                                      \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, where); \
    } while (0)

thread_local int64_t t_h2d = 0;  // bytes uploaded by the current call

template <typename T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = b.ensure(std::max<size_t>(1, v.size() * sizeof(T)));
    if (e != cudaSuccess) return e;
    if (v.empty()) return cudaSuccess;
    t_h2d += (int64_t)(v.size() * sizeof(T));
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

void case_scalars(const cpg_flow& f, const cpg_refs& r, cpg::CaseScalars& cs) {
    // cpCase::windToBody, CPanel/cpCase.cpp:142-165
    double a = f.alpha * (kPi / 180), b = f.beta * (kPi / 180);
    double T[9] = {std::cos(a) * std::cos(b), std::cos(a) * std::sin(b), -std::sin(a),
                   -std::sin(b), std::cos(b), 0,
                   std::sin(a) * std::cos(b), std::sin(a) * std::sin(b), std::cos(a)};
    for (int q = 0; q < 9; q++) cs.T[q] = T[q];
    for (int q = 0; q < 3; q++) cs.Vinf[q] = T[3 * q] * f.V + T[3 * q + 1] * 0 + T[3 * q + 2] * 0;
    cs.V = f.V;
    cs.PG = std::sqrt(1 - std::pow(f.mach, 2));
    cs.Sref = r.Sref;
    cs.bref = r.bref;
    cs.cref = r.cref;
    for (int q = 0; q < 3; q++) cs.cg[q] = r.cg[q];
}

// The post-processing tables (CHTLS weights, Trefftz operator) do not depend on the
// solve, so they are built on the context's aux stream while the main stream assembles,
// factors and solves; launch_post waits for g->post_ev.
int prepare_post(cpg_geometry* g) {
    cpg_ctx* ctx = g->ctx;
    if (g->post_ready) return CPG_OK;
    if (!ctx->aux) CK(make_stream(&ctx->aux, true), "aux stream");
    if (!g->post_ev) CK(cudaEventCreateWithFlags(&g->post_ev, cudaEventDisableTiming), "event");
    cudaStream_t s = ctx->aux;
    const cpg::HostMesh& H = g->H;
    int64_t n = H.n_body;
    CK(g->F3.ensure(sizeof(double) * n * 3 * (cpg::kClMax - 1)), "alloc F3");
    CK(g->F2.ensure(sizeof(double) * n * 2 * (cpg::kClMax - 1)), "alloc F2");
    CK(g->mode.ensure(sizeof(int32_t) * n), "alloc mode");
    bool host_weights = false;
    if (g->chtls.valid()) {  // computed on the host threads beside the assembly: the same bits
        try {
            g->chtls.get();
            host_weights = true;
        } catch (...) {  // a host allocation failed: the device kernel below instead
        }
    }
    if (host_weights) {
        CK(cudaMemcpyAsync(g->F3.p, g->hF3.data(), sizeof(double) * g->hF3.size(), cudaMemcpyHostToDevice, s),
           "upload F3");
        CK(cudaMemcpyAsync(g->F2.p, g->hF2.data(), sizeof(double) * g->hF2.size(), cudaMemcpyHostToDevice, s),
           "upload F2");
        CK(cudaMemcpyAsync(g->mode.p, g->hmode.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s),
           "upload mode");
        CK(cudaStreamSynchronize(s), "upload CHTLS weights");  // the host arrays are freed next
        std::vector<double>().swap(g->hF3);
        std::vector<double>().swap(g->hF2);
        std::vector<int32_t>().swap(g->hmode);
    } else {
        CK(cudaMemsetAsync(g->F2.p, 0, g->F2.bytes, s), "clear F2");
    }
    cpg::PostTables& T = g->T;
    T.n = n;
    T.nw = H.n_wake;
    T.rec = g->rec.as<double>();
    T.bez = g->bez.as<double>();
    T.cl_ptr = g->clp.as<int32_t>();
    T.cl_idx = g->cli.as<int32_t>();
    T.tip = g->tip.as<int32_t>();
    T.tsorder = g->ts.as<int32_t>();
    T.widx = g->widx.as<int32_t>();
    T.wcoef = g->wcoef.as<double>();
    T.F3 = g->F3.as<double>();
    T.F2 = g->F2.as<double>();
    T.mode = g->mode.as<int32_t>();
    // Trefftz tables (uploaded before the kernels below: a pageable copy waits for the
    // work queued before it on its stream)
    std::vector<double> st;
    std::vector<int32_t> ln;
    int nst = 0;
    for (const auto& W : H.trefftz) {
        nst = (int)W.st.size();
        for (const auto& S : W.st) {
            st.push_back(S.y);
            st.push_back(S.interp);
            for (int a = 0; a < 6; a++) st.push_back(S.Fy[a]);
            for (int a = 0; a < 6; a++) st.push_back(S.Fz[a]);
            st.push_back(W.step);
            ln.push_back(S.line_up1);
            ln.push_back(S.line_lo1);
            ln.push_back(S.line_up2);
            ln.push_back(S.line_lo2);
            ln.push_back(S.pt0);
        }
    }
    T.n_wakes = (int)H.trefftz.size();
    T.n_st = nst;
    T.n_pts = (int64_t)H.tz_pts.size() / 3;
    // the host tables first, while the aux stream is idle (a pageable copy returns only when the
    // work queued before it on its stream is done), then the wait for the geometry's uploads and
    // whatever the caller queued before this call
    CK(upload(g->tzst, st, s), "upload Trefftz");
    CK(upload(g->tzln, ln, s), "upload Trefftz");
    CK(upload(g->tzpts, H.tz_pts, s), "upload Trefftz");
    CK(cudaEventRecord(g->post_ev, ctx->stream), "event");
    CK(cudaStreamWaitEvent(s, g->post_ev, 0), "event");
    if (!host_weights) CK(cpg::launch_chtls_weights(T, s), "CHTLS weights");
    CK(g->G.ensure(std::max<size_t>(8, sizeof(double) * T.n_pts * H.n_wake)), "alloc G");
    CK(cpg::launch_wake_potential_op(g->wrec.as<double>(), H.n_wake, g->tzpts.as<double>(), T.n_pts,
                                     g->G.as<double>(), s),
       "Trefftz operator");
    T.tz_station = g->tzst.as<double>();
    T.tz_lines = g->tzln.as<int32_t>();
    T.G = g->G.as<double>();
    CK(cudaEventRecord(g->post_ev, s), "event");
    g->post_ready = true;
    return CPG_OK;
}

}  // namespace

extern "C" {

int cpg_create(cpg_ctx** out, int device) {
    if (!out) return CPG_E_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return CPG_E_NO_DEVICE;
    if (device < 0 || device >= count) return CPG_E_INVALID;
    cpg_ctx* c = new (std::nothrow) cpg_ctx();
    if (!c) return CPG_E_OOM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || make_stream(&c->stream, false) != cudaSuccess) {
        delete c;
        return CPG_E_CUDA;
    }
    c->own_stream = true;
    *out = c;
    return CPG_OK;
}

void cpg_destroy(cpg_ctx* c) {
    if (!c) return;
    for (cpg_ctx* w : c->workers) cpg_destroy(w);
    for (auto& sp : c->spare) {
        cudaEventSynchronize(sp.ev);
        cudaEventDestroy(sp.ev);
        cudaFree(sp.p);
    }
    c->spare.clear();
    delete c->prof;
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->lu_pool) {
        c->lu_pool->release();
        delete c->lu_pool;
    }
    delete c;
}

const char* cpg_last_error(const cpg_ctx* c) { return c ? c->err.c_str() : "null context"; }

int cpg_release_spares(cpg_ctx* c) {
    if (!c) return CPG_E_INVALID;
    while (!c->spare.empty()) spare_free_oldest(c);
    return CPG_OK;
}

int cpg_set_stream(cpg_ctx* ctx, void* stream) {
    if (!ctx) return CPG_E_INVALID;
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    if (!stream) {
        CK(make_stream(&ctx->stream, false), "stream");
        ctx->own_stream = true;
    }
    return CPG_OK;
}

int cpg_synchronize(cpg_ctx* ctx) {
    if (!ctx) return CPG_E_INVALID;
    CK(cudaStreamSynchronize(ctx->stream), "synchronize");
    return CPG_OK;
}

int cpg_geometry_create(cpg_ctx* ctx, const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                        int64_t n_tris, cpg_geometry** out) {
    if (!ctx || !out || !nodes || !tris || !ids) return fail(ctx, CPG_E_INVALID, "null argument");
    *out = nullptr;
    cpg_geometry* g = new (std::nothrow) cpg_geometry();
    if (!g) return fail(ctx, CPG_E_OOM, "host allocation");
    g->ctx = ctx;
    std::string msg = cpg::build_mesh(nodes, n_nodes, tris, ids, n_tris, g->H);
    if (!msg.empty()) {
        delete g;
        return fail(ctx, CPG_E_BAD_MESH, msg);
    }
    const cpg::HostMesh& H = g->H;
    int64_t n = H.n_body;
    if (n < 2) {
        delete g;
        return fail(ctx, CPG_E_BAD_MESH, "fewer than two body panels");
    }
    cudaStream_t s = ctx->stream;
    t_h2d = 0;
    // double-float far-field records: c, n, area as (hi, lo) FP32 pairs, longSide
    std::vector<float> fr(n * F_STRIDE_HOST, 0.f);
    auto split = [](double v, float* hi, float* lo) {
        *hi = (float)v;
        *lo = (float)(v - (double)*hi);
    };
    cpg::host_parallel((size_t)n, [&](unsigned, size_t lo, size_t hi) {
        for (int64_t i = (int64_t)lo; i < (int64_t)hi; i++) {
            const double* r = &H.body[i * cpg::PF_STRIDE];
            float* o = &fr[i * F_STRIDE_HOST];
            for (int q = 0; q < 3; q++) {
                split(r[cpg::PF_C + q], o + q, o + 3 + q);
                split(r[cpg::PF_N + q], o + 6 + q, o + 9 + q);
            }
            split(r[cpg::PF_AREA], o + 12, o + 13);
            o[14] = (float)r[cpg::PF_LONG];
            // exact-formula band: vertices about the centroid, n x s_k, |s_k|, 1/|s_k|
            const double* c = r + cpg::PF_C;
            const double* nv = r + cpg::PF_N;
            for (int k = 0; k < 3; k++) {
                const double* v = r + cpg::PF_V0 + 3 * k;
                const double* w = r + cpg::PF_V0 + 3 * ((k + 1) % 3);
                double sv[3] = {w[0] - v[0], w[1] - v[1], w[2] - v[2]};
                double ns[3] = {nv[1] * sv[2] - nv[2] * sv[1], nv[2] * sv[0] - nv[0] * sv[2], nv[0] * sv[1] - nv[1] * sv[0]};
                double S = std::sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
                for (int q = 0; q < 3; q++) {
                    split(v[q] - c[q], o + 16 + 2 * (3 * k + q), o + 17 + 2 * (3 * k + q));
                    split(ns[q], o + 34 + 2 * (3 * k + q), o + 35 + 2 * (3 * k + q));
                }
                split(S, o + 52 + 2 * k, o + 53 + 2 * k);
                split(1.0 / S, o + 58 + 2 * k, o + 59 + 2 * k);
            }
        }
    });
    // FP64 edge constants of the mixed near field: |s_k|, 1/|s_k|, s_k.m (E_STRIDE = 12 per panel),
    // rounded exactly as the device would form them (no contraction in this file)
    std::vector<double> er(n * 12, 0.0);
    cpg::host_parallel((size_t)n, [&](unsigned, size_t lo, size_t hi) {
        for (int64_t i = (int64_t)lo; i < (int64_t)hi; i++) {
            const double* r = &H.body[i * cpg::PF_STRIDE];
            const double* m = r + cpg::PF_M;
            for (int k = 0; k < 3; k++) {
                const double* v = r + cpg::PF_V0 + 3 * k;
                const double* w = r + cpg::PF_V0 + 3 * ((k + 1) % 3);
                const double sx = w[0] - v[0], sy = w[1] - v[1], sz = w[2] - v[2];
                const double S = std::sqrt(sx * sx + sy * sy + sz * sz);
                er[i * 12 + k] = S;
                er[i * 12 + 3 + k] = 1 / S;
                er[i * 12 + 6 + k] = sx * m[0] + sy * m[1] + sz * m[2];
            }
        }
    });
    cudaError_t e;
    if ((e = upload(g->rec, H.body, s)) != cudaSuccess || (e = upload(g->frec, fr, s)) != cudaSuccess ||
        (e = upload(g->erec, er, s)) != cudaSuccess ||
        (e = upload(g->bez, H.bez, s)) != cudaSuccess || (e = upload(g->clp, H.cl_ptr, s)) != cudaSuccess ||
        (e = upload(g->cli, H.cl_idx, s)) != cudaSuccess || (e = upload(g->tip, H.tip, s)) != cudaSuccess ||
        (e = upload(g->ts, H.tsorder, s)) != cudaSuccess || (e = upload(g->wrec, H.wake, s)) != cudaSuccess ||
        (e = upload(g->widx, H.widx, s)) != cudaSuccess || (e = upload(g->wcoef, H.wcoef, s)) != cudaSuccess ||
        (e = g->count.ensure(64)) != cudaSuccess) {
        cpg_geometry_destroy(g);
        return cuda_fail(ctx, e, "geometry upload");
    }
    g->h2d_bytes = t_h2d;
    *out = g;
    return CPG_OK;
}

void cpg_geometry_destroy(cpg_geometry* g) {
    if (!g) return;
    if (g->chtls.valid()) g->chtls.wait();  // it reads the host mesh
    for (DevBuf* b : {&g->A32, &g->Alo, &g->LU, &g->A64, &g->B64}) park(g->ctx, *b);
    DevBuf* bufs[] = {&g->rec, &g->frec, &g->bez, &g->clp, &g->cli, &g->tip, &g->ts, &g->wrec, &g->widx,
                      &g->wcoef, &g->tzst, &g->tzln, &g->tzpts, &g->G, &g->F3, &g->F2, &g->mode, &g->A64,
                      &g->B64, &g->A32, &g->Alo, &g->rb, &g->LU, &g->bad, &g->count, &g->work, &g->post_work, &g->cases, &g->outs,
                      &g->order, &g->erec};
    // cudaFree synchronizes with outstanding work; the context may already be gone
    for (DevBuf* b : bufs) b->release();
    cpg_ctx* c = g->ctx;
    if (c && g->graphs.dinv && !c->lu_pool) {  // kept for the context's next geometry
        c->lu_pool = new (std::nothrow) cpg::LuGraphs(g->graphs);
        if (c->lu_pool) g->graphs = cpg::LuGraphs();
    }
    g->graphs.release();
    if (g->post_ev) cudaEventDestroy(g->post_ev);
    delete g;
}

int cpg_geometry_info_get(const cpg_geometry* g, cpg_geometry_info* o) {
    if (!g || !o) return CPG_E_INVALID;
    o->n_body = g->H.n_body;
    o->n_wake = g->H.n_wake;
    o->n_wakes = (int64_t)g->H.trefftz.size();
    o->n_wakelines = g->H.n_lines;
    o->n_tip = g->H.n_tip;
    o->n_nodes = g->H.n_nodes;
    o->h2d_bytes = g->h2d_bytes;
    return CPG_OK;
}

int cpg_geometry_tables(const cpg_geometry* g, double* body, double* wake, int32_t* idx4, double* coef,
                        int32_t* clusters) {
    if (!g) return CPG_E_INVALID;
    const cpg::HostMesh& H = g->H;
    for (int64_t i = 0; i < H.n_body && body; i++) {
        const double* r = &H.body[i * cpg::PF_STRIDE];
        double* o = body + 18 * i;
        for (int q = 0; q < 3; q++) {
            o[q] = r[cpg::PF_C + q];
            o[3 + q] = r[cpg::PF_N + q];
            o[6 + q] = r[cpg::PF_L + q];
        }
        o[9] = r[cpg::PF_AREA];
        o[10] = r[cpg::PF_LONG];
        o[11] = H.tip[i];
        o[12] = H.upper[i];
        o[13] = H.lower[i];
        o[14] = H.tsorder[i];
        o[15] = H.surf_id[i];
        o[16] = H.cl_ptr[i + 1] - H.cl_ptr[i];
        o[17] = H.file_tri[i];
    }
    for (int64_t j = 0; j < H.n_wake; j++) {
        const double* r = &H.wake[j * cpg::PF_STRIDE];
        if (wake) {
            double* o = wake + 8 * j;
            for (int q = 0; q < 3; q++) {
                o[q] = r[cpg::PF_C + q];
                o[3 + q] = r[cpg::PF_N + q];
            }
            o[6] = r[cpg::PF_AREA];
            o[7] = r[cpg::PF_LONG];
        }
        if (idx4)
            for (int q = 0; q < 4; q++) idx4[4 * j + q] = H.widx[4 * j + q];
        if (coef) coef[j] = H.wcoef[j];
    }
    if (clusters)
        for (int64_t i = 0; i < H.n_body; i++)
            for (int q = 0; q < 32; q++) {
                int a = H.cl_ptr[i] + q;
                clusters[32 * i + q] = a < H.cl_ptr[i + 1] ? H.cl_idx[a] : -1;
            }
    return CPG_OK;
}

int cpg_topology(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids, int64_t n_tris,
                 cpg_geometry_info* info, double* body, double* wake, int32_t* idx4, double* coef,
                 int32_t* clusters) {
    if (!nodes || !tris || !ids || !info) return CPG_E_INVALID;
    cpg_geometry tmp;
    std::string msg = cpg::build_mesh(nodes, n_nodes, tris, ids, n_tris, tmp.H);
    if (!msg.empty()) return CPG_E_BAD_MESH;
    cpg_geometry_info_get(&tmp, info);
    return cpg_geometry_tables(&tmp, body, wake, idx4, coef, clusters);
}

int cpg_topology_wake_tris(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                           int64_t n_tris, int64_t* wake_tris) {
    if (!nodes || !tris || !ids || !wake_tris) return CPG_E_INVALID;
    cpg_geometry tmp;
    std::string msg = cpg::build_mesh(nodes, n_nodes, tris, ids, n_tris, tmp.H);
    if (!msg.empty()) return CPG_E_BAD_MESH;
    for (size_t j = 0; j < tmp.H.wake_file_tri.size(); j++) wake_tris[j] = tmp.H.wake_file_tri[j];
    return CPG_OK;
}

int cpg_set_inf_coeff(cpg_geometry* g, int precision) {
    if (!g) return CPG_E_INVALID;
    cpg_ctx* ctx = g->ctx;
    ProfInstall pi(ctx);
    cudaStream_t s = ctx->stream;
    int64_t n = g->H.n_body;
    size_t nn = (size_t)n * n;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    CK(cudaMemsetAsync(g->count.p, 0, sizeof(unsigned long long), s), "clear counter");
    CK(cudaEventRecord(e0, s), "event");
    if (precision == CPG_PLAIN_FP64) {
        CK(ensure_big(ctx, g->A64, sizeof(double) * nn), "alloc A (FP64)");
        CK(ensure_big(ctx, g->B64, sizeof(double) * nn), "alloc B (FP64)");
        CK(cpg::launch_assemble_fp64(g->rec.as<double>(), n, g->wrec.as<double>(), g->widx.as<int32_t>(),
                                     g->wcoef.as<double>(), g->H.n_wake, g->A64.as<double>(), g->B64.as<double>(),
                                     g->count.as<unsigned long long>(), s),
           "assembly (FP64)");
        g->have64 = true;
    } else if (precision == CPG_MIXED) {
        CK(ensure_big(g->ctx, g->A32, sizeof(float) * nn), "alloc A (FP32)");
        CK(ensure_big(g->ctx, g->Alo, sizeof(float) * nn), "alloc A low part (FP32)");
        CK(g->rb.ensure(sizeof(double) * (3 * n + cpg::mixed_rb_part_doubles(n, g->H.n_wake))), "alloc rhs basis");
        if (g->order_n != n) {  // block schedule, once per geometry
            std::vector<int> ord;
            cpg::mixed_block_order(n, g->H.body.data() + cpg::PF_C, cpg::PF_STRIDE, g->H.body.data() + cpg::PF_LONG,
                                   cpg::PF_STRIDE, ord);
            CK(upload(g->order, ord, s), "upload block order");
            g->order_n = n;
        }
        CK(cpg::launch_assemble_mixed(g->rec.as<double>(), g->frec.as<float>(), g->erec.as<double>(), n,
                                      g->wrec.as<double>(),
                                      g->widx.as<int32_t>(), g->wcoef.as<double>(), g->H.n_wake, g->order.as<int>(),
                                      g->A32.as<float>(), g->Alo.as<float>(), g->rb.as<double>(), g->rb.as<double>() + 3 * n,
                                      g->count.as<unsigned long long>(), s),
           "assembly (mixed)");
        g->have32 = true;
        g->lu_ready = false;
    } else {
        return fail(ctx, CPG_E_INVALID, "unknown precision");
    }
    CK(cudaEventRecord(e1, s), "event");
    if (!g->post_ready && !g->chtls.valid()) {  // the post tables' CHTLS weights, beside the assembly
        try {
            g->chtls = std::async(std::launch::async, [g] {
                const size_t nb = (size_t)g->H.n_body;
                g->hF3.assign(nb * 3 * (cpg::kClMax - 1), 0.0);
                g->hF2.assign(nb * 2 * (cpg::kClMax - 1), 0.0);
                g->hmode.assign(nb, 0);
                cpg::chtls_weights_host(g->H, g->hF3.data(), g->hF2.data(), g->hmode.data());
            });
        } catch (...) {  // no thread: prepare_post launches the device kernel
        }
    }
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(&cnt, g->count.p, sizeof(cnt), cudaMemcpyDeviceToHost, s), "counter");
    CK(cudaStreamSynchronize(s), "assembly");
    cudaEventElapsedTime(&g->ms_asm, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (precision == CPG_PLAIN_FP64)
        g->n_near64 = (int64_t)cnt;
    else
        g->n_near32 = (int64_t)cnt;
    return CPG_OK;
}

int cpg_get_A(cpg_geometry* g, double* host) {
    if (!g || !host) return CPG_E_INVALID;
    cpg_ctx* ctx = g->ctx;
    size_t nn = (size_t)g->H.n_body * g->H.n_body;
    if (g->have64) {
        CK(cudaMemcpyAsync(host, g->A64.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, ctx->stream), "copy A");
    } else if (g->have32) {
        DevBuf tmp;
        CK(tmp.ensure(sizeof(double) * nn), "alloc");
        CK(cpg::launch_widen(g->A32.as<float>(), g->Alo.as<float>(), tmp.as<double>(), (int64_t)nn, ctx->stream),
           "widen");
        CK(cudaMemcpyAsync(host, tmp.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, ctx->stream), "copy A");
        CK(cudaStreamSynchronize(ctx->stream), "copy A");
        tmp.release();
    } else {
        return fail(ctx, CPG_E_INVALID, "no assembled matrix");
    }
    CK(cudaStreamSynchronize(ctx->stream), "copy A");
    return CPG_OK;
}

int cpg_get_B(cpg_geometry* g, double* host) {
    if (!g || !host) return CPG_E_INVALID;
    cpg_ctx* ctx = g->ctx;
    if (!g->have64) return fail(ctx, CPG_E_INVALID, "B is only stored by the FP64 assembly");
    size_t nn = (size_t)g->H.n_body * g->H.n_body;
    CK(cudaMemcpyAsync(host, g->B64.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, ctx->stream), "copy B");
    CK(cudaStreamSynchronize(ctx->stream), "copy B");
    return CPG_OK;
}

int cpg_solve_cases(cpg_geometry* g, const cpg_flow* flows, int k, const cpg_refs* refs, int precision,
                    const cpg_case_out* out, cpg_solve_stats* stats) {
    if (!g || !flows || !refs || k <= 0) return CPG_E_INVALID;
    cpg_ctx* ctx = g->ctx;
    ProfInstall pi(ctx);
    if (precision != CPG_PLAIN_FP64 && precision != CPG_MIXED) return fail(ctx, CPG_E_INVALID, "unknown precision");
    if (precision == CPG_MIXED && k > 4096) return fail(ctx, CPG_E_INVALID, "too many cases");
    cudaStream_t s = ctx->stream;
    int64_t n = g->H.n_body, nw = g->H.n_wake;
    int rc;
    if ((precision == CPG_PLAIN_FP64 && !g->have64) || (precision == CPG_MIXED && !g->have32))
        if ((rc = cpg_set_inf_coeff(g, precision)) != CPG_OK) return rc;
    float ms_asm = g->ms_asm;
    // the post tables (CHTLS weights, Trefftz operator) of a new geometry go on the aux stream: in the
    // plain path beside the solve; in the mixed path after the factorization, beside the refinement,
    // where they do not take SMs from the factorization's serial diagonal-block chain
    if (precision == CPG_PLAIN_FP64 && (rc = prepare_post(g)) != CPG_OK) return rc;
    std::vector<cpg::CaseScalars> cs(k);
    for (int c = 0; c < k; c++) case_scalars(flows[c], *refs, cs[c]);
    CK(upload(g->cases, cs, s), "upload cases");
    const cpg::CaseScalars* dcs = g->cases.as<cpg::CaseScalars>();
    size_t kn = (size_t)k * n;
    // outputs: mu sigma rhs phi cp (kn each), vel (3kn), forces 9k, tz 2k, wake mu k*nw
    size_t need = sizeof(double) * (8 * kn + 9 * (size_t)k + 2 * (size_t)k + (size_t)k * nw) + 8 * 256;
    CK(g->outs.ensure(need), "alloc outputs");
    double* mu = g->outs.as<double>();
    double* sigma = mu + kn;
    double* rhs = sigma + kn;
    double* phi = rhs + kn;
    double* cp = phi + kn;
    double* vel = cp + kn;
    double* forces = vel + 3 * kn;
    double* tz = forces + 9 * (size_t)k;
    double* wmu = tz + 2 * (size_t)k;
    cpg::SolveStats st;
    cudaEvent_t e0, e1, e2;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    CK(cudaEventCreate(&e2), "event");
    CK(cudaEventRecord(e0, s), "event");
    CK(cpg::launch_sigma(g->rec.as<double>(), n, k, dcs, sigma, s), "sigma");
    if (precision == CPG_PLAIN_FP64) {
        size_t wb = std::max(cpg::solve_fp64_work_bytes(n, k), (size_t)0);
        CK(g->work.ensure(wb), "alloc solver workspace");
        // RHS = -B sigma, CPanel/cpCase.cpp:192
        CK(cpg::gemm_fp64_nk(g->B64.as<double>(), n, k, sigma, rhs, -1.0, g->work.p, s), "rhs");
        CK(cpg::solve_fp64(g->A64.as<double>(), n, k, rhs, mu, g->work.p, 2.220446049250313e-16, 2 * n, &st, s),
           "BiCGSTAB (FP64)");
    } else {
        if (!g->lu_ready && !g->graphs.dinv && ctx->lu_pool) {  // a destroyed geometry's factorization state
            g->graphs = *ctx->lu_pool;
            delete ctx->lu_pool;
            ctx->lu_pool = nullptr;
        }
        if (!g->lu_ready) {  // per-geometry factorization, reused by every case
            CK(ensure_big(g->ctx, g->LU, sizeof(float) * (size_t)n * n), "alloc LU");
            CK(g->bad.ensure(sizeof(int)), "alloc flag");
            CK(cudaMemsetAsync(g->bad.p, 0, sizeof(int), s), "clear flag");
            CK(cudaMemcpyAsync(g->LU.p, g->A32.p, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, s), "copy A");
            CK(cpg::lu_factor_fp32(&g->graphs, g->LU.as<float>(), n, g->bad.as<int>(), s),
               "LU factorization");
            g->lu_ready = true;
        }
        if ((rc = prepare_post(g)) != CPG_OK) return rc;
        size_t wb = cpg::solve_lu_work_bytes(n, k);
        CK(g->work.ensure(wb), "alloc solver workspace");
        CK(cpg::launch_rhs_basis(g->rb.as<double>(), n, k, dcs, rhs, s), "rhs");
        CK(cpg::solve_lu_refined(&g->graphs, g->A32.as<float>(), g->Alo.as<float>(), g->LU.as<float>(), n, k, rhs,
                                 mu, g->work.p, kMixedRefineTol, 16, &st, s),
           "refined solve (mixed)");
    }
    CK(cudaEventRecord(e1, s), "event");
    CK(g->post_work.ensure(cpg::post_work_bytes(g->T, k)), "alloc post workspace");
    CK(cudaStreamWaitEvent(s, g->post_ev, 0), "wait for the post tables");
    g->post_k = 0;
    CK(cpg::launch_post(g->T, k, dcs, mu, phi, vel, cp, forces, tz, wmu, g->post_work.p, s), "post");
    g->post_k = k;
    g->post_pg.resize(k);
    for (int c = 0; c < k; c++) g->post_pg[c] = cs[c].PG;
    g->post_bref = refs->bref;
    CK(cudaEventRecord(e2, s), "event");
    // host outputs
    auto copy = [&](double* dst, const double* src, size_t cnt) -> cudaError_t {
        if (!dst) return cudaSuccess;
        return cudaMemcpyAsync(dst, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s);
    };
    std::vector<double> hf(9 * (size_t)k), ht(2 * (size_t)k);
    if (out) {
        CK(copy(out->mu, mu, kn), "copy mu");
        CK(copy(out->sigma, sigma, kn), "copy sigma");
        CK(copy(out->phi, phi, kn), "copy phi");
        CK(copy(out->vel, vel, 3 * kn), "copy vel");
        CK(copy(out->cp, cp, kn), "copy cp");
    }
    CK(cudaMemcpyAsync(hf.data(), forces, sizeof(double) * 9 * k, cudaMemcpyDeviceToHost, s), "copy forces");
    CK(cudaMemcpyAsync(ht.data(), tz, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, s), "copy CL");
    CK(cudaStreamSynchronize(s), "solve cases");
    if (out) {
        for (int c = 0; c < k; c++) {
            if (out->CL) out->CL[c] = ht[2 * c];
            if (out->CDi) out->CDi[c] = ht[2 * c + 1];
            for (int q = 0; q < 3; q++) {
                if (out->Fbody) out->Fbody[3 * c + q] = hf[9 * c + q];
                if (out->Fwind) out->Fwind[3 * c + q] = hf[9 * c + 3 + q];
                if (out->CM) out->CM[3 * c + q] = hf[9 * c + 6 + q];
            }
        }
    }
    float ms_solve = 0, ms_post = 0;
    cudaEventElapsedTime(&ms_solve, e0, e1);
    cudaEventElapsedTime(&ms_post, e1, e2);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (stats) {
        stats->iters_max = st.iters_max;
        stats->iters_total = st.iters_total;
        stats->refinements = st.refinements;
        stats->residual_max = st.residual_max;
        stats->n_near = precision == CPG_PLAIN_FP64 ? g->n_near64 : g->n_near32;
        stats->n_far = n * n - stats->n_near;
        stats->ms_assemble = ms_asm;
        stats->ms_solve = ms_solve;
        stats->ms_post = ms_post;
    }
    if (st.residual_max > (precision == CPG_PLAIN_FP64 ? 1e-10 : 1e-9))
        return fail(ctx, CPG_E_NOT_CONVERGED, "solver stopped above tolerance");
    return CPG_OK;
}

int cpg_trefftz_wakes(const cpg_geometry* g) { return g ? (int)g->H.trefftz.size() : 0; }

int cpg_spanwise_loads(cpg_geometry* g, int c, int wake, double* y2b, double* cl, double* cdi, int* n) {
    if (!g || !n) return CPG_E_INVALID;
    cpg_ctx* ctx = g->ctx;
    if (g->post_k <= 0) return fail(ctx, CPG_E_INVALID, "no steady case solved on this geometry yet");
    if (c < 0 || c >= g->post_k) return fail(ctx, CPG_E_INVALID, "case index out of range");
    if (wake < 0 || wake >= (int)g->H.trefftz.size()) return fail(ctx, CPG_E_INVALID, "wake index out of range");
    const cpg::TrefftzWake& W = g->H.trefftz[wake];
    const int nst = (int)W.st.size(), m = nst + 2;  // the reference's stations 0..164
    if (*n < m || !y2b || !cl || !cdi) {
        *n = m;
        return fail(ctx, CPG_E_INVALID, "spanwise buffers shorter than the station count");
    }
    std::vector<double> raw(2 * (size_t)nst);
    CK(cudaSetDevice(ctx->device), "device");
    CK(cudaMemcpyAsync(raw.data(), cpg::post_station_loads(g->T, g->post_k, c, wake, g->post_work.p),
                       sizeof(double) * raw.size(), cudaMemcpyDeviceToHost, ctx->stream),
       "copy station loads");
    CK(cudaStreamSynchronize(ctx->stream), "copy station loads");
    // cpCase::writeSpanwiseData (CPanel/cpCase.cpp:915-917) on wake::trefftzPlane's yLoc, Cl and Cd
    // (wake.cpp:153-176): the end stations are yMin and yMax with zero loads
    const double PG = g->post_pg[c], b = g->post_bref;
    for (int i = 0; i < m; i++) {
        const double y = i == 0 ? W.y0 : i == m - 1 ? W.y1 : W.y0 + i * W.step;
        const bool inner = i > 0 && i < m - 1;
        y2b[i] = 2 * y / b;
        cl[i] = (inner ? raw[2 * (i - 1)] : 0.0) / PG;
        cdi[i] = (inner ? raw[2 * (i - 1) + 1] : 0.0) / std::pow(PG, 2);
    }
    *n = m;
    return CPG_OK;
}

// cpCase::velocityAtPoint's device state for one case (CPanel/cpCase.cpp:1007-1021): the packed body
// and wake panel records and the case's strengths, uploaded once by prepare(); eval() then serves
// any number of point batches through the batched panel-velocity kernel.
struct PointField {
    cpg_ctx* ctx = nullptr;
    cudaStream_t s = nullptr;
    int64_t n = 0, nw = 0;
    DevBuf rec, sm, pv, vv;
    ~PointField() {
        rec.release();
        sm.release();
        pv.release();
        vv.release();
    }
    int prepare(cpg_geometry* g, const double* sigma, const double* mu) {
        ctx = g->ctx;
        s = ctx->stream;
        const cpg::HostMesh& H = g->H;
        n = H.n_body;
        nw = H.n_wake;
        // wake doublets implied by the assembly's wake columns (CPanel/wakePanel.cpp:48-100):
        // mu_w = (1 - t)(mu_up1 - mu_lo1) + t (mu_up2 - mu_lo2)
        std::vector<double> wmu(std::max<int64_t>(1, nw), 0.0);
        for (int64_t j = 0; j < nw; j++) {
            const int32_t* ix = &H.widx[4 * j];
            const double t = H.wcoef[j];
            wmu[j] = (1 - t) * (mu[ix[0]] - mu[ix[1]]) + t * (mu[ix[2]] - mu[ix[3]]);
        }
        const size_t R = 24;  // doubles per packed panel record
        CK(rec.ensure(sizeof(double) * R * (size_t)(n + nw)), "alloc records");
        CK(cudaMemcpyAsync(rec.p, g->rec.p, sizeof(double) * R * n, cudaMemcpyDeviceToDevice, s), "records");
        if (nw > 0)
            CK(cudaMemcpyAsync(rec.as<double>() + R * n, g->wrec.p, sizeof(double) * R * nw, cudaMemcpyDeviceToDevice,
                               s),
               "wake records");
        CK(sm.ensure(sizeof(double) * (2 * n + nw)), "alloc strengths");
        CK(cudaMemcpyAsync(sm.as<double>(), sigma, sizeof(double) * n, cudaMemcpyHostToDevice, s), "sigma");
        CK(cudaMemcpyAsync(sm.as<double>() + n, mu, sizeof(double) * n, cudaMemcpyHostToDevice, s), "mu");
        if (nw > 0)
            CK(cudaMemcpyAsync(sm.as<double>() + 2 * n, wmu.data(), sizeof(double) * nw, cudaMemcpyHostToDevice, s),
               "wake mu");
        CK(cudaStreamSynchronize(s), "point field");  // wmu is a local: its copy has to finish here
        return CPG_OK;
    }
    int eval(const double* pts, int64_t m, double* vel) {
        if (m <= 0) return CPG_OK;
        CK(pv.ensure(sizeof(double) * 3 * m), "alloc points");
        CK(vv.ensure(sizeof(double) * 3 * m), "alloc velocities");
        CK(cudaMemcpyAsync(pv.p, pts, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, s), "points");
        {
            cpg::ProfScope ps(cpg::Prof::POST, s);
            CK(cpg::launch_panels_velocity_rec(rec.as<double>(), sm.as<double>(), sm.as<double>() + n, n,
                                               sm.as<double>() + 2 * n, nw, pv.as<double>(), m, vv.as<double>(), s),
               "panel velocities");
        }
        CK(cudaMemcpyAsync(vel, vv.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, s), "velocities");
        CK(cudaStreamSynchronize(s), "volume velocity");
        return CPG_OK;
    }
};

int cpg_volume_velocity(cpg_geometry* g, const double* sigma, const double* mu, const double* pts, int64_t m,
                        double* vel) {
    if (!g || !sigma || !mu || (m > 0 && (!pts || !vel)) || m < 0) return CPG_E_INVALID;
    if (m == 0) return CPG_OK;
    ProfInstall pi(g->ctx);
    PointField f;
    int rc = f.prepare(g, sigma, mu);
    return rc != CPG_OK ? rc : f.eval(pts, m, vel);
}

int cpg_streamlines(cpg_geometry* g, const double* sigma, const double* mu, const cpg_flow* flow,
                    const double* starts, int n_lines, double x_max, double tol, int max_points, double* pts,
                    double* vel, int32_t* counts, int32_t* ended) {
    if (!g || !sigma || !mu || !flow || n_lines < 0 || max_points < 0 || !(tol > 0) || !(flow->V > 0))
        return CPG_E_INVALID;
    if (n_lines > 0 && (!starts || !counts || !ended || (max_points > 0 && (!pts || !vel)))) return CPG_E_INVALID;
    if (!(flow->mach >= 0 && flow->mach < 1)) return CPG_E_INVALID;
    ProfInstall pi(g->ctx);
    PointField f;
    int rc = f.prepare(g, sigma, mu);
    if (rc != CPG_OK) return rc;
    cpg_refs refs{1, 1, 1, {0, 0, 0}};
    cpg::CaseScalars cs;
    case_scalars(*flow, refs, cs);
    struct Field {
        PointField* f;
        double vinf[3], pg;
    } u{&f, {cs.Vinf[0], cs.Vinf[1], cs.Vinf[2]}, cs.PG};
    // geometry::pntVelocity (CPanel/geometry.cpp:1239-1253): the panels' velocity plus V_inf, the x
    // component then divided by the Prandtl-Glauert factor
    cpg_velocity_fn fn = [](void* user, const double* p, int64_t m, double* v) -> int {
        Field* u = (Field*)user;
        int e = u->f->eval(p, m, v);
        if (e != CPG_OK) return e;
        for (int64_t i = 0; i < m; i++) {
            for (int c = 0; c < 3; c++) v[3 * i + c] += u->vinf[c];
            v[3 * i] /= u->pg;
        }
        return CPG_OK;
    };
    const double speed = std::sqrt(cs.Vinf[0] * cs.Vinf[0] + cs.Vinf[1] * cs.Vinf[1] + cs.Vinf[2] * cs.Vinf[2]);
    return cpg::streamlines_rkf45(fn, &u, speed, starts, n_lines, x_max, tol, max_points, pts, vel, counts, ended);
}

int cpg_stability_derivatives(cpg_geometry* g, const cpg_flow* flow, const cpg_refs* refs, int precision,
                              const cpg_case_out* base, cpg_stability* out) {
    if (!g || !flow || !refs || !out) return CPG_E_INVALID;
    const double delta = 0.5, dRad = delta * kPi / 180;  // CPanel/cpCase.cpp:637-638
    cpg_flow fl[3] = {*flow, *flow, *flow};
    fl[1].alpha += delta;
    fl[2].beta += delta;
    const int64_t n = g->H.n_body;
    // per-panel outputs of all three cases where the caller wants the base case's
    std::vector<double> mu, sigma, phi, vel, cp;
    cpg_case_out o{};
    if (base) {
        auto want = [&](double* dst, std::vector<double>& v, size_t per) -> double* {
            if (!dst) return nullptr;
            v.assign(3 * per, 0.0);
            return v.data();
        };
        o.mu = want(base->mu, mu, n);
        o.sigma = want(base->sigma, sigma, n);
        o.phi = want(base->phi, phi, n);
        o.vel = want(base->vel, vel, 3 * n);
        o.cp = want(base->cp, cp, n);
    }
    double CL[3], CDi[3], Fb[9], Fw[9], CM[9];
    o.CL = CL;
    o.CDi = CDi;
    o.Fbody = Fb;
    o.Fwind = Fw;
    o.CM = CM;
    const int rc = cpg_solve_cases(g, fl, 3, refs, precision, &o, nullptr);
    if (rc != CPG_OK && rc != CPG_E_NOT_CONVERGED) return rc;
    auto F = [&](int c, int q) { return q == 0 ? CDi[c] : (q == 2 ? CL[c] : Fw[3 * c + 1]); };
    for (int q = 0; q < 3; q++) {
        out->dF_dAlpha[q] = (F(1, q) - F(0, q)) / dRad;
        out->dF_dBeta[q] = (F(2, q) - F(0, q)) / dRad;
        out->dM_dAlpha[q] = (CM[3 + q] - CM[q]) / dRad;
        out->dM_dBeta[q] = (CM[6 + q] - CM[q]) / dRad;
    }
    if (base) {
        auto put = [&](double* dst, const std::vector<double>& v, size_t per) {
            if (dst) std::copy(v.begin(), v.begin() + per, dst);
        };
        put(base->mu, mu, n);
        put(base->sigma, sigma, n);
        put(base->phi, phi, n);
        put(base->vel, vel, 3 * n);
        put(base->cp, cp, n);
        if (base->CL) base->CL[0] = CL[0];
        if (base->CDi) base->CDi[0] = CDi[0];
        for (int q = 0; q < 3; q++) {
            if (base->Fbody) base->Fbody[q] = Fb[q];
            if (base->Fwind) base->Fwind[q] = Fw[q];
            if (base->CM) base->CM[q] = CM[q];
        }
    }
    return rc;
}

int cpg_panel_phi_inf(cpg_ctx* ctx, const double* verts, const double* poi, int64_t m, double* src, double* dub) {
    if (!ctx || m < 0 || (m > 0 && (!verts || !poi || !src || !dub))) return fail(ctx, CPG_E_INVALID, "bad argument");
    CK(cpg::launch_phi_batch(verts, poi, m, src, dub, 0, ctx->stream), "panelPhiInf");
    CK(cudaStreamSynchronize(ctx->stream), "panelPhiInf");
    return CPG_OK;
}

int cpg_dub_phi_inf(cpg_ctx* ctx, const double* verts, const double* poi, int64_t m, double* dub) {
    if (!ctx || m < 0 || (m > 0 && (!verts || !poi || !dub))) return fail(ctx, CPG_E_INVALID, "bad argument");
    CK(cpg::launch_phi_batch(verts, poi, m, nullptr, dub, 1, ctx->stream), "dubPhiInf");
    CK(cudaStreamSynchronize(ctx->stream), "dubPhiInf");
    return CPG_OK;
}

int cpg_panel_v_inf(cpg_ctx* ctx, const double* verts, const double* poi, int64_t m, double* vs, double* vd) {
    if (!ctx || m < 0 || (m > 0 && (!verts || !poi || !vs || !vd))) return fail(ctx, CPG_E_INVALID, "bad argument");
    CK(cpg::launch_v_batch(verts, poi, m, vs, vd, ctx->stream), "panelVInf");
    CK(cudaStreamSynchronize(ctx->stream), "panelVInf");
    return CPG_OK;
}

int cpg_prof_enable(cpg_ctx* ctx, int on) {
    if (!ctx) return CPG_E_INVALID;
    if (on) {
        if (!ctx->prof) ctx->prof = new (std::nothrow) cpg::Prof();
        if (!ctx->prof) return CPG_E_OOM;
        CK(cudaStreamSynchronize(ctx->stream), "profiler");
        ctx->prof->reset();
    } else {
        CK(cudaStreamSynchronize(ctx->stream), "profiler");
        delete ctx->prof;
        ctx->prof = nullptr;
    }
    return CPG_OK;
}

int cpg_prof_read(cpg_ctx* ctx, cpg_prof* out) {
    if (!ctx || !out) return CPG_E_INVALID;
    for (int c = 0; c < CPG_PROF_NCLS; c++) {
        out->launches[c] = 0;
        out->ms[c] = 0;
    }
    if (!ctx->prof) return CPG_OK;
    CK(cudaStreamSynchronize(ctx->stream), "profiler");
    ctx->prof->collect();
    for (int c = 0; c < CPG_PROF_NCLS && c < cpg::Prof::NCLS; c++) {
        out->launches[c] = ctx->prof->launches[c];
        out->ms[c] = ctx->prof->ms[c];
    }
    return CPG_OK;
}

int cpg_measure_fp64_peak(cpg_ctx* ctx, double* tflops) {
    if (!ctx || !tflops) return CPG_E_INVALID;
    *tflops = cpg::measure_fp64_tflops(ctx->stream);
    return *tflops > 0 ? CPG_OK : fail(ctx, CPG_E_CUDA, "FP64 probe failed");
}

int cpg_compiled_arch(void) { return CPG_COMPILED_ARCH; }

/* ------------------------------------------------ vortex-particle operators */

int cpg_ptree_build(cpg_ctx* ctx, const double* pos, const double* strength, const double* radius, int64_t n,
                    int64_t max_members, double theta, cpg_ptree** out) {
    if (!ctx || !out || n < 0 || max_members < 1 || !(theta > 0) || (n > 0 && (!pos || !strength || !radius)))
        return fail(ctx, CPG_E_INVALID, "bad argument");
    if (n > (int64_t)INT32_MAX / 2) return fail(ctx, CPG_E_INVALID, "too many particles");
    *out = nullptr;
    cpg_ptree* t = new (std::nothrow) cpg_ptree();
    if (!t) return fail(ctx, CPG_E_OOM, "host allocation");
    t->ctx = ctx;
    cudaStream_t s = ctx->stream;
    std::vector<double> hp(3 * n), hs(3 * n), hr(n);
    if (n > 0) {
        cudaError_t e = cudaMemcpyAsync(hp.data(), pos, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hs.data(), strength, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hr.data(), radius, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            delete t;
            return cuda_fail(ctx, e, "particle download");
        }
    }
    cpg::build_particle_tree(hp.data(), hs.data(), hr.data(), n, max_members, theta, t->T);
    cudaError_t e = upload(t->nodes, t->T.nodes, s);
    if (e == cudaSuccess) e = upload(t->fnodes, t->T.fnodes, s);
    if (e == cudaSuccess) e = upload(t->parts, t->T.parts, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cpg_ptree_destroy(t);
        return cuda_fail(ctx, e, "tree upload");
    }
    *out = t;
    return CPG_OK;
}

void cpg_ptree_destroy(cpg_ptree* t) {
    if (!t) return;
    t->nodes.release();
    t->fnodes.release();
    t->parts.release();
    delete t;
}

int cpg_ptree_info_get(const cpg_ptree* t, cpg_ptree_info* o) {
    if (!t || !o) return CPG_E_INVALID;
    o->n_particles = t->T.n;
    o->n_nodes = (int64_t)t->T.nodes.size();
    o->n_leaves = 0;
    for (const auto& nd : t->T.nodes) o->n_leaves += nd.leaf ? 1 : 0;
    o->n_levels = t->T.levels;
    return CPG_OK;
}

int cpg_ptree_table(const cpg_ptree* t, double* nodes, int64_t* leaf_members) {
    if (!t) return CPG_E_INVALID;
    if (nodes) cpg::particle_tree_table(t->T, nodes);
    if (leaf_members)
        for (size_t q = 0; q < t->T.perm.size(); q++) leaf_members[q] = t->T.perm[q];
    return CPG_OK;
}

int cpg_ptree_host_table(const double* pos, const double* strength, const double* radius, int64_t n,
                         int64_t max_members, double* nodes, int64_t cap_nodes, int64_t* leaf_members,
                         cpg_ptree_info* info) {
    if (n < 0 || max_members < 1 || !info || (n > 0 && (!pos || !strength || !radius))) return CPG_E_INVALID;
    if (n > (int64_t)INT32_MAX / 2) return CPG_E_INVALID;
    cpg::ParticleTree T;
    cpg::build_particle_tree(pos, strength, radius, n, max_members, 0.5, T);
    info->n_particles = n;
    info->n_nodes = (int64_t)T.nodes.size();
    info->n_leaves = 0;
    for (const auto& nd : T.nodes) info->n_leaves += nd.leaf ? 1 : 0;
    info->n_levels = T.levels;
    if (leaf_members)
        for (int64_t q = 0; q < n; q++) leaf_members[q] = T.perm[q];
    if (!nodes) return CPG_OK;
    if (cap_nodes < info->n_nodes) return CPG_E_INVALID;
    cpg::particle_tree_table(T, nodes);
    return CPG_OK;
}

int cpg_bh_velocity_points(cpg_ptree* t, const double* pts, int64_t m, double* vel) {
    if (!t) return CPG_E_INVALID;
    cpg_ctx* ctx = t->ctx;
    if (m < 0 || (m > 0 && (!pts || !vel))) return fail(ctx, CPG_E_INVALID, "bad argument");
    if (m == 0) return CPG_OK;
    ProfInstall pi(ctx);
    int nn = (int)t->T.nodes.size();
    if (nn <= 1) {  // the root alone: no children to visit, the reference returns zero
        CK(cudaMemsetAsync(vel, 0, sizeof(double) * 3 * m, ctx->stream), "barnesHutVel");
    } else {
        cpg::ProfScope ps(cpg::Prof::PARTICLES, ctx->stream);
        CK(cpg::launch_bh_points(t->nodes.as<cpg::BHNode>(),
                                 t->precision == CPG_MIXED ? t->fnodes.as<cpg::BHNodeF>() : nullptr, nn,
                                 t->parts.as<cpg::BHPart>(), t->T.theta, pts, m,
                                 cpg::vp_constants(), vel, ctx->stream),
           "barnesHutVel");
    }
    CK(cudaStreamSynchronize(ctx->stream), "barnesHutVel");
    return CPG_OK;
}

int cpg_set_particle_precision(cpg_ctx* ctx, int precision) {
    if (!ctx || (precision != CPG_PLAIN_FP64 && precision != CPG_MIXED)) return CPG_E_INVALID;
    ctx->particle_precision = precision;
    return CPG_OK;
}

int cpg_ptree_set_precision(cpg_ptree* t, int precision) {
    if (!t || (precision != CPG_PLAIN_FP64 && precision != CPG_MIXED)) return CPG_E_INVALID;
    t->precision = precision;
    return CPG_OK;
}

int cpg_bh_particles(cpg_ptree* t, double* vel, double* stretch, double* diff) {
    if (!t) return CPG_E_INVALID;
    cpg_ctx* ctx = t->ctx;
    int64_t n = t->T.n;
    if (n == 0 || (!vel && !stretch && !diff)) return CPG_OK;
    ProfInstall pi(ctx);
    int nn = (int)t->T.nodes.size();
    if (nn <= 1) {
        for (double* o : {vel, stretch, diff})
            if (o) CK(cudaMemsetAsync(o, 0, sizeof(double) * 3 * n, ctx->stream), "barnesHut");
    } else {
        cpg::ProfScope ps(cpg::Prof::PARTICLES, ctx->stream);
        CK(cpg::launch_bh_particles(t->nodes.as<cpg::BHNode>(),
                                    t->precision == CPG_MIXED ? t->fnodes.as<cpg::BHNodeF>() : nullptr, nn,
                                    t->parts.as<cpg::BHPart>(), n, t->T.theta,
                                    cpg::vp_constants(), vel, stretch, diff, ctx->stream),
           "barnesHut");
    }
    CK(cudaStreamSynchronize(ctx->stream), "barnesHut");
    return CPG_OK;
}

int cpg_particles_velocity(cpg_ctx* ctx, const double* pos, const double* strength, const double* radius, int64_t n,
                           const double* pts, int64_t m, int kernel, double* vel) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !strength || !radius))) return fail(ctx, CPG_E_INVALID, "bad argument");
    if (kernel < CPG_VEL_GAUSS_SYM || kernel > CPG_VEL_ALG) return fail(ctx, CPG_E_INVALID, "unknown kernel");
    if (!pts) m = n;
    if (m < 0 || (m > 0 && !vel)) return fail(ctx, CPG_E_INVALID, "bad argument");
    if (pts && kernel == CPG_VEL_GAUSS_SYM) return fail(ctx, CPG_E_INVALID, "symmetrised core needs particle targets");
    if (m == 0) return CPG_OK;
    ProfInstall pi(ctx);
    cudaStream_t s = ctx->stream;
    DevBuf parts, split;
    CK(parts.ensure(sizeof(cpg::BHPart) * std::max<int64_t>(1, n)), "alloc particles");
    CK(cpg::launch_pack_parts(pos, strength, radius, n, parts.as<cpg::BHPart>(), s), "pack particles");
    {
        cpg::ProfScope ps(cpg::Prof::PARTICLES, s);
        const cpg::BHPart* tg = pts ? nullptr : parts.as<cpg::BHPart>();
        const int64_t need = cpg::direct_scratch_doubles(n, m);
        if (need > 0) CK(split.ensure(sizeof(double) * need), "alloc direct-sum ranges");
        CK(cpg::launch_direct(kernel, false, false, parts.as<cpg::BHPart>(), n, tg, pts, m, cpg::vp_constants(), vel,
                              nullptr, nullptr, s, split.as<double>(), need),
           "particle velocity");
    }
    cudaError_t e = cudaStreamSynchronize(s);
    parts.release();
    split.release();
    CK(e, "particle velocity");
    return CPG_OK;
}

int cpg_particles_stretch_diff(cpg_ctx* ctx, const double* pos, const double* strength, const double* radius,
                               int64_t n, double* stretch, double* diff) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !strength || !radius))) return fail(ctx, CPG_E_INVALID, "bad argument");
    if (n == 0 || (!stretch && !diff)) return CPG_OK;
    ProfInstall pi(ctx);
    cudaStream_t s = ctx->stream;
    DevBuf parts, split;
    CK(parts.ensure(sizeof(cpg::BHPart) * n), "alloc particles");
    CK(cpg::launch_pack_parts(pos, strength, radius, n, parts.as<cpg::BHPart>(), s), "pack particles");
    {
        cpg::ProfScope ps(cpg::Prof::PARTICLES, s);
        const int64_t need = cpg::direct_scratch_doubles(n, n);
        if (need > 0) CK(split.ensure(sizeof(double) * need), "alloc direct-sum ranges");
        CK(cpg::launch_direct(0, stretch != nullptr, diff != nullptr, parts.as<cpg::BHPart>(), n,
                              parts.as<cpg::BHPart>(), nullptr, n, cpg::vp_constants(), nullptr, stretch, diff, s,
                              split.as<double>(), need),
           "particle strength update");
    }
    cudaError_t e = cudaStreamSynchronize(s);
    parts.release();
    split.release();
    CK(e, "particle strength update");
    return CPG_OK;
}

int cpg_panels_velocity(cpg_ctx* ctx, const double* body_verts, const double* sigma, const double* mu, int64_t nb,
                        const double* wake_verts, const double* wake_mu, int64_t nw, const double* pts, int64_t m,
                        double* vel) {
    if (!ctx || nb < 0 || nw < 0 || m < 0) return fail(ctx, CPG_E_INVALID, "bad argument");
    if ((nb > 0 && (!body_verts || !sigma || !mu)) || (nw > 0 && (!wake_verts || !wake_mu)) ||
        (m > 0 && (!pts || !vel)))
        return fail(ctx, CPG_E_INVALID, "bad argument");
    if (m == 0) return CPG_OK;
    ProfInstall pi(ctx);
    cudaStream_t s = ctx->stream;
    DevBuf rec, scr;
    CK(rec.ensure(sizeof(double) * 24 * std::max<int64_t>(1, nb + nw)), "alloc panel records");
    if (ctx->particle_precision == CPG_MIXED) {
        // body panels through the chunked kernel with the far field in FP32, then the wake
        // triangles (FP64) added on top
        CK(scr.ensure(sizeof(double) * std::max<int64_t>(cpg::vp_scratch_doubles(m, nb), 3 * m)), "alloc scratch");
        cpg::ProfScope ps(cpg::Prof::PARTICLES, s);
        CK(cpg::launch_pack_records(body_verts, nb, rec.as<double>(), s), "panel records");
        CK(cpg::vp_launch_panel_vel(rec.as<double>(), sigma, mu, nb, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr,
                                    0, pts, m, 0.0, vel, scr.as<double>(), s, true),
           "panel velocity");
        if (nw > 0) {
            CK(cpg::launch_panels_velocity(nullptr, nullptr, nullptr, 0, wake_verts, wake_mu, nw, pts, m,
                                           rec.as<double>(), scr.as<double>(), s),
               "wake velocity");
            CK(cpg::vp_launch_add(vel, scr.as<double>(), 3 * m, s), "wake velocity");
        }
    } else {
        cpg::ProfScope ps(cpg::Prof::PARTICLES, s);
        CK(cpg::launch_panels_velocity(body_verts, sigma, mu, nb, wake_verts, wake_mu, nw, pts, m, rec.as<double>(),
                                       vel, s),
           "panel velocity");
    }
    cudaError_t e = cudaStreamSynchronize(s);
    rec.release();
    scr.release();
    CK(e, "panel velocity");
    return CPG_OK;
}


// ---- grouped assembly of many geometries (include/cpanel_batch.h) ----

int cpg_group_default_shape(cpg_group_shape* sh) {
    if (!sh) return CPG_E_INVALID;
    sh->chunks_per_item = 2;
    sh->near_band = 1;
    sh->blocks_per_sm = 0;  // the occupancy limit
    return CPG_OK;
}

static bool group_shape_valid(const cpg_group_shape& s) {
    return s.chunks_per_item >= 1 && s.chunks_per_item <= 16 && s.near_band >= 0 && s.near_band <= 64 &&
           s.blocks_per_sm >= 0 && s.blocks_per_sm <= 64;
}

static int group_schedule_impl(const int64_t* n_body, int m, const cpg_group_shape* shape, int32_t* items,
                               int64_t cap, int64_t* count, int64_t* chunk_len) {
    if (!n_body || m <= 0 || !count) return CPG_E_INVALID;
    cpg_group_shape sh;
    cpg_group_default_shape(&sh);
    if (shape) sh = *shape;
    if (!group_shape_valid(sh)) return CPG_E_INVALID;
    for (int q = 0; q < m; q++)
        if (n_body[q] < 1) return CPG_E_INVALID;
    std::vector<int> it;
    int64_t ni = cpg::group_schedule(n_body, m, sh.chunks_per_item, sh.near_band, it);
    *count = ni;
    if (chunk_len)
        for (int q = 0; q < m; q++) chunk_len[q] = cpg::mixed_chunk(n_body[q]);
    if (items) {
        if (cap < ni) return CPG_E_INVALID;
        for (size_t t = 0; t < it.size(); t++) items[t] = (int32_t)it[t];
    }
    return CPG_OK;
}

int cpg_group_schedule(const int64_t* n_body, int m, const cpg_group_shape* shape, int32_t* items, int64_t cap,
                       int64_t* count, int64_t* chunk_len) {
    try {
        return group_schedule_impl(n_body, m, shape, items, cap, count, chunk_len);
    } catch (const std::bad_alloc&) {
        return CPG_E_OOM;
    }
}

namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, cpg_group_shape> g_tune_cache;  // (device, log2 m, 2 log2 pairs)
}  // namespace

static int set_inf_coeff_grouped_impl(cpg_geometry* const* gs, int m, int tune, const cpg_group_shape* shape,
                              cpg_group_report* rep) {
    if (!gs || m <= 0) return CPG_E_INVALID;
    for (int q = 0; q < m; q++)
        if (!gs[q]) return CPG_E_INVALID;
    cpg_ctx* ctx = gs[0]->ctx;
    ProfInstall pi(ctx);
    for (int q = 0; q < m; q++)
        if (gs[q]->ctx->device != ctx->device) return fail(ctx, CPG_E_INVALID, "geometries on different devices");
    if (tune < CPG_TUNE_OFF || tune > CPG_TUNE_FORCE) return fail(ctx, CPG_E_INVALID, "unknown tune mode");
    if (tune == CPG_TUNE_OFF && shape && !group_shape_valid(*shape)) return fail(ctx, CPG_E_INVALID, "bad shape");
    CK(cudaSetDevice(ctx->device), "device");
    cudaStream_t s = ctx->stream;
    // the launch follows the work already queued on every geometry's stream (its uploads)
    std::vector<cpg_ctx*> others;
    for (int q = 0; q < m; q++)
        if (gs[q]->ctx != ctx && std::find(others.begin(), others.end(), gs[q]->ctx) == others.end())
            others.push_back(gs[q]->ctx);
    cudaEvent_t join, e0, e1;
    CK(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "event");
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    struct EvGuard {
        cudaEvent_t a, b, c;
        ~EvGuard() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            cudaEventDestroy(c);
        }
    } evg{join, e0, e1};
    for (cpg_ctx* c : others) {
        CK(cudaEventRecord(join, c->stream), "event");
        CK(cudaStreamWaitEvent(s, join, 0), "join");
    }
    std::vector<cpg::MixedMeshDesc> desc(m);
    std::vector<int64_t> ns(m);
    int64_t rows = 0;
    double pairs = 0;
    int64_t max_nw = 0;
    for (int q = 0; q < m; q++) {
        cpg_geometry* g = gs[q];
        const int64_t n = g->H.n_body;
        const size_t nn = (size_t)n * n;
        CK(ensure_big(g->ctx, g->A32, sizeof(float) * nn), "alloc A (FP32)");
        CK(ensure_big(g->ctx, g->Alo, sizeof(float) * nn), "alloc A low part (FP32)");
        CK(g->rb.ensure(sizeof(double) * (3 * n + cpg::mixed_rb_part_doubles(n, g->H.n_wake))), "alloc rhs basis");
        desc[q] = cpg::MixedMeshDesc{g->rec.as<double>(), g->frec.as<float>(), g->erec.as<double>(), n,
                                     cpg::mixed_chunk(n), g->A32.as<float>(), g->Alo.as<float>(),
                                     g->rb.as<double>() + 3 * n, g->rb.as<double>(),
                                     g->count.as<unsigned long long>(), g->wrec.as<double>(), g->widx.as<int32_t>(),
                                     g->wcoef.as<double>(), g->H.n_wake, rows};
        ns[q] = n;
        rows += n;
        pairs += (double)n * (double)n;
        max_nw = std::max<int64_t>(max_nw, g->H.n_wake);
    }
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
    const int maxb = cpg::assemble_mixed_grouped_max_blocks_per_sm();
    // queue capacity: one chunk per item is the longest queue of any shape
    std::vector<int> items;
    const int64_t max_items = cpg::group_schedule(ns.data(), m, 1, 0, items);
    cpg::MixedMeshDesc* ddesc = nullptr;
    int* ditems = nullptr;
    int* dnext = nullptr;
    CK(cudaMallocAsync((void**)&ddesc, sizeof(cpg::MixedMeshDesc) * m, s), "alloc group descriptors");
    struct FreeGuard {
        void *a, *b, *c;
        cudaStream_t s;
        ~FreeGuard() {
            if (a) cudaFreeAsync(a, s);
            if (b) cudaFreeAsync(b, s);
            if (c) cudaFreeAsync(c, s);
        }
    } fg{ddesc, nullptr, nullptr, s};
    CK(cudaMallocAsync((void**)&ditems, sizeof(int) * 4 * std::max<int64_t>(1, max_items), s), "alloc work queue");
    fg.b = ditems;
    CK(cudaMallocAsync((void**)&dnext, sizeof(int), s), "alloc queue counter");
    fg.c = dnext;
    CK(cudaMemcpyAsync(ddesc, desc.data(), sizeof(cpg::MixedMeshDesc) * m, cudaMemcpyHostToDevice, s), "descriptors");
    auto resolve = [&](cpg_group_shape sh) {
        if (sh.blocks_per_sm <= 0 || sh.blocks_per_sm > maxb) sh.blocks_per_sm = maxb;
        return sh;
    };
    // queue one shape: upload its items and launch the persistent assembly kernel
    int64_t nitems = 0;
    auto launch_core = [&](const cpg_group_shape& sh) -> cudaError_t {
        nitems = cpg::group_schedule(ns.data(), m, sh.chunks_per_item, sh.near_band, items);
        cudaError_t e = cudaMemcpyAsync(ditems, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        return cpg::launch_assemble_mixed_grouped_core(ddesc, ditems, (int)nitems, sh.blocks_per_sm * nsm, dnext, s);
    };
    cpg_group_shape use;
    cpg_group_default_shape(&use);
    int tuned = 0, candidates = 0;
    const auto key = std::make_tuple(ctx->device, (int)std::floor(std::log2((double)m)),
                                     (int)std::floor(2.0 * std::log2(std::max(1.0, pairs))));
    bool have = false;
    if (tune == CPG_TUNE_OFF) {
        if (shape) use = *shape;
        have = true;
    } else if (tune == CPG_TUNE_AUTO) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            use = it->second;
            have = true;
            tuned = 2;
        }
    }
    use = resolve(use);
    if (!have) {
        // coordinate search over shapes that all give the same bits: chunks per far item,
        // then the near band, then the resident blocks per SM; one timed launch each
        cpg::Prof* saved = cpg::g_prof;
        cpg::g_prof = nullptr;  // tuning launches are not part of the profile
        auto timed = [&](const cpg_group_shape& sh, float* ms) -> cudaError_t {
            cudaError_t e;
            if ((e = cudaEventRecord(e0, s)) != cudaSuccess) return e;
            if ((e = launch_core(sh)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(e1, s)) != cudaSuccess) return e;
            if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
            candidates++;
            return cudaEventElapsedTime(ms, e0, e1);
        };
        cudaError_t e = cudaSuccess;
        float best_ms = 0, t = 0;
        cpg_group_shape best = use;
        if (e == cudaSuccess) e = timed(best, &t);  // warm-up: first touch of the matrices
        if (e == cudaSuccess) e = timed(best, &best_ms);
        const int chunk_opts[] = {1, 4, 8};
        for (int c : chunk_opts) {
            if (e != cudaSuccess) break;
            cpg_group_shape sh = best;
            sh.chunks_per_item = c;
            if ((e = timed(sh, &t)) == cudaSuccess && t < best_ms) best_ms = t, best = sh;
        }
        const int band_opts[] = {0, 2, 4};
        for (int b : band_opts) {
            if (e != cudaSuccess) break;
            if (b == best.near_band) continue;
            cpg_group_shape sh = best;
            sh.near_band = b;
            if ((e = timed(sh, &t)) == cudaSuccess && t < best_ms) best_ms = t, best = sh;
        }
        const int bps_opts[] = {maxb - 1, maxb / 2};
        for (int bp : bps_opts) {
            if (e != cudaSuccess) break;
            if (bp < 1 || bp == best.blocks_per_sm || (bp == maxb / 2 && maxb / 2 == maxb - 1)) continue;
            cpg_group_shape sh = best;
            sh.blocks_per_sm = bp;
            if ((e = timed(sh, &t)) == cudaSuccess && t < best_ms) best_ms = t, best = sh;
        }
        cpg::g_prof = saved;
        CK(e, "assembly shape tuning");
        use = best;
        tuned = 1;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = use;
    }
    for (int q = 0; q < m; q++) CK(cudaMemsetAsync(gs[q]->count.p, 0, sizeof(unsigned long long), s), "clear counter");
    CK(cudaEventRecord(e0, s), "event");
    CK(launch_core(use), "grouped assembly (mixed)");
    if (max_nw > 65535) return fail(ctx, CPG_E_INVALID, "more than 65,535 wake panels");
    CK(cpg::launch_assemble_mixed_grouped_finish(ddesc, m, rows, max_nw, s), "grouped sums and wake columns");
    CK(cudaEventRecord(e1, s), "event");
    // every geometry's stream continues after the grouped launch
    for (cpg_ctx* c : others) CK(cudaStreamWaitEvent(c->stream, e1, 0), "join");
    std::vector<unsigned long long> cnt(m, 0);
    for (int q = 0; q < m; q++)
        CK(cudaMemcpyAsync(&cnt[q], gs[q]->count.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s), "counter");
    CK(cudaStreamSynchronize(s), "grouped assembly");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    int64_t near = 0;
    for (int q = 0; q < m; q++) {
        cpg_geometry* g = gs[q];
        g->have32 = true;
        g->lu_ready = false;
        g->n_near32 = (int64_t)cnt[q];
        g->ms_asm = (float)(ms * ((double)ns[q] * (double)ns[q]) / pairs);  // its share of the launch
        near += (int64_t)cnt[q];
    }
    if (rep) {
        rep->shape = use;
        rep->tuned = tuned;
        rep->candidates = candidates;
        rep->items = nitems;
        rep->pairs = (int64_t)pairs;
        rep->near_pairs = near;
        rep->ms = ms;
    }
    return CPG_OK;
}

int cpg_set_inf_coeff_grouped(cpg_geometry* const* gs, int m, int tune, const cpg_group_shape* shape,
                              cpg_group_report* rep) {
    try {
        return set_inf_coeff_grouped_impl(gs, m, tune, shape, rep);
    } catch (const std::bad_alloc&) {
        return fail((gs && m > 0 && gs[0]) ? gs[0]->ctx : nullptr, CPG_E_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail((gs && m > 0 && gs[0]) ? gs[0]->ctx : nullptr, CPG_E_INVALID, e.what());
    }
}


static int lu_factor_grouped_impl(cpg_geometry* const* gs, int m, double* ms_out) {
    if (!gs || m <= 0) return CPG_E_INVALID;
    for (int q = 0; q < m; q++)
        if (!gs[q]) return CPG_E_INVALID;
    cpg_ctx* ctx = gs[0]->ctx;
    ProfInstall pi(ctx);
    for (int q = 0; q < m; q++) {
        if (gs[q]->ctx->device != ctx->device) return fail(ctx, CPG_E_INVALID, "geometries on different devices");
        if (!gs[q]->have32) return fail(ctx, CPG_E_INVALID, "no CPG_MIXED matrix: assemble first");
    }
    CK(cudaSetDevice(ctx->device), "device");
    cudaStream_t s = ctx->stream;
    std::vector<cpg_ctx*> others;
    for (int q = 0; q < m; q++)
        if (gs[q]->ctx != ctx && std::find(others.begin(), others.end(), gs[q]->ctx) == others.end())
            others.push_back(gs[q]->ctx);
    cudaEvent_t join, e0, e1;
    CK(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "event");
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    struct EvGuard {
        cudaEvent_t a, b, c;
        ~EvGuard() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            cudaEventDestroy(c);
        }
    } evg{join, e0, e1};
    for (cpg_ctx* c : others) {
        CK(cudaEventRecord(join, c->stream), "event");
        CK(cudaStreamWaitEvent(s, join, 0), "join");
    }
    std::vector<cpg::LuGraphs*> G(m);
    std::vector<float*> LU(m);
    std::vector<int64_t> ns(m);
    std::vector<int*> bad(m);
    for (int q = 0; q < m; q++) {
        cpg_geometry* g = gs[q];
        const int64_t n = g->H.n_body;
        CK(ensure_big(g->ctx, g->LU, sizeof(float) * (size_t)n * n), "alloc LU");
        CK(g->bad.ensure(sizeof(int)), "alloc flag");
        CK(cudaMemsetAsync(g->bad.p, 0, sizeof(int), s), "clear flag");
        CK(cudaMemcpyAsync(g->LU.p, g->A32.p, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, s), "copy A");
        G[q] = &g->graphs;
        LU[q] = g->LU.as<float>();
        ns[q] = n;
        bad[q] = g->bad.as<int>();
    }
    CK(cudaEventRecord(e0, s), "event");
    CK(cpg::lu_factor_batched(G.data(), LU.data(), ns.data(), bad.data(), m, s), "grouped LU factorization");
    CK(cudaEventRecord(e1, s), "event");
    for (cpg_ctx* c : others) CK(cudaStreamWaitEvent(c->stream, e1, 0), "join");
    CK(cudaEventSynchronize(e1), "grouped LU factorization");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_out) *ms_out = ms;
    for (int q = 0; q < m; q++) gs[q]->lu_ready = true;
    return CPG_OK;
}

int cpg_lu_factor_grouped(cpg_geometry* const* gs, int m, double* ms_out) {
    try {
        return lu_factor_grouped_impl(gs, m, ms_out);
    } catch (const std::bad_alloc&) {
        return fail((gs && m > 0 && gs[0]) ? gs[0]->ctx : nullptr, CPG_E_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail((gs && m > 0 && gs[0]) ? gs[0]->ctx : nullptr, CPG_E_INVALID, e.what());
    }
}


}  // extern "C"

// ---- grouped solves of the batch path (csrc/batch.cpp) ----
namespace cpg {

int geometry_prepare_post(cpg_geometry* g) { return g ? prepare_post(g) : CPG_E_INVALID; }

// cpg_solve_cases (CPG_MIXED) for m geometries that hold their mixed matrices and LU factors
// (cpg_set_inf_coeff_grouped, cpg_lu_factor_grouped): right-hand sides per geometry, the
// refined solves of all of them in lockstep (substitutions on gs[0]'s context stream), then
// each one's post-processing; each geometry's own work runs on its context's stream.  status[q]: each geometry's cpg_status; returns the first failure.
int solve_cases_grouped(cpg_geometry* const* gs, int m, const cpg_flow* const* flows, const int* ks,
                        const cpg_refs* refs, const cpg_case_out* outs, int* status) {
    if (!gs || m <= 0) return CPG_E_INVALID;
    cpg_ctx* ctx = gs[0]->ctx;
    ProfInstall pi(ctx);
    CK(cudaSetDevice(ctx->device), "device");
    cudaStream_t s = ctx->stream;
    cudaEvent_t join;
    CK(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "event");
    struct EvGuard {
        cudaEvent_t e;
        ~EvGuard() { cudaEventDestroy(e); }
    } jg{join};
    for (int q = 0; q < m; q++)
        if (gs[q]->ctx != ctx) {
            CK(cudaEventRecord(join, gs[q]->ctx->stream), "event");
            CK(cudaStreamWaitEvent(s, join, 0), "join");
        }
    struct Out {
        double *mu, *sigma, *rhs, *phi, *cp, *vel, *forces, *tz, *wmu;
    };
    std::vector<Out> O(m);
    std::vector<cpg::RefineMesh> rm(m);
    for (int q = 0; q < m; q++) {
        cpg_geometry* g = gs[q];
        const int k = ks[q];
        const int64_t n = g->H.n_body, nw = g->H.n_wake;
        if (!g->have32 || !g->lu_ready || k < 1 || k > 4096)
            return fail(ctx, CPG_E_INVALID, "grouped solve: geometry without mixed matrix or factors, or bad k");
        int rc = prepare_post(g);
        if (rc != CPG_OK) return rc;
        cudaStream_t t = g->ctx->stream;  // this geometry's own work
        std::vector<cpg::CaseScalars> cs(k);
        for (int c = 0; c < k; c++) case_scalars(flows[q][c], refs[q], cs[c]);
        CK(upload(g->cases, cs, t), "upload cases");
        const size_t kn = (size_t)k * n;
        const size_t need = sizeof(double) * (8 * kn + 9 * (size_t)k + 2 * (size_t)k + (size_t)k * nw) + 8 * 256;
        CK(g->outs.ensure(need), "alloc outputs");
        Out& o = O[q];
        o.mu = g->outs.as<double>();
        o.sigma = o.mu + kn;
        o.rhs = o.sigma + kn;
        o.phi = o.rhs + kn;
        o.cp = o.phi + kn;
        o.vel = o.cp + kn;
        o.forces = o.vel + 3 * kn;
        o.tz = o.forces + 9 * (size_t)k;
        o.wmu = o.tz + 2 * (size_t)k;
        CK(g->work.ensure(cpg::solve_lu_work_bytes(n, k)), "alloc solver workspace");
        const cpg::CaseScalars* dcs = g->cases.as<cpg::CaseScalars>();
        CK(cpg::launch_sigma(g->rec.as<double>(), n, k, dcs, o.sigma, t), "sigma");
        CK(cpg::launch_rhs_basis(g->rb.as<double>(), n, k, dcs, o.rhs, t), "rhs");
        rm[q] = cpg::RefineMesh{g->A32.as<float>(), g->Alo.as<float>(), g->LU.as<float>(), g->graphs.dinv, n, k,
                                o.rhs, o.mu, g->work.p, t};
    }
    std::vector<cpg::SolveStats> st(m);
    CK(cpg::solve_lu_refined_batched(rm.data(), m, kMixedRefineTol, 16, st.data(), s), "refined solves (grouped)");
    for (int q = 0; q < m; q++) {
        cpg_geometry* g = gs[q];
        const int k = ks[q];
        cudaStream_t t = g->ctx->stream;
        CK(g->post_work.ensure(cpg::post_work_bytes(g->T, k)), "alloc post workspace");
        CK(cudaStreamWaitEvent(t, g->post_ev, 0), "wait for the post tables");
        const Out& o = O[q];
        CK(cpg::launch_post(g->T, k, g->cases.as<cpg::CaseScalars>(), o.mu, o.phi, o.vel, o.cp, o.forces, o.tz, o.wmu,
                            g->post_work.p, t),
           "post");
    }
    std::vector<std::vector<double>> hf(m), ht(m);
    for (int q = 0; q < m; q++) {
        const int k = ks[q];
        const size_t kn = (size_t)k * gs[q]->H.n_body;
        const Out& o = O[q];
        const cpg_case_out* co = outs ? &outs[q] : nullptr;
        cudaStream_t t = gs[q]->ctx->stream;
        auto copy = [&](double* dst, const double* src, size_t cnt) -> cudaError_t {
            if (!dst) return cudaSuccess;
            return cudaMemcpyAsync(dst, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, t);
        };
        if (co) {
            CK(copy(co->mu, o.mu, kn), "copy mu");
            CK(copy(co->sigma, o.sigma, kn), "copy sigma");
            CK(copy(co->phi, o.phi, kn), "copy phi");
            CK(copy(co->vel, o.vel, 3 * kn), "copy vel");
            CK(copy(co->cp, o.cp, kn), "copy cp");
        }
        hf[q].resize(9 * (size_t)k);
        ht[q].resize(2 * (size_t)k);
        CK(cudaMemcpyAsync(hf[q].data(), o.forces, sizeof(double) * 9 * k, cudaMemcpyDeviceToHost, t), "copy forces");
        CK(cudaMemcpyAsync(ht[q].data(), o.tz, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, t), "copy CL");
    }
    for (int q = 0; q < m; q++) CK(cudaStreamSynchronize(gs[q]->ctx->stream), "grouped solves");
    int first = CPG_OK;
    for (int q = 0; q < m; q++) {
        const int k = ks[q];
        const cpg_case_out* co = outs ? &outs[q] : nullptr;
        if (co)
            for (int c = 0; c < k; c++) {
                if (co->CL) co->CL[c] = ht[q][2 * c];
                if (co->CDi) co->CDi[c] = ht[q][2 * c + 1];
                for (int a = 0; a < 3; a++) {
                    if (co->Fbody) co->Fbody[3 * c + a] = hf[q][9 * c + a];
                    if (co->Fwind) co->Fwind[3 * c + a] = hf[q][9 * c + 3 + a];
                    if (co->CM) co->CM[3 * c + a] = hf[q][9 * c + 6 + a];
                }
            }
        status[q] = st[q].residual_max > 1e-9 ? CPG_E_NOT_CONVERGED : CPG_OK;
        if (status[q] != CPG_OK && first == CPG_OK) first = status[q];
    }
    if (first != CPG_OK) ctx_set_error(ctx, "grouped solve: a system stopped above tolerance");
    return first;
}

}  // namespace cpg

// ---- C ABI: the FP32 LU and its block substitutions on caller-owned device matrices ----
extern "C" int cpg_lu_solve_f32(cpg_ctx* ctx, int64_t n, float* A, int64_t k, float* X) {
    if (!ctx || n < 0 || k < 0 || k > INT32_MAX || (n > 0 && (!A || (k > 0 && !X)))) return CPG_E_INVALID;
    if (n == 0) return CPG_OK;
    ProfInstall pi(ctx);
    cudaStream_t s = ctx->stream;
    cpg::LuGraphs G;
    int* bad = nullptr;
    int hbad = 0;
    cudaError_t e = cudaMalloc(&bad, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cpg::lu_factor_fp32(&G, A, n, bad, s);
    if (e == cudaSuccess && k > 0) e = cpg::lu_solve_fp32(&G, A, n, X, (int)k, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    G.release();
    if (bad) cudaFree(bad);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(ctx, std::string("lu: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA;
    }
    if (hbad == 2) {
        cpg::ctx_set_error(ctx, "lu: non-finite entry");
        return CPG_E_INVALID;
    }
    if (hbad != 0) {
        cpg::ctx_set_error(ctx, "lu: zero pivot, or a wait of a tensor-core product ran out");
        return CPG_E_INVALID;
    }
    return CPG_OK;
}

// ---- C ABI: the tensor-core GEMM on caller-owned FP32 device matrices ----
extern "C" int cpg_gemm_f32_tc(cpg_ctx* ctx, int64_t m, int64_t n, int64_t k, float alpha, const float* A,
                               int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                               int sm_budget) {
    if (!ctx || m < 0 || n < 0 || k < 0 || (m > 0 && (!C || ldc < m)) || (k > 0 && (!A || !B || lda < m || ldb < k)))
        return CPG_E_INVALID;
    if (m == 0 || n == 0) return CPG_OK;
    ProfInstall pi(ctx);
    cudaStream_t s = ctx->stream;
    const int64_t kp = std::max<int64_t>(cpg::kTcK, (k + cpg::kTcK - 1) / cpg::kTcK * cpg::kTcK);
    const size_t ba = cpg::tc_operand_bytes(m, kp), bb = cpg::tc_operand_bytes(n, kp);
    void* mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, ba + bb + 256);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(ctx, std::string("gemm: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA;
    }
    cpg::TcOperand opA, opB;
    cpg::tc_operand_bind(opA, mem, m, kp);
    cpg::tc_operand_bind(opB, (char*)mem + ba, n, kp);
    int* err = (int*)((char*)mem + ba + bb);
    int herr = 0;
    const int budget = sm_budget > 0 ? sm_budget : cpg::tc_num_sms();
    if ((e = cudaMemsetAsync(mem, 0, ba + bb + 256, s)) == cudaSuccess &&
        (k == 0 || (e = cpg::tc_split(A, 1, lda, m, k, opA, err, s)) == cudaSuccess) &&
        (k == 0 || (e = cpg::tc_split(B, ldb, 1, n, k, opB, err, s)) == cudaSuccess))
        e = cpg::tc_gemm(opA, m, opB, n, alpha, beta, C, ldc, budget, err, s, err + 16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(mem);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(ctx, std::string("gemm: ") + cudaGetErrorString(e));
        return CPG_E_CUDA;
    }
    if (herr == 2) {
        cpg::ctx_set_error(ctx, "gemm: non-finite operand");
        return CPG_E_INVALID;
    }
    if (herr != 0) {
        cpg::ctx_set_error(ctx, "gemm: a wait of the kernel timed out");
        return CPG_E_TIMEOUT;
    }
    return CPG_OK;
}
