// The C++ drop-in shim (include/cpanel_shim.hpp): CPanel's hot-path classes over the C ABI.
//
// Single-point operators stage their few doubles through one small device buffer per device
// (grown on demand, guarded by a mutex) and wait for the result; the contexts the shim creates
// live until the process ends.
#include "../../include/cpanel_shim.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <fstream>
#include <mutex>

namespace cpg {
namespace shim {

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_ctx_mu, g_scr_mu;
cpg_ctx* g_ctx[kMaxDevices] = {};

struct Scratch {
    double* p = nullptr;
    size_t cap = 0;
};
Scratch g_scr[kMaxDevices];

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw error(CPG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// device buffer of at least `doubles` doubles on the device (call with g_scr_mu held)
double* scratch(int dev, size_t doubles) {
    Scratch& s = g_scr[dev];
    if (s.cap < doubles) {
        if (s.p) cudaFree(s.p);
        s.p = nullptr;
        s.cap = 0;
        cuda_check(cudaMalloc(&s.p, sizeof(double) * doubles), "shim scratch");
        s.cap = doubles;
    }
    return s.p;
}

void h2d(double* d, const double* h, size_t n) { cuda_check(cudaMemcpy(d, h, sizeof(double) * n, cudaMemcpyHostToDevice), "copy"); }
void d2h(double* h, const double* d, size_t n) { cuda_check(cudaMemcpy(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost), "copy"); }

}  // namespace

cpg_ctx* context(int device) {
    if (device < 0 || device >= kMaxDevices) throw error(CPG_E_INVALID, "shim: device index out of range");
    std::lock_guard<std::mutex> l(g_ctx_mu);
    if (!g_ctx[device]) {
        cpg_ctx* c = nullptr;
        const int st = cpg_create(&c, device);
        if (st != CPG_OK) throw error(st, "shim: cpg_create failed");
        g_ctx[device] = c;
    }
    return g_ctx[device];
}

void check(int status, cpg_ctx* ctx, const char* what) {
    if (status != CPG_OK) throw error(status, std::string(what) + ": " + (ctx ? cpg_last_error(ctx) : ""));
}

// ---- one triangle at m points (the verts are repeated per point, as the C ABI pairs them) ----
namespace {
template <class F>
void tri_call(const double* verts, const double* poi, int64_t m, int nout, double* o1, double* o2, F call) {
    if (m <= 0) return;
    cpg_ctx* ctx = context(0);
    std::lock_guard<std::mutex> l(g_scr_mu);
    cuda_check(cudaSetDevice(0), "device");
    double* d = scratch(0, (size_t)m * (12 + 2 * nout));
    std::vector<double> v((size_t)m * 9);
    for (int64_t i = 0; i < m; i++) std::copy(verts, verts + 9, v.begin() + 9 * i);
    h2d(d, v.data(), v.size());
    h2d(d + 9 * m, poi, (size_t)(3 * m));
    double* r1 = d + 12 * m;
    double* r2 = r1 + nout * m;
    check(call(ctx, d, d + 9 * m, r1, r2), ctx, "shim: panel influence");
    check(cpg_synchronize(ctx), ctx, "shim: synchronize");
    if (o1) d2h(o1, r1, (size_t)(nout * m));
    if (o2) d2h(o2, r2, (size_t)(nout * m));
}
}  // namespace

void tri_phi_inf(const double* verts, const double* poi, int64_t m, double* phi_src, double* phi_dub) {
    tri_call(verts, poi, m, 1, phi_src, phi_dub, [&](cpg_ctx* c, const double* v, const double* p, double* a, double* b) {
        return cpg_panel_phi_inf(c, v, p, m, a, b);
    });
}

void tri_dub_phi_inf(const double* verts, const double* poi, int64_t m, double* phi_dub) {
    tri_call(verts, poi, m, 1, phi_dub, nullptr, [&](cpg_ctx* c, const double* v, const double* p, double* a, double*) {
        return cpg_dub_phi_inf(c, v, p, m, a);
    });
}

void tri_v_inf(const double* verts, const double* poi, int64_t m, double* v_src, double* v_dub) {
    tri_call(verts, poi, m, 3, v_src, v_dub, [&](cpg_ctx* c, const double* v, const double* p, double* a, double* b) {
        return cpg_panel_v_inf(c, v, p, m, a, b);
    });
}

// panel::setGeom's centre and longest side (CPanel/panel.cpp:33-72), for the near/far choice
void bodyPanel::geom() {
    longSide_ = 0;
    for (int k = 0; k < 3; k++) {
        const double* a = v_ + 3 * k;
        const double* b = v_ + 3 * ((k + 1) % 3);
        const double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
        longSide_ = std::max(longSide_, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    for (int q = 0; q < 3; q++) c_[q] = (v_[q] + v_[3 + q] + v_[6 + q]) / 3.0;
}

// ---- geometry ----
geometry::geometry(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids, int64_t n_tris,
                   int device) {
    ctx_ = context(device);
    check(cpg_geometry_create(ctx_, nodes, n_nodes, tris, ids, n_tris, &g_), ctx_, "geometry::readTri");
    cpg_geometry_info info;
    check(cpg_geometry_info_get(g_, &info), ctx_, "geometry info");
    n_ = info.n_body;
    std::vector<double> body((size_t)(n_ * 18));
    check(cpg_geometry_tables(g_, body.data(), nullptr, nullptr, nullptr, nullptr), ctx_, "geometry tables");
    cen_.resize((size_t)(3 * n_));
    nrm_.resize((size_t)(3 * n_));
    for (int64_t i = 0; i < n_; i++)
        for (int q = 0; q < 3; q++) {
            cen_[3 * i + q] = body[18 * i + q];
            nrm_[3 * i + q] = body[18 * i + 3 + q];
        }
}

std::unique_ptr<geometry> geometry::readTri(const std::string& path, int device) {
    std::ifstream f(path);
    if (!f) throw error(CPG_E_INVALID, "readTri: cannot open " + path);
    int64_t nn = 0, nt = 0;
    f >> nn >> nt;
    if (!f || nn <= 0 || nt <= 0) throw error(CPG_E_BAD_MESH, "readTri: bad header in " + path);
    std::vector<double> nodes((size_t)(3 * nn));
    std::vector<int64_t> tris((size_t)(3 * nt));
    std::vector<int32_t> ids((size_t)nt);
    for (double& x : nodes) f >> x;
    for (int64_t& t : tris) f >> t;
    for (int32_t& s : ids) f >> s;
    if (!f) throw error(CPG_E_BAD_MESH, "readTri: truncated file " + path);
    return std::unique_ptr<geometry>(new geometry(nodes.data(), nn, tris.data(), ids.data(), nt, device));
}

geometry::~geometry() {
    if (g_) cpg_geometry_destroy(g_);
}

void geometry::setInfCoeff() {
    check(cpg_set_inf_coeff(g_, CPG_PLAIN_FP64), ctx_, "geometry::setInfCoeff");
    A_.reset();
    B_.reset();
    assembled_ = true;
}

Matrix* geometry::getA() {
    if (!assembled_) setInfCoeff();
    if (!A_) {
        A_.reset(new Matrix(n_, n_));
        check(cpg_get_A(g_, A_->data()), ctx_, "geometry::getA");
    }
    return A_.get();
}

Matrix* geometry::getB() {
    if (!assembled_) setInfCoeff();
    if (!B_) {
        B_.reset(new Matrix(n_, n_));
        check(cpg_get_B(g_, B_->data()), ctx_, "geometry::getB");
    }
    return B_.get();
}

// ---- cpCase ----
cpCase::cpCase(geometry* geom, double V, double alpha, double beta, double mach, double Sref, double bref,
               double cref, const double cg[3], bool mixed)
    : geom_(geom), flow_{V, alpha, beta, mach}, refs_{Sref, bref, cref, {cg[0], cg[1], cg[2]}}, mixed_(mixed) {}

bool cpCase::solveMatrixEq() {
    const int64_t n = geom_->nBodyPanels();
    mu_.assign((size_t)n, 0.0);
    sigma_.assign((size_t)n, 0.0);
    cp_.assign((size_t)n, 0.0);
    cpg_case_out out{mu_.data(), sigma_.data(), nullptr, nullptr, cp_.data(), &CL_, &CDi_, Fb_, Fw_, CM_};
    cpg_solve_stats st;
    const int rc = cpg_solve_cases(geom_->handle(), &flow_, 1, &refs_, mixed_ ? CPG_MIXED : CPG_PLAIN_FP64, &out, &st);
    if (rc == CPG_E_NOT_CONVERGED) return false;  // results valid, above the tolerance
    check(rc, geom_->ctx(), "cpCase::solveMatrixEq");
    return true;
}

// ---- particles ----
void particles_velocity_at(const double* pos, const double* strength, const double* radius, int64_t n,
                           const double* pts, int64_t m, int kernel, double* vel) {
    if (n <= 0 || m <= 0) return;
    cpg_ctx* ctx = context(0);
    std::lock_guard<std::mutex> l(g_scr_mu);
    cuda_check(cudaSetDevice(0), "device");
    double* d = scratch(0, (size_t)(7 * n + 6 * m));
    h2d(d, pos, (size_t)(3 * n));
    h2d(d + 3 * n, strength, (size_t)(3 * n));
    h2d(d + 6 * n, radius, (size_t)n);
    h2d(d + 7 * n, pts, (size_t)(3 * m));
    double* dv = d + 7 * n + 3 * m;
    check(cpg_particles_velocity(ctx, d, d + 3 * n, d + 6 * n, n, d + 7 * n, m, kernel, dv), ctx,
          "particle::velInfl");
    check(cpg_synchronize(ctx), ctx, "shim: synchronize");
    d2h(vel, dv, (size_t)(3 * m));
}

void particles_mutual(const double* pos, const double* strength, const double* radius, int64_t n, double* vel,
                      double* stretch, double* diff) {
    if (n <= 0) return;
    cpg_ctx* ctx = context(0);
    std::lock_guard<std::mutex> l(g_scr_mu);
    cuda_check(cudaSetDevice(0), "device");
    double* d = scratch(0, (size_t)(16 * n));
    h2d(d, pos, (size_t)(3 * n));
    h2d(d + 3 * n, strength, (size_t)(3 * n));
    h2d(d + 6 * n, radius, (size_t)n);
    double *dv = d + 7 * n, *ds = d + 10 * n, *dd = d + 13 * n;
    if (vel)
        check(cpg_particles_velocity(ctx, d, d + 3 * n, d + 6 * n, n, nullptr, n, CPG_VEL_GAUSS_SYM, dv), ctx,
              "particle::velInfl");
    if (stretch || diff)
        check(cpg_particles_stretch_diff(ctx, d, d + 3 * n, d + 6 * n, n, stretch ? ds : nullptr, diff ? dd : nullptr),
              ctx, "particle::vortexStretching");
    check(cpg_synchronize(ctx), ctx, "shim: synchronize");
    if (vel) d2h(vel, dv, (size_t)(3 * n));
    if (stretch) d2h(stretch, ds, (size_t)(3 * n));
    if (diff) d2h(diff, dd, (size_t)(3 * n));
}

// what: 0 velocity at part induced by this (part is the influenced particle), 1 this particle's
// stretching by part, 2 its diffusion by part; zero for the particle itself, as the reference
void particle::pair(const particle* part, int what, double* out) const {
    out[0] = out[1] = out[2] = 0;
    if (part == this) return;
    const double pos[6] = {pos_[0], pos_[1], pos_[2], part->pos_[0], part->pos_[1], part->pos_[2]};
    const double str[6] = {str_[0], str_[1], str_[2], part->str_[0], part->str_[1], part->str_[2]};
    const double rad[2] = {radius, part->radius};
    double r[6];
    if (what == 0) {
        particles_mutual(pos, str, rad, 2, r, nullptr, nullptr);
        std::copy(r + 3, r + 6, out);  // at part, from this
    } else {
        particles_mutual(pos, str, rad, 2, nullptr, what == 1 ? r : nullptr, what == 2 ? r : nullptr);
        std::copy(r, r + 3, out);  // on this, from part
    }
}

void particleFMM::release() {
    if (tree_) cpg_ptree_destroy(tree_);
    tree_ = nullptr;
    if (dev_) cudaFree(dev_);
    dev_ = nullptr;
    n_ = 0;
    index_.clear();
    table_.clear();
    have_table_ = false;
}

particleFMM::~particleFMM() { release(); }

void particleFMM::build(particleOctree* tree) {
    release();
    cpg_ctx* ctx = context(device_);
    const std::vector<particle*>& parts = tree->data();
    n_ = (int64_t)parts.size();
    if (n_ == 0) return;
    std::vector<double> host((size_t)(7 * n_));
    for (int64_t i = 0; i < n_; i++) {
        const particle* p = parts[(size_t)i];
        for (int q = 0; q < 3; q++) {
            host[3 * i + q] = p->pos()[q];
            host[3 * n_ + 3 * i + q] = p->strength()[q];
        }
        host[6 * n_ + i] = p->radius;
        index_[p] = i;
    }
    cuda_check(cudaSetDevice(device_), "device");
    cuda_check(cudaMalloc(&dev_, sizeof(double) * host.size()), "particleFMM::build");
    double* d = (double*)dev_;
    h2d(d, host.data(), host.size());
    check(cpg_ptree_build(ctx, d, d + 3 * n_, d + 6 * n_, n_, tree->maxMembers(), theta_, &tree_), ctx,
          "particleFMM::build");
}

void particleFMM::velocity_points(const double* pts, int64_t m, double* vel) {
    if (m <= 0) return;
    if (!tree_) throw error(CPG_E_INVALID, "particleFMM: build() a tree first");
    cpg_ctx* ctx = context(device_);
    std::lock_guard<std::mutex> l(g_scr_mu);
    cuda_check(cudaSetDevice(device_), "device");
    double* d = scratch(device_, (size_t)(6 * m));
    h2d(d, pts, (size_t)(3 * m));
    check(cpg_bh_velocity_points(tree_, d, m, d + 3 * m), ctx, "particleFMM::barnesHutVel");
    check(cpg_synchronize(ctx), ctx, "shim: synchronize");
    d2h(vel, d + 3 * m, (size_t)(3 * m));
}

const double* particleFMM::row(const particle* part, int what) {
    if (!tree_) throw error(CPG_E_INVALID, "particleFMM: build() a tree first");
    auto it = index_.find(part);
    if (it == index_.end()) throw error(CPG_E_INVALID, "particleFMM: particle not in the tree");
    if (!have_table_) {  // velocity, stretching and diffusion of every particle, one traversal
        cpg_ctx* ctx = context(device_);
        std::lock_guard<std::mutex> l(g_scr_mu);
        cuda_check(cudaSetDevice(device_), "device");
        double* d = scratch(device_, (size_t)(9 * n_));
        check(cpg_bh_particles(tree_, d, d + 3 * n_, d + 6 * n_), ctx, "particleFMM::barnesHut");
        check(cpg_synchronize(ctx), ctx, "shim: synchronize");
        std::vector<double> h((size_t)(9 * n_));
        d2h(h.data(), d, h.size());
        table_.resize((size_t)(9 * n_));
        for (int64_t i = 0; i < n_; i++)
            for (int w = 0; w < 3; w++)
                for (int q = 0; q < 3; q++) table_[9 * i + 3 * w + q] = h[3 * n_ * w + 3 * i + q];
        have_table_ = true;
    }
    return &table_[(size_t)(9 * it->second + 3 * what)];
}

}  // namespace shim
}  // namespace cpg
