// The vortex-particle case driven step by step (include/cpanel_vp.h, cpg_vpcase_*).
//
// Restates cpCaseVP::run (CPanel/cpCaseVP.cpp:26-117), including its Trefftz-plane early
// stop (cpg_vpcase_step advances a given number of steps).  State lives on the
// device; the host keeps the shedding bookkeeping, builds the octree after the strength
// update (as the reference does) and solves the small sequential pieces of the shedding.
//
// Precision: CPG_PLAIN_FP64 is the reference method in FP64.  CPG_MIXED evaluates far
// particle nodes and far panels in FP32 (the near field -- leaf members, panels within
// five lengths -- stays FP64, and every near/far decision equals the FP64 one) and
// replaces the per-step BiCGSTAB by the FP32 LU of A (factored once; A does not change)
// refined against the FP64 matrix, held as a float pair, to a relative residual of
// 1e-12 (the LU is turned once into an FP32 inverse, so each pass is one matrix-vector
// product), falling back to BiCGSTAB for a step whose refinement stalls.  The shedding
// and its bookkeeping are the same in both.
//
// Per step (timestep >= 3):
//   convectParticles   particle term (Barnes-Hut on the previous step's tree, or direct
//                      Gaussian sums) + panel/filament term, AB2 (k_vp_convect);
//   collapseBufferWake edge strengths on the host, RK4 positions from batched device
//                      evaluations of the whole velocity field, radius from neighbours;
//   convectBufferWake  second-row doublets from their parents (k_vp_buffer);
//   particleStrengthUpdate stretching/diffusion (Barnes-Hut or direct) + panel
//                      stretching, AB2 (k_vp_strength);
//   octree rebuild, setSourceStrengthsVP, solveVPmatrixEq (FP64 BiCGSTAB on the device
//   with the reference's tolerance; the same A every step).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/cpanel_gpu.h"
#include "../../include/cpanel_vp.h"
#include "assemble.h"
#include "mesh.h"
#include "octree.h"
#include "particles.h"
#include "post.h"
#include "vpgeom.h"
#include "vpkern.h"

namespace cpg {
// context accessors (api.cpp): last error message, stream
void ctx_set_error(cpg_ctx* ctx, const std::string& msg);
cudaStream_t ctx_stream(cpg_ctx* ctx);
int ctx_particle_precision(cpg_ctx* ctx);
}  // namespace cpg

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b, cudaStream_t s, bool keep = false) {
        if (b <= bytes) return cudaSuccess;
        size_t nb = std::max(b, bytes * 2);
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, nb);
        if (e != cudaSuccess) return e;
        if (keep && p && bytes) {
            e = cudaMemcpyAsync(q, p, bytes, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                cudaFree(q);
                return e;
            }
        }
        if (p) cudaFree(p);
        p = q;
        bytes = nb;
        return cudaSuccess;
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

template <typename T>
cudaError_t up(Buf& b, const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = b.ensure(std::max<size_t>(1, v.size() * sizeof(T)), s);
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

// particle::velInfl(POI), CPanel/particle.cpp:60-77 (host; particles shed earlier in the
// same collapse, direct branch only)
void velGaussPointHost(const double* p, const double* a, double r, const double* poi, double* out) {
    double ddx = p[0] - poi[0], ddy = p[1] - poi[1], ddz = p[2] - poi[2];
    if (std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz) == 0) return;
    double sig = 1.5 * r;
    double d[3] = {poi[0] - p[0], poi[1] - p[1], poi[2] - p[2]};
    double rho = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / sig;
    double K = (1 / (4 * kPi * rho) * std::erf(rho / std::pow(2, 0.5)) -
                1 / (std::pow(2 * kPi, 1.5)) * std::exp(-0.5 * rho * rho)) /
               (rho * rho);
    double f = -1 / std::pow(sig, 3) * K;
    out[0] += f * (d[1] * a[2] - d[2] * a[1]);
    out[1] += f * (d[2] * a[0] - d[0] * a[2]);
    out[2] += f * (d[0] * a[1] - d[1] * a[0]);
}

}  // namespace

struct cpg_vpcase {
    cpg_ctx* ctx = nullptr;
    cudaStream_t s = nullptr;
    cpg::VPGeom G;
    double V = 1, alpha = 0, beta = 0, cref = 1, dt = 0;
    bool accelerate = true;
    double vinf[3] = {0, 0, 0};
    int timestep = 0;
    int64_t n = 0, n1 = 0, n2 = 0;
    int64_t np = 0;                  // particles
    int64_t last_iters = 0;
    std::vector<int32_t> shed, parent;
    // device: geometry and matrices
    Buf rec, q1, q2, widx, wcoef, par, A, B, C, work;
    // device: strengths
    Buf sigma, mu, mu1, prev1, mu2, prev2, rhs, fil, vcent;
    Buf vtot;  // onset velocity at the body centres (VinfPlusVecPot) of the last source strengths
    // surface pass (cpCaseVP::compVelocity): CHTLS clusters of the body with the buffer wake's
    // trailing-edge parents, weights built on the first call
    cpg::HostMesh H;
    cpg::PostTables PT;
    bool post_ready = false;
    Buf p_bez, p_clp, p_cli, p_tip, p_ts, p_F3, p_F2, p_mode, p_cs, p_work, p_out;
    // device: particles
    Buf pos, str, rad, pvel, pstr, packed, tP, tQ, tS, tD, tPan;
    // device: tree
    cpg::ParticleTree T;
    bool tree_built = false;
    Buf tnodes, tperm, tslots;
    // device: shedding evaluation points; scratch of the chunked panel kernels and of the
    // source-split direct sums
    Buf spts, sout, scr, dsplit;
    std::vector<double> filh;  // host copy of the filaments (8 per w2 panel)
    bool have_fil = false;
    // Trefftz plane (cpCase CL_trefftz / CD_trefftz) and the early stop
    double Sref = 1, PG = 1;
    double CLt = 0, CDt = 0;
    bool converged = false;
    bool run_all = false;  // keep stepping after the check has fired
    // mixed precision: FP32 far fields, LU-refined solve
    int precision = CPG_PLAIN_FP64;
    Buf fnodes, A32, Alo, LU, bad, Ainv;
    cpg::LuGraphs lug;
    int64_t fallbacks = 0;  // steps whose refinement stalled and that BiCGSTAB solved
    bool mixed() const { return precision == CPG_MIXED; }
    const cpg::BHNodeF* fn() const { return mixed() ? fnodes.as<cpg::BHNodeF>() : nullptr; }
};

namespace {

// wind-to-body transform of cpCase::windToBody, CPanel/cpCase.cpp:142-165
void wind_to_body(double V, double a, double b, double* out) {
    a *= kPi / 180;
    b *= kPi / 180;
    double T[3][3] = {{std::cos(a) * std::cos(b), std::cos(a) * std::sin(b), -std::sin(a)},
                      {-std::sin(b), std::cos(b), 0},
                      {std::sin(a) * std::cos(b), std::sin(a) * std::sin(b), std::cos(a)}};
    for (int q = 0; q < 3; q++) out[q] = T[q][0] * V + T[q][1] * 0 + T[q][2] * 0;
}

cudaError_t pack_current(cpg_vpcase& S) {
    cudaError_t e = S.packed.ensure(sizeof(cpg::BHPart) * std::max<int64_t>(1, S.np), S.s);
    if (e != cudaSuccess) return e;
    return cpg::launch_pack_parts(S.pos.as<double>(), S.str.as<double>(), S.rad.as<double>(), S.np,
                                  S.packed.as<cpg::BHPart>(), S.s);
}

cudaError_t refresh_slots(cpg_vpcase& S) {
    return cpg::launch_refresh_slots(S.tperm.as<int64_t>(), (int64_t)S.T.perm.size(), S.pos.as<double>(),
                                     S.str.as<double>(), S.rad.as<double>(), S.tslots.as<cpg::BHPart>(), S.s);
}

// direct sums over n sources at m targets, source ranges split across blocks when the
// targets alone would leave the GPU idle
cudaError_t direct_sums(cpg_vpcase& S, int vk, bool st, bool df, int64_t n, const cpg::BHPart* tgt, const double* pts,
                   int64_t m, double* vel, double* str, double* dif) {
    const int64_t need = cpg::direct_scratch_doubles(n, m);
    cudaError_t e;
    if (need > 0 && (e = S.dsplit.ensure(sizeof(double) * need, S.s)) != cudaSuccess) return e;
    return cpg::launch_direct(vk, st, df, S.packed.as<cpg::BHPart>(), n, tgt, pts, m, cpg::vp_constants(), vel, str,
                              dif, S.s, S.dsplit.as<double>(), need);
}

// particle velocity term at m points: Barnes-Hut (algebraic) or direct Gaussian sums over
// the first nsrc particles
cudaError_t particle_term_points(cpg_vpcase& S, bool bh, const double* pts, int64_t m, int64_t nsrc, double* out) {
    if (m <= 0) return cudaSuccess;
    if (bh) {
        int nn = (int)S.T.nodes.size();
        if (nn <= 1) return cudaMemsetAsync(out, 0, sizeof(double) * 3 * m, S.s);
        cudaError_t e = refresh_slots(S);
        if (e != cudaSuccess) return e;
        return cpg::launch_bh_points(S.tnodes.as<cpg::BHNode>(), S.fn(), nn, S.tslots.as<cpg::BHPart>(), S.T.theta, pts, m,
                                     cpg::vp_constants(), out, S.s);
    }
    if (nsrc <= 0) return cudaMemsetAsync(out, 0, sizeof(double) * 3 * m, S.s);
    return direct_sums(S, 2, false, false, nsrc, nullptr, pts, m, out, nullptr, nullptr);
}

cudaError_t ensure_particles(cpg_vpcase& S, int64_t cap) {
    cudaError_t e;
    Buf* bufs3[] = {&S.pos, &S.str, &S.pvel, &S.pstr};
    for (Buf* b : bufs3)
        if ((e = b->ensure(sizeof(double) * 3 * cap, S.s, true)) != cudaSuccess) return e;
    if ((e = S.rad.ensure(sizeof(double) * cap, S.s, true)) != cudaSuccess) return e;
    Buf* tmp[] = {&S.tP, &S.tQ, &S.tS, &S.tD, &S.tPan};
    for (Buf* b : tmp)
        if ((e = b->ensure(sizeof(double) * 3 * cap, S.s)) != cudaSuccess) return e;
    return cudaSuccess;
}

constexpr double kVPRefineTol = 1e-12;

// solveMatrixEq / solveVPmatrixEq, CPanel/cpCaseVP.cpp:231-301
cudaError_t solve(cpg_vpcase& S, bool with_c) {
    cudaError_t e = cpg::gemm_fp64_nk(S.B.as<double>(), S.n, 1, S.sigma.as<double>(), S.rhs.as<double>(), -1.0,
                                      S.work.p, S.s);
    if (e != cudaSuccess) return e;
    if (with_c && (e = cpg::vp_launch_rhs_c(S.C.as<double>(), S.n, S.n2, S.mu2.as<double>(), S.rhs.as<double>(), S.s)) !=
                      cudaSuccess)
        return e;
    cpg::SolveStats st;
    bool done = false;
    if (S.mixed()) {
        e = cpg::solve_lu_refined(&S.lug, S.A32.as<float>(), S.Alo.as<float>(), nullptr, S.n, 1,
                                  S.rhs.as<double>(), S.mu.as<double>(), S.work.p, kVPRefineTol, 8, &st, S.s,
                                  S.Ainv.as<float>());
        if (e != cudaSuccess) return e;
        done = st.residual_max <= kVPRefineTol;
        S.last_iters = st.refinements;
        if (!done) S.fallbacks++;
    }
    if (!done) {
        st = cpg::SolveStats();
        e = cpg::solve_fp64(S.A.as<double>(), S.n, 1, S.rhs.as<double>(), S.mu.as<double>(), S.work.p,
                            2.220446049250313e-16, 2 * S.n, &st, S.s);
        if (e != cudaSuccess) return e;
        S.last_iters = st.iters_max;
    }
    return cpg::vp_launch_wake_mu(S.mu.as<double>(), S.widx.as<int32_t>(), S.wcoef.as<double>(), S.n1,
                                  S.mu1.as<double>(), S.prev1.as<double>(), with_c ? 1 : 0, S.s);
}

// the whole velocity field at host points (cpCaseVP::velocityInflFromEverything(POI),
// CPanel/cpCaseVP.cpp:642-678), particle term over the first nsrc particles
cudaError_t field_at(cpg_vpcase& S, bool bh, const std::vector<double>& pts, int64_t nsrc, std::vector<double>& out) {
    int64_t m = (int64_t)pts.size() / 3;
    out.assign(3 * m, 0.0);
    if (m == 0) return cudaSuccess;
    cudaError_t e;
    if ((e = S.spts.ensure(sizeof(double) * 3 * m, S.s)) != cudaSuccess) return e;
    if ((e = S.sout.ensure(sizeof(double) * 6 * m, S.s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S.spts.p, pts.data(), sizeof(double) * 3 * m, cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return e;
    double* P = S.sout.as<double>();
    double* Q = P + 3 * m;
    if ((e = particle_term_points(S, bh, S.spts.as<double>(), m, nsrc, P)) != cudaSuccess) return e;
    if ((e = S.scr.ensure(sizeof(double) * cpg::vp_scratch_doubles(m, S.n), S.s)) != cudaSuccess) return e;
    if ((e = cpg::vp_launch_panel_vel(S.rec.as<double>(), S.sigma.as<double>(), S.mu.as<double>(), S.n,
                                      S.q1.as<double>(), S.mu1.as<double>(), S.n1, S.q2.as<double>(),
                                      S.mu2.as<double>(), S.n2, S.fil.as<double>(), S.have_fil ? S.n2 : 0,
                                      S.spts.as<double>(), m, 0.0, Q, S.scr.as<double>(), S.s, S.mixed())) !=
        cudaSuccess)
        return e;
    std::vector<double> h(6 * m);
    if ((e = cudaMemcpyAsync(h.data(), P, sizeof(double) * 6 * m, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return e;
    for (int64_t i = 0; i < m; i++)
        for (int k = 0; k < 3; k++) out[3 * i + k] = (S.vinf[k] + h[3 * i + k]) + h[3 * m + 3 * i + k];
    return cudaSuccess;
}

// cpCaseVP::collapseBufferWake, CPanel/cpCaseVP.cpp:315-368
cudaError_t collapse(cpg_vpcase& S) {
    const cpg::VPGeom& G = S.G;
    const int64_t n2 = S.n2;
    std::vector<double> m2(n2), p2(n2);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(m2.data(), S.mu2.p, sizeof(double) * n2, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(p2.data(), S.prev2.p, sizeof(double) * n2, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return e;
    auto node = [&](int id, int k) { return G.nodes[3 * id + k]; };
    // strengths: wakePanel::edgeStrength over edges 1..3 not used by an earlier panel
    std::vector<int> used;
    std::vector<double> strength(3 * n2, 0.0);
    for (int64_t k = 0; k < n2; k++) {
        const int32_t* eio = &G.eio[4 * k];
        const int32_t* pio = &G.pio[4 * k];
        double acc[3] = {0, 0, 0};
        for (int j = 1; j < 4; j++) {
            if (std::find(used.begin(), used.end(), eio[j]) != used.end()) continue;
            used.push_back(eio[j]);
            int ri, rj;
            double coef;
            if (j == 2) {
                rj = pio[2];
                ri = pio[3];
                coef = m2[k] - p2[k];
            } else {
                int o = G.nbr_eio[2 * k + (j == 1 ? 0 : 1)];
                rj = j == 1 ? pio[1] : pio[3];
                ri = j == 1 ? pio[2] : pio[0];
                coef = o >= 0 ? m2[k] - m2[o] : m2[k];
            }
            for (int q = 0; q < 3; q++) acc[q] = acc[q] + coef * (node(ri, q) - node(rj, q));
        }
        for (int q = 0; q < 3; q++) strength[3 * k + q] = acc[q];
    }
    // RK4 (cpCaseVP::rungeKuttaStepper, :627-640)
    const bool bh = S.accelerate && S.timestep > 3;
    const int64_t nold = S.np;
    std::vector<double> newpos(3 * n2), radius(n2);
    auto centre = [&](int64_t k, int q) { return G.w2[k * cpg::QF_STRIDE + cpg::QF_C + q]; };
    if (bh) {
        // new particles are in no leaf: all panels advance together, stage by stage
        std::vector<double> X(3 * n2), k1, k2, k3, k4, pts(3 * n2);
        for (int64_t k = 0; k < n2; k++)
            for (int q = 0; q < 3; q++) X[3 * k + q] = centre(k, q);
        if ((e = field_at(S, true, X, nold, k1)) != cudaSuccess) return e;
        for (int64_t i = 0; i < 3 * n2; i++) pts[i] = X[i] + k1[i] * S.dt / 2;
        if ((e = field_at(S, true, pts, nold, k2)) != cudaSuccess) return e;
        for (int64_t i = 0; i < 3 * n2; i++) pts[i] = X[i] + k2[i] * S.dt / 2;
        if ((e = field_at(S, true, pts, nold, k3)) != cudaSuccess) return e;
        for (int64_t i = 0; i < 3 * n2; i++) pts[i] = X[i] + k3[i] * S.dt;
        if ((e = field_at(S, true, pts, nold, k4)) != cudaSuccess) return e;
        for (int64_t i = 0; i < 3 * n2; i++)
            newpos[i] = X[i] + S.dt * (k1[i] / 6 + k2[i] / 3 + k3[i] / 3 + k4[i] / 6);
    } else {
        // direct sums: a particle shed earlier in this collapse already acts on the next
        // panel's RK4 stages, so panels go one after another
        for (int64_t k = 0; k < n2; k++) {
            double X[3] = {centre(k, 0), centre(k, 1), centre(k, 2)};
            double kk[4][3];
            double P[3] = {X[0], X[1], X[2]};
            for (int st = 0; st < 4; st++) {
                if (st > 0)
                    for (int q = 0; q < 3; q++)
                        P[q] = st < 3 ? X[q] + kk[st - 1][q] * S.dt / 2 : X[q] + kk[st - 1][q] * S.dt;
                std::vector<double> pts(P, P + 3), v;
                if ((e = field_at(S, false, pts, nold, v)) != cudaSuccess) return e;
                for (int64_t j = 0; j < k; j++)
                    velGaussPointHost(&newpos[3 * j], &strength[3 * j], radius[j], P, v.data());
                for (int q = 0; q < 3; q++) kk[st][q] = v[q];
            }
            for (int q = 0; q < 3; q++)
                newpos[3 * k + q] = X[q] + S.dt * (kk[0][q] / 6 + kk[1][q] / 3 + kk[2][q] / 3 + kk[3][q] / 6);
            // wakePanel::getPartRadius, CPanel/wakePanel.cpp:228-249
            double sum = 0;
            int cnt = 0;
            for (int s_ = 0; s_ < 2; s_++) {
                int o = G.nbr_raw[2 * k + s_];
                if (o < 0) continue;
                double d[3];
                for (int q = 0; q < 3; q++) d[q] = (centre(k, q) + S.dt * S.vinf[q]) - (centre(o, q) + S.dt * S.vinf[q]);
                sum += std::abs(std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
                cnt++;
            }
            radius[k] = (0.0 + sum) / static_cast<double>(cnt);
        }
    }
    if (bh)
        for (int64_t k = 0; k < n2; k++) {
            double sum = 0;
            int cnt = 0;
            for (int s_ = 0; s_ < 2; s_++) {
                int o = G.nbr_raw[2 * k + s_];
                if (o < 0) continue;
                double d[3];
                for (int q = 0; q < 3; q++) d[q] = (centre(k, q) + S.dt * S.vinf[q]) - (centre(o, q) + S.dt * S.vinf[q]);
                sum += std::abs(std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
                cnt++;
            }
            radius[k] = (0.0 + sum) / static_cast<double>(cnt);
        }
    // append the new particles
    int64_t nnew = nold + n2;
    if ((e = ensure_particles(S, nnew)) != cudaSuccess) return e;
    std::vector<double> zero(3 * n2, 0.0);
    if ((e = cudaMemcpyAsync(S.pos.as<double>() + 3 * nold, newpos.data(), sizeof(double) * 3 * n2,
                             cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(S.str.as<double>() + 3 * nold, strength.data(), sizeof(double) * 3 * n2,
                             cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(S.rad.as<double>() + nold, radius.data(), sizeof(double) * n2, cudaMemcpyHostToDevice,
                             S.s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(S.pvel.as<double>() + 3 * nold, zero.data(), sizeof(double) * 3 * n2,
                             cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(S.pstr.as<double>() + 3 * nold, zero.data(), sizeof(double) * 3 * n2,
                             cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return e;
    for (int64_t k = 0; k < n2; k++) {
        S.shed.push_back(S.timestep);
        S.parent.push_back((int32_t)k);
    }
    S.np = nnew;
    // filaments: created at the first collapse on the downstream edges, strength -mu
    if (!S.have_fil) {
        S.filh.assign(8 * n2, 0.0);
        for (int64_t k = 0; k < n2; k++) {
            const int32_t* pio = &G.pio[4 * k];
            for (int q = 0; q < 3; q++) {
                S.filh[8 * k + q] = node(pio[2], q);
                S.filh[8 * k + 3 + q] = node(pio[3], q);
            }
        }
        S.have_fil = true;
    }
    for (int64_t k = 0; k < n2; k++) S.filh[8 * k + 6] = -m2[k];
    if ((e = S.fil.ensure(sizeof(double) * 8 * n2, S.s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S.fil.p, S.filh.data(), sizeof(double) * 8 * n2, cudaMemcpyHostToDevice, S.s)) !=
        cudaSuccess)
        return e;
    return cudaStreamSynchronize(S.s);
}

cudaError_t build_tree(cpg_vpcase& S) {
    std::vector<double> hp(3 * S.np), hs(3 * S.np), hr(S.np);
    cudaError_t e;
    if (S.np > 0) {
        if ((e = cudaMemcpyAsync(hp.data(), S.pos.p, sizeof(double) * 3 * S.np, cudaMemcpyDeviceToHost, S.s)) !=
            cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(hs.data(), S.str.p, sizeof(double) * 3 * S.np, cudaMemcpyDeviceToHost, S.s)) !=
            cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(hr.data(), S.rad.p, sizeof(double) * S.np, cudaMemcpyDeviceToHost, S.s)) !=
            cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return e;
    }
    cpg::build_particle_tree(hp.data(), hs.data(), hr.data(), S.np, 10, 0.5, S.T);
    if ((e = up(S.tnodes, S.T.nodes, S.s)) != cudaSuccess) return e;
    if ((e = up(S.fnodes, S.T.fnodes, S.s)) != cudaSuccess) return e;
    if ((e = up(S.tperm, S.T.perm, S.s)) != cudaSuccess) return e;
    if ((e = S.tslots.ensure(sizeof(cpg::BHPart) * std::max<int64_t>(1, S.np), S.s)) != cudaSuccess) return e;
    S.tree_built = true;
    return cudaStreamSynchronize(S.s);
}

struct T3 {
    double x, y, z;
};
inline T3 tsub(T3 a, T3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline T3 tadd(T3 a, T3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline T3 tmul(double s, T3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double tnorm(T3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline T3 tunit(T3 a) {  // Eigen's normalized(): unchanged when zero
    double z = a.x * a.x + a.y * a.y + a.z * a.z;
    if (z > 0) {
        double r = std::sqrt(z);
        return {a.x / r, a.y / r, a.z / r};
    }
    return a;
}

// wake::wakeStrength, CPanel/wake.cpp:478-506: (mu_upper - mu_lower) interpolated in y
// between the wake lines (wakeLine::getStrength, CPanel/wakeLine.cpp:26-29)
double wake_strength(const cpg::VPGeom& G, const std::vector<double>& mu, double y) {
    const size_t L = G.line_y.size();
    size_t a = 0, b = 1;
    if (y < G.line_y[1]) {
        a = 0;
        b = 1;
    } else if (y >= G.line_y[L - 1]) {
        a = L - 2;
        b = L - 1;
    } else {
        for (size_t i = 1; i + 1 < L; i++)
            if (G.line_y[i] <= y && G.line_y[i + 1] > y) {
                a = i;
                b = i + 1;
            }
    }
    double interp = (y - G.line_y[a]) / (G.line_y[b] - G.line_y[a]);
    double sa = mu[G.line_up[a]] - mu[G.line_lo[a]];
    double sb = mu[G.line_up[b]] - mu[G.line_lo[b]];
    return sa + interp * (sb - sa);
}

// wake::trefftzPlaneVP, CPanel/wake.cpp:191-320 (particlePntInWakeY :322-351,
// stretchFactor :353-361) over the one buffer wake, scaled as in
// cpCaseVP::trefftzPlaneAnalysisVP (CPanel/cpCaseVP.cpp:418-429).  The particle row shed
// at step ceil_even(timestep)/2 + 2 is ordered by its parents' centre y and joined into
// a curve; 3N points spaced evenly along it carry dPhi (the wake strength at the
// interpolated parent y times the stretch of the row) and the downwash |w| of all
// particles (Gaussian sums on the device); Simpson's rule integrates both.  A row of
// fewer than two particles (undefined in the reference) gives zero.
cudaError_t trefftz(cpg_vpcase& S, double& CL, double& CD) {
    CL = CD = 0;
    const cpg::VPGeom& G = S.G;
    int steps = S.timestep;
    if (steps % 2 != 0) steps++;
    const int row = steps / 2 + 2;
    std::vector<int64_t> unsorted;
    for (int64_t i = 0; i < S.np; i++)
        if (S.shed[i] == row) unsorted.push_back(i);
    if (unsorted.size() < 2) return cudaSuccess;
    cudaError_t e;
    std::vector<double> hp(3 * S.np), mu(S.n);
    if ((e = cudaMemcpyAsync(hp.data(), S.pos.p, sizeof(double) * 3 * S.np, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(mu.data(), S.mu.p, sizeof(double) * S.n, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return e;
    auto pos = [&](int64_t i) { return T3{hp[3 * i], hp[3 * i + 1], hp[3 * i + 2]}; };
    auto pc = [&](int64_t i) {
        const double* c = &G.w2[(size_t)S.parent[i] * cpg::QF_STRIDE + cpg::QF_C];
        return T3{c[0], c[1], c[2]};
    };
    // repeated extraction of the lowest parent y (first one on ties)
    std::vector<int64_t> sorted;
    while (!unsorted.empty()) {
        size_t li = 0;
        double lowest = pc(unsorted[0]).y;
        for (size_t i = 0; i < unsorted.size(); i++)
            if (pc(unsorted[i]).y < lowest) {
                lowest = pc(unsorted[i]).y;
                li = i;
            }
        sorted.push_back(unsorted[li]);
        unsorted.erase(unsorted.begin() + (long)li);
    }
    double Slen = 0;
    for (size_t i = 0; i + 1 < sorted.size(); i++) Slen += tnorm(tsub(pos(sorted[i + 1]), pos(sorted[i])));
    const int npts = (int)sorted.size() * 3;
    const double step = Slen / npts;
    std::vector<T3> pts{pos(sorted[0])};
    std::vector<int64_t> p1{sorted[0]}, p2{sorted[1]};
    T3 next = pos(sorted[1]);
    size_t ni = 1;
    T3 pt = pos(sorted[0]);
    for (int i = 1; i < npts; i++) {
        if (step < tnorm(tsub(next, pt))) {
            T3 q = tadd(pt, tmul(step, tunit(tsub(next, pt))));
            pts.push_back(q);
            p1.push_back(sorted[ni - 1]);
            p2.push_back(sorted[ni]);
            pt = q;
        } else {
            double cov = tnorm(tsub(next, pt));
            if (ni + 1 >= sorted.size()) break;  // rounding at the curve's end
            pt = next;
            next = pos(sorted[ni + 1]);
            ni++;
            T3 q = tadd(pt, tmul(step - cov, tunit(tsub(next, pt))));
            pts.push_back(q);
            p1.push_back(sorted[ni - 1]);
            p2.push_back(sorted[ni]);
            pt = q;
        }
    }
    // downwash of all particles at the curve points (Gaussian sums, as particle::velInfl)
    const int64_t m = (int64_t)pts.size();
    std::vector<double> hq(3 * m), hv(3 * m);
    for (int64_t i = 0; i < m; i++) {
        hq[3 * i] = pts[i].x;
        hq[3 * i + 1] = pts[i].y;
        hq[3 * i + 2] = pts[i].z;
    }
    if ((e = S.spts.ensure(sizeof(double) * 3 * m, S.s)) != cudaSuccess) return e;
    if ((e = S.sout.ensure(sizeof(double) * 6 * m, S.s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S.spts.p, hq.data(), sizeof(double) * 3 * m, cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return e;
    if ((e = pack_current(S)) != cudaSuccess) return e;
    if ((e = particle_term_points(S, false, S.spts.as<double>(), m, S.np, S.sout.as<double>())) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(hv.data(), S.sout.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return e;
    std::vector<double> Cl(npts + 1, 0.0), Cd(npts + 1, 0.0);
    for (int64_t i = 1; i < m; i++) {
        T3 A = pos(p1[i]), B = pos(p2[i]);
        double d = tnorm(tsub(B, A)), a = tnorm(tsub(pts[i], A)), b = tnorm(tsub(B, pts[i]));
        double yA = pc(p1[i]).y, yB = pc(p2[i]).y, y;
        if (a < 1e-10)
            y = yA;
        else if (b < 1e-10)
            y = yB;
        else
            y = yA + (a / d) * (yB - yA);
        double fac = tnorm(tsub(pc(p2[i]), pc(p1[i]))) / tnorm(tsub(B, A));
        double w = std::abs(hv[3 * i + 2]);
        double dphi = -wake_strength(G, mu, y) * fac;
        Cl[i] = 2 * dphi / (S.V * S.Sref);
        Cd[i] = dphi * w / (S.V * S.V * S.Sref);
    }
    for (int i = 0; i < (int)Cl.size() - 2; i += 2) {
        CL += 1.0 / 3 * step * (Cl[i] + 4 * Cl[i + 1] + Cl[i + 2]);
        CD += 1.0 / 3 * step * (Cd[i] + 4 * Cd[i + 1] + Cd[i + 2]);
    }
    CL /= S.PG;
    CD /= std::pow(S.PG, 2);
    return cudaSuccess;
}

// cpCaseVP::solutionConvergence, CPanel/cpCaseVP.cpp:204-229 (steady case)
cudaError_t convergence_check(cpg_vpcase& S) {
    if (S.timestep < 5) return cudaSuccess;
    double prevCL = S.CLt, prevCD = S.CDt;
    cudaError_t e = trefftz(S, S.CLt, S.CDt);
    if (e != cudaSuccess) return e;
    double dCD = std::abs((S.CDt - prevCD) / prevCD), dCL = std::abs((S.CLt - prevCL) / prevCL);
    if (dCL < 0.0001 && dCD < 0.0001) S.converged = true;  // stays set (a run_all_steps case goes on)
    return cudaSuccess;
}

cudaError_t step_once(cpg_vpcase& S) {
    cudaError_t e;
    const double vinf[3] = {S.vinf[0], S.vinf[1], S.vinf[2]};
    if (S.timestep == 0) {  // setSourceStrengths + solveMatrixEq
        if ((e = cpg::vp_launch_sigma(S.rec.as<double>(), S.n, nullptr, nullptr, 0, vinf, S.sigma.as<double>(),
                                      S.vtot.as<double>(), S.s)) != cudaSuccess)
            return e;
        if ((e = solve(S, false)) != cudaSuccess) return e;
        S.timestep = 1;
        return cudaStreamSynchronize(S.s);
    }
    S.timestep++;
    if (S.timestep == 2) {
        if ((e = cpg::vp_launch_buffer(S.mu1.as<double>(), S.par.as<int32_t>(), S.n2, S.mu2.as<double>(),
                                       S.prev2.as<double>(), S.s)) != cudaSuccess)
            return e;
        if ((e = solve(S, true)) != cudaSuccess) return e;
        return cudaStreamSynchronize(S.s);
    }
    const cpg::VPConst c = cpg::vp_constants();
    // convectParticles
    if (S.np > 0) {
        if ((e = pack_current(S)) != cudaSuccess) return e;
        const int64_t m = S.np;
        if (S.accelerate && S.timestep > 2 && S.tree_built && S.T.nodes.size() > 1) {
            if ((e = refresh_slots(S)) != cudaSuccess) return e;
            if ((e = cpg::launch_bh_targets(S.tnodes.as<cpg::BHNode>(), S.fn(), (int)S.T.nodes.size(),
                                            S.tslots.as<cpg::BHPart>(), S.T.theta, S.packed.as<cpg::BHPart>(), m, c,
                                            S.tP.as<double>(), nullptr, nullptr, S.s)) != cudaSuccess)
                return e;
        } else if (S.accelerate && S.timestep > 2) {
            if ((e = cudaMemsetAsync(S.tP.p, 0, sizeof(double) * 3 * m, S.s)) != cudaSuccess) return e;
        } else {
            if ((e = direct_sums(S, 2, false, false, m, S.packed.as<cpg::BHPart>(), nullptr, m, S.tP.as<double>(), nullptr,
                            nullptr)) != cudaSuccess)
                return e;
        }
        if ((e = S.scr.ensure(sizeof(double) * cpg::vp_scratch_doubles(m, S.n), S.s)) != cudaSuccess) return e;
        if ((e = cpg::vp_launch_panel_vel(S.rec.as<double>(), S.sigma.as<double>(), S.mu.as<double>(), S.n,
                                          S.q1.as<double>(), S.mu1.as<double>(), S.n1, S.q2.as<double>(),
                                          S.mu2.as<double>(), S.n2, S.fil.as<double>(), S.have_fil ? S.n2 : 0,
                                          S.pos.as<double>(), m, 12 * S.cref, S.tQ.as<double>(), S.scr.as<double>(),
                                          S.s, S.mixed())) != cudaSuccess)
            return e;
        if ((e = cpg::vp_launch_convect(S.pos.as<double>(), S.pvel.as<double>(), S.tP.as<double>(), S.tQ.as<double>(), m,
                                        vinf, S.cref, S.dt, S.s)) != cudaSuccess)
            return e;
    }
    // collapseBufferWake (the direct branch sums over the current particles, packed here)
    if ((e = pack_current(S)) != cudaSuccess) return e;
    if ((e = collapse(S)) != cudaSuccess) return e;
    // convectBufferWake
    if ((e = cpg::vp_launch_buffer(S.mu1.as<double>(), S.par.as<int32_t>(), S.n2, S.mu2.as<double>(),
                                   S.prev2.as<double>(), S.s)) != cudaSuccess)
        return e;
    // particleStrengthUpdate
    if (S.np > 0) {
        const int64_t m = S.np;
        if ((e = pack_current(S)) != cudaSuccess) return e;
        bool bh = S.accelerate && S.timestep > 3 && S.tree_built;
        if (bh && S.T.nodes.size() > 1) {
            if ((e = refresh_slots(S)) != cudaSuccess) return e;
            if ((e = cpg::launch_bh_targets(S.tnodes.as<cpg::BHNode>(), S.fn(), (int)S.T.nodes.size(),
                                            S.tslots.as<cpg::BHPart>(), S.T.theta, S.packed.as<cpg::BHPart>(), m, c,
                                            nullptr, S.tS.as<double>(), S.tD.as<double>(), S.s)) != cudaSuccess)
                return e;
        } else if (bh) {
            if ((e = cudaMemsetAsync(S.tS.p, 0, sizeof(double) * 3 * m, S.s)) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(S.tD.p, 0, sizeof(double) * 3 * m, S.s)) != cudaSuccess) return e;
        } else {
            if ((e = direct_sums(S, 0, true, true, m, S.packed.as<cpg::BHPart>(), nullptr, m, nullptr, S.tS.as<double>(),
                            S.tD.as<double>())) != cudaSuccess)
                return e;
        }
        if ((e = S.scr.ensure(sizeof(double) * cpg::vp_scratch_doubles(m, S.n), S.s)) != cudaSuccess) return e;
        if ((e = cpg::vp_launch_stretch_panels(S.rec.as<double>(), S.sigma.as<double>(), S.mu.as<double>(), S.n,
                                               S.q1.as<double>(), S.mu1.as<double>(), S.n1, S.pos.as<double>(),
                                               S.str.as<double>(), m, 12 * S.cref, S.tPan.as<double>(),
                                               S.scr.as<double>(), S.s, S.mixed())) != cudaSuccess)
            return e;
        if ((e = cpg::vp_launch_strength(S.pos.as<double>(), S.str.as<double>(), S.pstr.as<double>(), S.tS.as<double>(),
                                         S.tD.as<double>(), S.tPan.as<double>(), m, S.cref, S.dt, S.s)) != cudaSuccess)
            return e;
    }
    // octree rebuild
    if (S.accelerate && (e = build_tree(S)) != cudaSuccess) return e;
    // setSourceStrengthsVP
    if ((e = S.vcent.ensure(sizeof(double) * 3 * S.n, S.s)) != cudaSuccess) return e;
    {
        // the centres of the body panels as points
        std::vector<double> cen(3 * S.n);
        for (int64_t i = 0; i < S.n; i++)
            for (int q = 0; q < 3; q++) cen[3 * i + q] = S.G.body[i * cpg::PF_STRIDE + cpg::PF_C + q];
        if ((e = S.spts.ensure(sizeof(double) * 3 * S.n, S.s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(S.spts.p, cen.data(), sizeof(double) * 3 * S.n, cudaMemcpyHostToDevice, S.s)) !=
            cudaSuccess)
            return e;
        if ((e = pack_current(S)) != cudaSuccess) return e;
        if ((e = particle_term_points(S, S.accelerate, S.spts.as<double>(), S.n, S.np, S.vcent.as<double>())) !=
            cudaSuccess)
            return e;
        if ((e = cpg::vp_launch_sigma(S.rec.as<double>(), S.n, S.vcent.as<double>(), S.fil.as<double>(),
                                      S.have_fil ? S.n2 : 0, vinf, S.sigma.as<double>(), S.vtot.as<double>(), S.s)) !=
            cudaSuccess)
            return e;
    }
    if ((e = solve(S, true)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return e;
    return convergence_check(S);
}

}  // namespace

extern "C" {

int cpg_vpcase_create(cpg_ctx* ctx, const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids,
                      int64_t n_tris, const cpg_vp_params* prm, cpg_vpcase** out) {
    if (!ctx || !out || !prm || !nodes || !tris || !ids || n_nodes <= 0 || n_tris <= 0 || !(prm->V > 0) ||
        !(prm->Sref > 0) || !(std::abs(prm->mach) < 1) ||
        (prm->precision != CPG_PLAIN_FP64 && prm->precision != CPG_MIXED)) {
        if (ctx) cpg::ctx_set_error(ctx, "bad argument");
        return CPG_E_INVALID;
    }
    *out = nullptr;
    cpg_vpcase* Sp = new (std::nothrow) cpg_vpcase();
    if (!Sp) return CPG_E_OOM;
    cpg_vpcase& S = *Sp;
    S.ctx = ctx;
    S.s = cpg::ctx_stream(ctx);
    std::string err = cpg::build_vp_geometry(nodes, n_nodes, tris, ids, n_tris, prm->V, prm->dt, S.G);
    if (!err.empty()) {
        cpg::ctx_set_error(ctx, err);
        delete Sp;
        return CPG_E_BAD_MESH;
    }
    S.V = prm->V;
    S.alpha = prm->alpha;
    S.beta = prm->beta;
    S.cref = prm->cref > 0 ? prm->cref : 1.0;
    S.accelerate = prm->accelerate != 0;
    S.Sref = prm->Sref;
    S.precision = prm->precision;
    S.run_all = prm->run_all_steps != 0;
    S.PG = std::sqrt(1 - std::pow(prm->mach, 2));
    S.dt = S.G.dt;
    wind_to_body(S.V, S.alpha, S.beta, S.vinf);
    S.n = S.G.n_body;
    S.n1 = S.G.n_w1;
    S.n2 = S.G.n_w2;
    const int64_t n = S.n;
    // readTri grows the CHTLS clusters after the buffer wake exists (CPanel/geometry.cpp:473-484),
    // so its first row's trailing-edge parents bound them
    err = cpg::build_mesh(nodes, n_nodes, tris, ids, n_tris, S.H, S.G.line_up.data(), S.G.line_lo.data(),
                          (int64_t)S.G.line_up.size());
    bool same = err.empty() && S.H.n_body == n;
    for (int64_t i = 0; same && i < n * cpg::PF_STRIDE; i++) same = S.H.body[i] == S.G.body[i];
    if (!same) {
        cpg::ctx_set_error(ctx, err.empty() ? "surface topology disagrees with the vortex-particle geometry" : err);
        delete Sp;
        return CPG_E_BAD_MESH;
    }
    auto fail_cuda = [&](cudaError_t e, const char* where) {
        cpg::ctx_set_error(ctx, std::string(where) + ": " + cudaGetErrorString(e));
        cpg_vpcase_destroy(Sp);
        return e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA;
    };
    cudaError_t e;
    if ((e = up(S.rec, S.G.body, S.s)) != cudaSuccess) return fail_cuda(e, "upload");
    if ((e = up(S.q1, S.G.w1, S.s)) != cudaSuccess) return fail_cuda(e, "upload");
    if ((e = up(S.q2, S.G.w2, S.s)) != cudaSuccess) return fail_cuda(e, "upload");
    if ((e = up(S.widx, S.G.widx, S.s)) != cudaSuccess) return fail_cuda(e, "upload");
    if ((e = up(S.wcoef, S.G.wcoef, S.s)) != cudaSuccess) return fail_cuda(e, "upload");
    if ((e = up(S.par, S.G.parent, S.s)) != cudaSuccess) return fail_cuda(e, "upload");
    Buf* sq[] = {&S.A, &S.B};
    for (Buf* b : sq)
        if ((e = b->ensure(sizeof(double) * n * n, S.s)) != cudaSuccess) return fail_cuda(e, "alloc matrices");
    if ((e = S.C.ensure(sizeof(double) * std::max<int64_t>(1, n * S.n2), S.s)) != cudaSuccess)
        return fail_cuda(e, "alloc C");
    if ((e = S.work.ensure(std::max(cpg::solve_fp64_work_bytes(n, 1), cpg::solve_lu_work_bytes(n, 1)), S.s)) !=
        cudaSuccess)
        return fail_cuda(e, "alloc work");
    Buf* vec[] = {&S.sigma, &S.mu, &S.rhs};
    for (Buf* b : vec)
        if ((e = b->ensure(sizeof(double) * n, S.s)) != cudaSuccess) return fail_cuda(e, "alloc");
    if ((e = S.vtot.ensure(sizeof(double) * 3 * n, S.s)) != cudaSuccess) return fail_cuda(e, "alloc");
    Buf* w[] = {&S.mu1, &S.prev1, &S.mu2, &S.prev2};
    for (Buf* b : w) {
        if ((e = b->ensure(sizeof(double) * std::max<int64_t>(1, std::max(S.n1, S.n2)), S.s)) != cudaSuccess)
            return fail_cuda(e, "alloc");
        if ((e = cudaMemsetAsync(b->p, 0, b->bytes, S.s)) != cudaSuccess) return fail_cuda(e, "clear");
    }
    if ((e = S.fil.ensure(sizeof(double) * 8 * std::max<int64_t>(1, S.n2), S.s)) != cudaSuccess)
        return fail_cuda(e, "alloc");
    if ((e = ensure_particles(S, std::max<int64_t>(16, 8 * S.n2))) != cudaSuccess) return fail_cuda(e, "alloc");
    // geometry::setInfCoeff in VP mode: body A/B, first-row wake columns, C
    if ((e = cpg::launch_assemble_fp64(S.rec.as<double>(), n, nullptr, nullptr, nullptr, 0, S.A.as<double>(),
                                       S.B.as<double>(), nullptr, S.s)) != cudaSuccess)
        return fail_cuda(e, "assembly");
    if ((e = cpg::vp_launch_wake_columns(S.rec.as<double>(), n, S.q1.as<double>(), S.widx.as<int32_t>(),
                                         S.wcoef.as<double>(), S.n1, S.A.as<double>(), S.s)) != cudaSuccess)
        return fail_cuda(e, "wake columns");
    if ((e = cpg::vp_launch_cmat(S.rec.as<double>(), n, S.q2.as<double>(), S.n2, S.C.as<double>(), S.s)) != cudaSuccess)
        return fail_cuda(e, "C matrix");
    if (S.mixed()) {  // A as a float pair and its FP32 LU, once (A is the same every step)
        const size_t nn = (size_t)n * n;
        Buf* f32[] = {&S.A32, &S.Alo, &S.LU};
        for (Buf* b : f32)
            if ((e = b->ensure(sizeof(float) * nn, S.s)) != cudaSuccess) return fail_cuda(e, "alloc LU");
        if ((e = S.bad.ensure(sizeof(int), S.s)) != cudaSuccess) return fail_cuda(e, "alloc LU");
        if ((e = cudaMemsetAsync(S.bad.p, 0, sizeof(int), S.s)) != cudaSuccess) return fail_cuda(e, "LU");
        if ((e = cpg::vp_launch_split(S.A.as<double>(), (int64_t)nn, S.A32.as<float>(), S.Alo.as<float>(), S.s)) !=
            cudaSuccess)
            return fail_cuda(e, "split A");
        if ((e = cudaMemcpyAsync(S.LU.p, S.A32.p, sizeof(float) * nn, cudaMemcpyDeviceToDevice, S.s)) != cudaSuccess)
            return fail_cuda(e, "LU");
        if ((e = cpg::lu_factor_fp32(&S.lug, S.LU.as<float>(), n, S.bad.as<int>(), S.s)) != cudaSuccess)
            return fail_cuda(e, "LU factorization");
        // every step solves with the same A: its FP32 inverse makes each refinement pass one
        // matrix-vector product (the factors are not needed after this)
        if ((e = S.Ainv.ensure(sizeof(float) * nn, S.s)) != cudaSuccess) return fail_cuda(e, "alloc inverse");
        if ((e = cpg::lu_invert_fp32(&S.lug, S.LU.as<float>(), n, S.Ainv.as<float>(), S.s)) != cudaSuccess)
            return fail_cuda(e, "inverse");
        S.LU.release();
    }
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return fail_cuda(e, "assembly");
    *out = Sp;
    return CPG_OK;
}

void cpg_vpcase_destroy(cpg_vpcase* S) {
    if (!S) return;
    Buf* all[] = {&S->rec, &S->q1, &S->q2, &S->widx, &S->wcoef, &S->par, &S->A, &S->B, &S->C, &S->work,
                  &S->sigma, &S->mu, &S->mu1, &S->prev1, &S->mu2, &S->prev2, &S->rhs, &S->fil, &S->vcent,
                  &S->pos, &S->str, &S->rad, &S->pvel, &S->pstr, &S->packed, &S->tP, &S->tQ, &S->tS, &S->tD,
                  &S->tPan, &S->tnodes, &S->tperm, &S->tslots, &S->spts, &S->sout, &S->scr, &S->dsplit,
                  &S->fnodes, &S->A32, &S->Alo, &S->LU, &S->bad, &S->Ainv, &S->vtot, &S->p_bez, &S->p_clp,
                  &S->p_cli, &S->p_tip, &S->p_ts, &S->p_F3, &S->p_F2, &S->p_mode, &S->p_cs, &S->p_work, &S->p_out};
    for (Buf* b : all) b->release();
    S->lug.release();
    delete S;
}

int cpg_vpcase_info_get(const cpg_vpcase* S, cpg_vp_info* o) {
    if (!S || !o) return CPG_E_INVALID;
    o->n_body = S->n;
    o->n_w1 = S->n1;
    o->n_w2 = S->n2;
    o->n_particles = S->np;
    o->timestep = S->timestep;
    o->solver_iters = S->last_iters;
    o->dt = S->dt;
    o->n_tree_nodes = (int64_t)S->T.nodes.size();
    o->solve_fallbacks = S->fallbacks;
    return CPG_OK;
}

int cpg_vpcase_step(cpg_vpcase* Sp, int nsteps) {
    if (!Sp || nsteps < 0) return CPG_E_INVALID;
    cpg_vpcase& S = *Sp;
    for (int k = 0; k < nsteps && (S.run_all || !S.converged); k++) {
        cudaError_t e = step_once(S);
        if (e != cudaSuccess) {
            cpg::ctx_set_error(S.ctx, std::string("vortex-particle step: ") + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA;
        }
    }
    return CPG_OK;
}

int cpg_vpcase_trefftz(cpg_vpcase* Sp, double* CL, double* CD, int* converged) {
    if (!Sp) return CPG_E_INVALID;
    double cl = 0, cd = 0;
    cudaError_t e = trefftz(*Sp, cl, cd);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(Sp->ctx, std::string("trefftz: ") + cudaGetErrorString(e));
        return CPG_E_CUDA;
    }
    if (CL) *CL = cl;
    if (CD) *CD = cd;
    if (converged) *converged = Sp->converged ? 1 : 0;
    return CPG_OK;
}

int cpg_vpcase_velocities(cpg_vpcase* Sp, int precision, int direct, double* vel) {
    if (!Sp || (precision != CPG_PLAIN_FP64 && precision != CPG_MIXED)) return CPG_E_INVALID;
    cpg_vpcase& S = *Sp;
    const int64_t m = S.np;
    if (m == 0) return CPG_OK;
    if (!vel) return CPG_E_INVALID;
    const bool f32 = precision == CPG_MIXED;
    const cpg::VPConst c = cpg::vp_constants();
    cudaError_t e = pack_current(S);
    // particle term as convectParticles takes it (or the FP64 direct sum)
    if (e == cudaSuccess) {
        if (direct)
            e = direct_sums(S, 1, false, false, m, S.packed.as<cpg::BHPart>(), nullptr, m, S.tP.as<double>(), nullptr, nullptr);
        else if (S.accelerate && S.tree_built && S.T.nodes.size() > 1) {
            e = refresh_slots(S);
            if (e == cudaSuccess)
                e = cpg::launch_bh_targets(S.tnodes.as<cpg::BHNode>(), f32 ? S.fnodes.as<cpg::BHNodeF>() : nullptr,
                                           (int)S.T.nodes.size(), S.tslots.as<cpg::BHPart>(), S.T.theta,
                                           S.packed.as<cpg::BHPart>(), m, c, S.tP.as<double>(), nullptr, nullptr, S.s);
        } else if (S.accelerate)
            e = cudaMemsetAsync(S.tP.p, 0, sizeof(double) * 3 * m, S.s);
        else
            e = direct_sums(S, 2, false, false, m, S.packed.as<cpg::BHPart>(), nullptr, m, S.tP.as<double>(), nullptr, nullptr);
    }
    if (e == cudaSuccess) e = S.scr.ensure(sizeof(double) * cpg::vp_scratch_doubles(m, S.n), S.s);
    if (e == cudaSuccess)
        e = cpg::vp_launch_panel_vel(S.rec.as<double>(), S.sigma.as<double>(), S.mu.as<double>(), S.n,
                                     S.q1.as<double>(), S.mu1.as<double>(), S.n1, S.q2.as<double>(),
                                     S.mu2.as<double>(), S.n2, S.fil.as<double>(), S.have_fil ? S.n2 : 0,
                                     S.pos.as<double>(), m, 12 * S.cref, S.tQ.as<double>(), S.scr.as<double>(), S.s,
                                     f32);
    std::vector<double> hp(3 * m), hq(3 * m), hx(3 * m);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), S.tP.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hq.data(), S.tQ.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hx.data(), S.pos.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S.s);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(S.ctx, std::string("velocities: ") + cudaGetErrorString(e));
        return CPG_E_CUDA;
    }
    // the sum of k_vp_convect, with its 20 cref / 12 cref cut-offs
    for (int64_t i = 0; i < m; i++) {
        const double r = std::sqrt(hx[3 * i] * hx[3 * i] + hx[3 * i + 1] * hx[3 * i + 1] + hx[3 * i + 2] * hx[3 * i + 2]);
        for (int k = 0; k < 3; k++) {
            double v = S.vinf[k];
            if (!(r > 20 * S.cref)) {
                v = v + hp[3 * i + k];
                if (!(r > 12 * S.cref)) v = v + hq[3 * i + k];
            }
            vel[3 * i + k] = v;
        }
    }
    return CPG_OK;
}

int cpg_vpcase_particles(cpg_vpcase* Sp, double* pos, double* strength, double* radius, int32_t* shed_time,
                         int32_t* parent) {
    if (!Sp) return CPG_E_INVALID;
    cpg_vpcase& S = *Sp;
    const int64_t m = S.np;
    cudaError_t e = cudaSuccess;
    if (m > 0) {
        if (pos) e = cudaMemcpyAsync(pos, S.pos.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, S.s);
        if (e == cudaSuccess && strength)
            e = cudaMemcpyAsync(strength, S.str.p, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, S.s);
        if (e == cudaSuccess && radius) e = cudaMemcpyAsync(radius, S.rad.p, sizeof(double) * m, cudaMemcpyDeviceToHost, S.s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(S.s);
    }
    if (e != cudaSuccess) {
        cpg::ctx_set_error(S.ctx, std::string("particles: ") + cudaGetErrorString(e));
        return CPG_E_CUDA;
    }
    for (int64_t i = 0; i < m; i++) {
        if (shed_time) shed_time[i] = S.shed[i];
        if (parent) parent[i] = S.parent[i];
    }
    return CPG_OK;
}

int cpg_vpcase_strengths(cpg_vpcase* Sp, double* sigma, double* mu, double* mu_w1, double* mu_w2) {
    if (!Sp) return CPG_E_INVALID;
    cpg_vpcase& S = *Sp;
    cudaError_t e = cudaSuccess;
    if (sigma) e = cudaMemcpyAsync(sigma, S.sigma.p, sizeof(double) * S.n, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess && mu) e = cudaMemcpyAsync(mu, S.mu.p, sizeof(double) * S.n, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess && mu_w1 && S.n1)
        e = cudaMemcpyAsync(mu_w1, S.mu1.p, sizeof(double) * S.n1, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess && mu_w2 && S.n2)
        e = cudaMemcpyAsync(mu_w2, S.mu2.p, sizeof(double) * S.n2, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S.s);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(S.ctx, std::string("strengths: ") + cudaGetErrorString(e));
        return CPG_E_CUDA;
    }
    return CPG_OK;
}

int cpg_vpcase_surface(cpg_vpcase* Sp, const double* cg, double bref, double cref, double* phi, double* vel,
                       double* cp, double* forces) {
    if (!Sp || !cg || !(bref > 0) || !(cref > 0)) return CPG_E_INVALID;
    cpg_vpcase& S = *Sp;
    if (S.timestep < 1) {
        cpg::ctx_set_error(S.ctx, "surface: no step taken yet");
        return CPG_E_INVALID;
    }
    const int64_t n = S.n;
    cudaError_t e = cudaSuccess;
    auto fail = [&](const char* where) {
        cpg::ctx_set_error(S.ctx, std::string("surface: ") + where + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA;
    };
    if (!S.post_ready) {  // CHTLS weights of the clusters, once
        if ((e = up(S.p_bez, S.H.bez, S.s)) != cudaSuccess || (e = up(S.p_clp, S.H.cl_ptr, S.s)) != cudaSuccess ||
            (e = up(S.p_cli, S.H.cl_idx, S.s)) != cudaSuccess || (e = up(S.p_tip, S.H.tip, S.s)) != cudaSuccess ||
            (e = up(S.p_ts, S.H.tsorder, S.s)) != cudaSuccess)
            return fail("upload");
        if ((e = S.p_F3.ensure(sizeof(double) * n * 3 * (cpg::kClMax - 1), S.s)) != cudaSuccess ||
            (e = S.p_F2.ensure(sizeof(double) * n * 2 * (cpg::kClMax - 1), S.s)) != cudaSuccess ||
            (e = S.p_mode.ensure(sizeof(int32_t) * n, S.s)) != cudaSuccess)
            return fail("alloc");
        if ((e = cudaMemsetAsync(S.p_F2.p, 0, S.p_F2.bytes, S.s)) != cudaSuccess) return fail("clear");
        cpg::PostTables& T = S.PT;
        T = cpg::PostTables();
        T.n = n;
        T.rec = S.rec.as<double>();
        T.bez = S.p_bez.as<double>();
        T.cl_ptr = S.p_clp.as<int32_t>();
        T.cl_idx = S.p_cli.as<int32_t>();
        T.tip = S.p_tip.as<int32_t>();
        T.tsorder = S.p_ts.as<int32_t>();
        T.F3 = S.p_F3.as<double>();
        T.F2 = S.p_F2.as<double>();
        T.mode = S.p_mode.as<int32_t>();
        if ((e = cpg::launch_chtls_weights(T, S.s)) != cudaSuccess) return fail("CHTLS weights");
        S.post_ready = true;
    }
    // case scalars: cpCaseVP's free stream (steady), Vmag for Cp, the moment references
    cpg::CaseScalars cs;
    {
        double a = S.alpha * (kPi / 180), b = S.beta * (kPi / 180);
        double T[9] = {std::cos(a) * std::cos(b), std::cos(a) * std::sin(b), -std::sin(a),
                       -std::sin(b), std::cos(b), 0,
                       std::sin(a) * std::cos(b), std::sin(a) * std::sin(b), std::cos(a)};
        for (int q = 0; q < 9; q++) cs.T[q] = T[q];
        for (int q = 0; q < 3; q++) cs.Vinf[q] = S.vinf[q];
        cs.V = S.V;
        cs.PG = S.PG;
        cs.Sref = S.Sref;
        cs.bref = bref;
        cs.cref = cref;
        for (int q = 0; q < 3; q++) cs.cg[q] = cg[q];
    }
    if ((e = S.p_cs.ensure(sizeof(cs), S.s)) != cudaSuccess ||
        (e = S.p_work.ensure(cpg::post_work_bytes(S.PT, 1), S.s)) != cudaSuccess ||
        (e = S.p_out.ensure(sizeof(double) * (5 * n + 9), S.s)) != cudaSuccess)
        return fail("alloc");
    if ((e = cudaMemcpyAsync(S.p_cs.p, &cs, sizeof(cs), cudaMemcpyHostToDevice, S.s)) != cudaSuccess)
        return fail("upload");
    double* o = S.p_out.as<double>();
    if ((e = cpg::launch_surface(S.PT, S.p_cs.as<cpg::CaseScalars>(), S.mu.as<double>(), S.vtot.as<double>(), o,
                                 o + n, o + 4 * n, o + 5 * n, S.p_work.p, S.s)) != cudaSuccess)
        return fail("surface pass");
    if (phi && (e = cudaMemcpyAsync(phi, o, sizeof(double) * n, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return fail("copy");
    if (vel && (e = cudaMemcpyAsync(vel, o + n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return fail("copy");
    if (cp && (e = cudaMemcpyAsync(cp, o + 4 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, S.s)) != cudaSuccess)
        return fail("copy");
    if (forces && (e = cudaMemcpyAsync(forces, o + 5 * n, sizeof(double) * 9, cudaMemcpyDeviceToHost, S.s)) !=
                      cudaSuccess)
        return fail("copy");
    if ((e = cudaStreamSynchronize(S.s)) != cudaSuccess) return fail("sync");
    return CPG_OK;
}

int cpg_vpcase_wake(const cpg_vpcase* S, double* w1_verts, double* w2_verts) {
    if (!S) return CPG_E_INVALID;
    for (int64_t j = 0; j < S->n1 && w1_verts; j++)
        for (int k = 0; k < 12; k++) w1_verts[12 * j + k] = S->G.w1[j * cpg::QF_STRIDE + k];
    for (int64_t j = 0; j < S->n2 && w2_verts; j++)
        for (int k = 0; k < 12; k++) w2_verts[12 * j + k] = S->G.w2[j * cpg::QF_STRIDE + k];
    return CPG_OK;
}

int cpg_vpcase_matrices(cpg_vpcase* Sp, double* A, double* B, double* C) {
    if (!Sp) return CPG_E_INVALID;
    cpg_vpcase& S = *Sp;
    cudaError_t e = cudaSuccess;
    if (A) e = cudaMemcpyAsync(A, S.A.p, sizeof(double) * S.n * S.n, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess && B) e = cudaMemcpyAsync(B, S.B.p, sizeof(double) * S.n * S.n, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess && C && S.n2)
        e = cudaMemcpyAsync(C, S.C.p, sizeof(double) * S.n * S.n2, cudaMemcpyDeviceToHost, S.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S.s);
    if (e != cudaSuccess) {
        cpg::ctx_set_error(S.ctx, std::string("matrices: ") + cudaGetErrorString(e));
        return CPG_E_CUDA;
    }
    return CPG_OK;
}

int cpg_vp_topology(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids, int64_t n_tris,
                    double V, double dt, int64_t* counts, double* dt_out, double* w1_verts, double* w2_verts,
                    int32_t* w1_idx4, double* w1_coef, int32_t* w2_parent) {
    if (!nodes || !tris || !ids || !counts || !dt_out || !(V > 0)) return CPG_E_INVALID;
    cpg::VPGeom G;
    std::string err = cpg::build_vp_geometry(nodes, n_nodes, tris, ids, n_tris, V, dt, G);
    if (!err.empty()) return CPG_E_BAD_MESH;
    counts[0] = G.n_body;
    counts[1] = G.n_w1;
    counts[2] = G.n_w2;
    *dt_out = G.dt;
    for (int64_t j = 0; j < G.n_w1; j++) {
        for (int k = 0; k < 12 && w1_verts; k++) w1_verts[12 * j + k] = G.w1[j * cpg::QF_STRIDE + k];
        for (int k = 0; k < 4 && w1_idx4; k++) w1_idx4[4 * j + k] = G.widx[4 * j + k];
        if (w1_coef) w1_coef[j] = G.wcoef[j];
    }
    for (int64_t j = 0; j < G.n_w2; j++) {
        for (int k = 0; k < 12 && w2_verts; k++) w2_verts[12 * j + k] = G.w2[j * cpg::QF_STRIDE + k];
        if (w2_parent) w2_parent[j] = G.parent[j];
    }
    return CPG_OK;
}

int cpg_panels_stretching(cpg_ctx* ctx, const double* body_verts, const double* sigma, const double* mu, int64_t nb,
                          const double* wake_verts, const double* wake_mu, int64_t nw, const double* pos,
                          const double* strength, int64_t m, double* out) {
    if (!ctx || nb < 0 || nw < 0 || m < 0 || (nb > 0 && (!body_verts || !sigma || !mu)) ||
        (nw > 0 && (!wake_verts || !wake_mu)) || (m > 0 && (!pos || !strength || !out))) {
        if (ctx) cpg::ctx_set_error(ctx, "bad argument");
        return CPG_E_INVALID;
    }
    if (m == 0) return CPG_OK;
    cudaStream_t s = cpg::ctx_stream(ctx);
    Buf rec, q, scr;
    std::vector<double> hv(12 * nw), hq(cpg::QF_STRIDE * nw);
    cudaError_t e = rec.ensure(sizeof(double) * 24 * std::max<int64_t>(1, nb), s);
    if (e == cudaSuccess) e = scr.ensure(sizeof(double) * std::max<int64_t>(1, cpg::vp_scratch_doubles(m, nb)), s);
    if (e == cudaSuccess && nb > 0) e = cpg::launch_pack_records(body_verts, nb, rec.as<double>(), s);
    if (e == cudaSuccess && nw > 0) e = cudaMemcpyAsync(hv.data(), wake_verts, sizeof(double) * 12 * nw,
                                                        cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int64_t j = 0; j < nw && e == cudaSuccess; j++) cpg::pack_quad_record(&hv[12 * j], &hq[cpg::QF_STRIDE * j]);
    if (e == cudaSuccess) e = up(q, hq, s);
    if (e == cudaSuccess)
        e = cpg::vp_launch_stretch_panels(rec.as<double>(), sigma, mu, nb, q.as<double>(), wake_mu, nw, pos, strength, m,
                                          0.0, out, scr.as<double>(), s,
                                          cpg::ctx_particle_precision(ctx) == CPG_MIXED);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    rec.release();
    q.release();
    scr.release();
    if (e != cudaSuccess) {
        cpg::ctx_set_error(ctx, std::string("panel stretching: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? CPG_E_OOM : CPG_E_CUDA;
    }
    return CPG_OK;
}

}  // extern "C"
