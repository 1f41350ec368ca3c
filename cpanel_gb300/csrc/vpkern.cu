// Kernels of the vortex-particle case that involve panels: buffer-wake assembly
// columns, the C matrix, panel and filament velocity at points, panel-to-particle
// stretching, and the per-step updates.  Compiled with --fmad=false so that every
// branch (near/far, on-panel, near-filament, the AB2 start test) and every update
// rounds as the host's do.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "panel64.cuh"
#include "vp.cuh"
#include "vpkern.h"

namespace {

constexpr int VT = 128, TILE = 64;

// geometry::setInfCoeff wake scatter for the first buffer row (quads), one thread per
// row i, panels in order (CPanel/geometry.cpp:853-873)
__global__ void k_vp_wake_columns(const double* __restrict__ rec, int64_t n, const double* __restrict__ q1,
                                  const int32_t* __restrict__ widx, const double* __restrict__ wcoef, int64_t n1,
                                  double* __restrict__ A) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dv3 c = ld3(rec + i * R_STRIDE + R_C);
    for (int64_t j = 0; j < n1; j++) {
        double infl = dub_phi_inf_q(q1 + j * Q_STRIDE, c);
        double cf = wcoef[j];
        A[(int64_t)widx[4 * j + 0] * n + i] += infl * (1 - cf);
        A[(int64_t)widx[4 * j + 1] * n + i] += infl * (cf - 1);
        A[(int64_t)widx[4 * j + 2] * n + i] += infl * cf;
        A[(int64_t)widx[4 * j + 3] * n + i] -= infl * cf;
    }
}

// C(i, j) = w2Panels[j]->dubPhiInf(centre_i), CPanel/geometry.cpp:875-884
__global__ void k_vp_cmat(const double* __restrict__ rec, int64_t n, const double* __restrict__ q2, int64_t n2,
                          double* __restrict__ C) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n2) return;
    int64_t j = t / n, i = t % n;
    C[t] = dub_phi_inf_q(q2 + j * Q_STRIDE, ld3(rec + i * R_STRIDE + R_C));
}

// Panel and filament velocity at points: body panelV (sigma vSrc + mu vDub), first and
// second buffer rows (mu dubVInf), filaments (vortexFil::velInfl, CPanel/vortexFil.cpp:26-40).
// Points with |p| > skip_r (skip_r > 0) get zero: the reference returns before the panel
// terms there (CPanel/cpCaseVP.cpp:711-715).
// The body panels are split into chunks along grid.y so that a handful of points still
// fill the GPU; k_vp_panel_vel_fin adds the chunks in order, then the quads and filaments.
__global__ void __launch_bounds__(VT) k_vp_panel_vel_part(const double* __restrict__ rec,
                                                          const double* __restrict__ sigma,
                                                          const double* __restrict__ mu, int64_t nb,
                                                          int64_t chunk, const double* __restrict__ pts, int64_t m,
                                                          double skip_r, double* __restrict__ part) {
    __shared__ double tile[TILE * R_STRIDE];
    __shared__ double ts[TILE], tm[TILE];
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = q < m;
    dv3 poi = live ? ld3(pts + 3 * q) : mk3(0, 0, 0);
    if (live && skip_r > 0 && norm3(poi) > skip_r) live = false;
    const int64_t jb = (int64_t)blockIdx.y * chunk, je = min(nb, jb + chunk);
    dv3 acc = mk3(0, 0, 0);
    for (int64_t b = jb; b < je; b += TILE) {
        int lim = (int)((je - b) < TILE ? (je - b) : TILE);
        __syncthreads();
        for (int k = threadIdx.x; k < lim * R_STRIDE; k += VT) tile[k] = rec[b * R_STRIDE + k];
        for (int k = threadIdx.x; k < lim; k += VT) {
            ts[k] = sigma[b + k];
            tm[k] = mu[b + k];
        }
        __syncthreads();
        if (!live) continue;
        for (int k = 0; k < lim; k++) {
            dv3 vs, vd;
            panel_v_inf(tile + k * R_STRIDE, poi, vs, vd);
            acc = acc + (ts[k] * vs + tm[k] * vd);
        }
    }
    if (q >= m) return;
    double* o = part + ((int64_t)blockIdx.y * m + q) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
}

__global__ void k_vp_panel_vel_fin(const double* __restrict__ part, int64_t nchunk, const double* __restrict__ q1,
                                   const double* __restrict__ mu1, int64_t n1, const double* __restrict__ q2,
                                   const double* __restrict__ mu2, int64_t n2, const double* __restrict__ fil,
                                   int64_t nf, const double* __restrict__ pts, int64_t m, double skip_r,
                                   double* __restrict__ out) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    dv3 poi = ld3(pts + 3 * q);
    if (skip_r > 0 && norm3(poi) > skip_r) {
        out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = 0;
        return;
    }
    dv3 acc = mk3(0, 0, 0);
    for (int64_t c = 0; c < nchunk; c++) acc = acc + ld3(part + (c * m + q) * 3);
    for (int64_t j = 0; j < n1; j++) acc = acc + mu1[j] * dub_v_inf_q(q1 + j * Q_STRIDE, poi);
    for (int64_t j = 0; j < n2; j++) acc = acc + mu2[j] * dub_v_inf_q(q2 + j * Q_STRIDE, poi);
    for (int64_t j = 0; j < nf; j++) {
        const double* f = fil + 8 * j;
        dv3 p1 = ld3(f), p2 = ld3(f + 3);
        acc = acc + (f[6] * vortex_v(poi - p1, poi - p2, p2 - p1)) / CPG_FOUR_PI;
    }
    out[3 * q] = acc.x;
    out[3 * q + 1] = acc.y;
    out[3 * q + 2] = acc.z;
}

// sum over body panels of bodyPanel::partStretching and over first-row panels of
// wakePanel::partStretching (CPanel/bodyPanel.cpp:697-728, CPanel/wakePanel.cpp:266-289).
// Particles with |x| > skip_x (skip_x > 0) get zero (cpCaseVP.cpp:473-499).  Body
// panels in chunks along grid.y as for the velocity.
__global__ void __launch_bounds__(VT) k_vp_stretch_part(const double* __restrict__ rec,
                                                        const double* __restrict__ sigma,
                                                        const double* __restrict__ mu, int64_t nb, int64_t chunk,
                                                        const double* __restrict__ pos,
                                                        const double* __restrict__ str, int64_t m, double skip_x,
                                                        double* __restrict__ part) {
    __shared__ double tile[TILE * R_STRIDE];
    __shared__ double ts[TILE], tm[TILE];
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = q < m;
    dv3 x = live ? ld3(pos + 3 * q) : mk3(0, 0, 0);
    dv3 a = live ? ld3(str + 3 * q) : mk3(0, 0, 0);
    if (live && skip_x > 0 && fabs(x.x) > skip_x) live = false;
    const int64_t jb = (int64_t)blockIdx.y * chunk, je = min(nb, jb + chunk);
    dv3 acc = mk3(0, 0, 0);
    for (int64_t b = jb; b < je; b += TILE) {
        int lim = (int)((je - b) < TILE ? (je - b) : TILE);
        __syncthreads();
        for (int k = threadIdx.x; k < lim * R_STRIDE; k += VT) tile[k] = rec[b * R_STRIDE + k];
        for (int k = threadIdx.x; k < lim; k += VT) {
            ts[k] = sigma[b + k];
            tm[k] = mu[b + k];
        }
        __syncthreads();
        if (!live) continue;
        for (int k = 0; k < lim; k++) {
            const double* r = tile + k * R_STRIDE;
            dv3 c = ld3(r + R_C);
            dm3 G;
            if (norm3(x - c) / r[R_LONG] > 5) {
                dm3 g1 = vel_grad_point_source(c, r[R_AREA], ts[k], x);
                dm3 g2 = vel_grad_point_doublet(c, r[R_AREA], tm[k], x);
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) G.a[i][j] = (0 + g1.a[i][j]) + g2.a[i][j];
            } else {
                dm3 g1 = vel_grad_tri_source(r, ts[k], x);
                dm3 g2 = vel_grad_doublet(r, 3, c, ld3(r + R_N), ld3(r + R_L), ld3(r + R_M), r[R_LONG], tm[k], x);
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) G.a[i][j] = (0 + g1.a[i][j]) + g2.a[i][j];
            }
            acc = acc + mul_m3(G, a);
        }
    }
    if (q >= m) return;
    double* o = part + ((int64_t)blockIdx.y * m + q) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
}

__global__ void k_vp_stretch_fin(const double* __restrict__ part, int64_t nchunk, const double* __restrict__ q1,
                                 const double* __restrict__ mu1, int64_t n1, const double* __restrict__ pos,
                                 const double* __restrict__ str, int64_t m, double skip_x, double* __restrict__ out) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    dv3 x = ld3(pos + 3 * q), a = ld3(str + 3 * q);
    if (skip_x > 0 && fabs(x.x) > skip_x) {
        out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = 0;
        return;
    }
    dv3 acc = mk3(0, 0, 0);
    for (int64_t c = 0; c < nchunk; c++) acc = acc + ld3(part + (c * m + q) * 3);
    for (int64_t j = 0; j < n1; j++) {
        const double* w = q1 + j * Q_STRIDE;
        dv3 c = ld3(w + Q_C);
        dm3 G = norm3(x - c) / w[Q_LONG] > 5
                    ? vel_grad_point_doublet(c, w[Q_AREA], mu1[j], x)
                    : vel_grad_doublet(w, 4, c, ld3(w + Q_N), ld3(w + Q_L), ld3(w + Q_M), w[Q_LONG], mu1[j], x);
        acc = acc + mul_m3(G, a);
    }
    out[3 * q] = acc.x;
    out[3 * q + 1] = acc.y;
    out[3 * q + 2] = acc.z;
}

// Eigen's isZero(): every |component| <= 1e-12
__device__ __forceinline__ bool is_zero_eigen(dv3 v) {
    return fabs(v.x) <= 1e-12 && fabs(v.y) <= 1e-12 && fabs(v.z) <= 1e-12;
}

// cpCaseVP::velocityInflFromEverything(particle*) assembly of the terms and the AB2
// position update of convectParticles (CPanel/cpCaseVP.cpp:548-575,680-734).
// part: particle term; pan: panel + filament term (zero where skipped).
__global__ void k_vp_convect(double* __restrict__ pos, double* __restrict__ prevVel, const double* __restrict__ part,
                             const double* __restrict__ pan, int64_t m, dv3 vinf, double cref, double dt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    dv3 p = ld3(pos + 3 * i);
    dv3 v = vinf;
    double r = norm3(p);
    if (!(r > 20 * cref)) {
        v = v + ld3(part + 3 * i);
        if (!(r > 12 * cref)) v = v + ld3(pan + 3 * i);
    }
    dv3 pv = ld3(prevVel + 3 * i);
    dv3 np = is_zero_eigen(pv) ? p + dt * v : p + dt * (1.5 * v - 0.5 * pv);
    prevVel[3 * i] = v.x;
    prevVel[3 * i + 1] = v.y;
    prevVel[3 * i + 2] = v.z;
    pos[3 * i] = np.x;
    pos[3 * i + 1] = np.y;
    pos[3 * i + 2] = np.z;
}

// AB2 strength update of particleStrengthUpdate (CPanel/cpCaseVP.cpp:528-545):
// dv = (diffusion + panel stretching) + stretching, zero beyond 20 c in |x|.
__global__ void k_vp_strength(const double* __restrict__ pos, double* __restrict__ str, double* __restrict__ prevStr,
                              const double* __restrict__ dstr, const double* __restrict__ ddif,
                              const double* __restrict__ dpan, int64_t m, double cref, double dt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    dv3 x = ld3(pos + 3 * i);
    dv3 dv = mk3(0, 0, 0);
    if (!(fabs(x.x) > 20 * cref)) dv = (ld3(ddif + 3 * i) + ld3(dpan + 3 * i)) + ld3(dstr + 3 * i);
    dv3 a = ld3(str + 3 * i), pv = ld3(prevStr + 3 * i);
    dv3 na = is_zero_eigen(pv) ? a + dt * dv : a + dt * (1.5 * dv - 0.5 * pv);
    prevStr[3 * i] = dv.x;
    prevStr[3 * i + 1] = dv.y;
    prevStr[3 * i + 2] = dv.z;
    str[3 * i] = na.x;
    str[3 * i + 1] = na.y;
    str[3 * i + 2] = na.z;
}

// setSourceStrengthsVP, CPanel/cpCaseVP.cpp:173-202: sigma = -(Vinf + particles +
// filaments) . n (vpart: the particle term at the centres, or null for none)
__global__ void k_vp_sigma(const double* __restrict__ rec, int64_t n, const double* __restrict__ vpart,
                           const double* __restrict__ fil, int64_t nf, dv3 vinf, double* __restrict__ sigma) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dv3 c = ld3(rec + i * R_STRIDE + R_C), nn = ld3(rec + i * R_STRIDE + R_N);
    dv3 s = vpart ? ld3(vpart + 3 * i) : mk3(0, 0, 0);
    for (int64_t j = 0; j < nf; j++) {
        const double* f = fil + 8 * j;
        dv3 p1 = ld3(f), p2 = ld3(f + 3);
        s = s + (f[6] * vortex_v(c - p1, c - p2, p2 - p1)) / CPG_FOUR_PI;
    }
    sigma[i] = -dot3(vinf + s, nn) + 0;
}

// rhs -= C mu2
__global__ void k_vp_rhs_c(const double* __restrict__ C, int64_t n, int64_t n2, const double* __restrict__ mu2,
                           double* __restrict__ rhs) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = 0;
    for (int64_t j = 0; j < n2; j++) acc += C[j * n + i] * mu2[j];
    rhs[i] = rhs[i] - acc;
}

// wakePanel::setMu (first row, from the solved body doublets), keeping the previous value
__global__ void k_vp_wake_mu(const double* __restrict__ mu, const int32_t* __restrict__ widx,
                             const double* __restrict__ wcoef, int64_t n1, double* __restrict__ mu1,
                             double* __restrict__ prev1, int keep_prev) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n1) return;
    if (keep_prev) prev1[j] = mu1[j];
    double c = wcoef[j];
    mu1[j] = (1 - c) * mu[widx[4 * j]] + (c - 1) * mu[widx[4 * j + 1]] + c * mu[widx[4 * j + 2]] - c * mu[widx[4 * j + 3]];
}

// cpCaseVP::convectBufferWake, CPanel/cpCaseVP.cpp:160-171
__global__ void k_vp_buffer(const double* __restrict__ mu1, const int32_t* __restrict__ parent, int64_t n2,
                            double* __restrict__ mu2, double* __restrict__ prev2) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n2) return;
    prev2[k] = mu2[k];
    mu2[k] = mu1[parent[k]];
}

inline unsigned nblk(int64_t m, int t) { return (unsigned)((m + t - 1) / t); }

}  // namespace

namespace cpg {

cudaError_t vp_launch_wake_columns(const double* rec, int64_t n, const double* q1, const int32_t* widx,
                                   const double* wcoef, int64_t n1, double* A, cudaStream_t s) {
    if (n > 0 && n1 > 0) k_vp_wake_columns<<<nblk(n, VT), VT, 0, s>>>(rec, n, q1, widx, wcoef, n1, A);
    return cudaGetLastError();
}
cudaError_t vp_launch_cmat(const double* rec, int64_t n, const double* q2, int64_t n2, double* C, cudaStream_t s) {
    if (n > 0 && n2 > 0) k_vp_cmat<<<nblk(n * n2, 256), 256, 0, s>>>(rec, n, q2, n2, C);
    return cudaGetLastError();
}
// chunks of body panels along grid.y: enough blocks to fill the GPU several times over
int64_t vp_chunks(int64_t m, int64_t nb) {
    int64_t bx = (m + VT - 1) / VT;
    int64_t maxc = (nb + TILE - 1) / TILE;
    int64_t c = (4 * 152 + bx - 1) / bx;
    return std::max<int64_t>(1, std::min(c, maxc));
}

int64_t vp_scratch_doubles(int64_t m, int64_t nb) { return vp_chunks(m, nb) * m * 3; }

cudaError_t vp_launch_panel_vel(const double* rec, const double* sigma, const double* mu, int64_t nb, const double* q1,
                                const double* mu1, int64_t n1, const double* q2, const double* mu2, int64_t n2,
                                const double* fil, int64_t nf, const double* pts, int64_t m, double skip_r,
                                double* out, double* scratch, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    const int64_t nc = vp_chunks(m, nb);
    const int64_t chunk = nb > 0 ? ((nb + nc - 1) / nc + TILE - 1) / TILE * TILE : TILE;
    const int64_t ncu = nb > 0 ? (nb + chunk - 1) / chunk : 0;
    if (ncu > 0)
        k_vp_panel_vel_part<<<dim3(nblk(m, VT), (unsigned)ncu), VT, 0, s>>>(rec, sigma, mu, nb, chunk, pts, m, skip_r,
                                                                           scratch);
    k_vp_panel_vel_fin<<<nblk(m, 128), 128, 0, s>>>(scratch, ncu, q1, mu1, n1, q2, mu2, n2, fil, nf, pts, m, skip_r,
                                                    out);
    return cudaGetLastError();
}
cudaError_t vp_launch_stretch_panels(const double* rec, const double* sigma, const double* mu, int64_t nb,
                                     const double* q1, const double* mu1, int64_t n1, const double* pos,
                                     const double* str, int64_t m, double skip_x, double* out, double* scratch,
                                     cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    const int64_t nc = vp_chunks(m, nb);
    const int64_t chunk = nb > 0 ? ((nb + nc - 1) / nc + TILE - 1) / TILE * TILE : TILE;
    const int64_t ncu = nb > 0 ? (nb + chunk - 1) / chunk : 0;
    if (ncu > 0)
        k_vp_stretch_part<<<dim3(nblk(m, VT), (unsigned)ncu), VT, 0, s>>>(rec, sigma, mu, nb, chunk, pos, str, m,
                                                                         skip_x, scratch);
    k_vp_stretch_fin<<<nblk(m, 128), 128, 0, s>>>(scratch, ncu, q1, mu1, n1, pos, str, m, skip_x, out);
    return cudaGetLastError();
}
cudaError_t vp_launch_convect(double* pos, double* prevVel, const double* part, const double* pan, int64_t m,
                              const double vinf[3], double cref, double dt, cudaStream_t s) {
    if (m > 0) k_vp_convect<<<nblk(m, 256), 256, 0, s>>>(pos, prevVel, part, pan, m, dv3{vinf[0], vinf[1], vinf[2]}, cref, dt);
    return cudaGetLastError();
}
cudaError_t vp_launch_strength(const double* pos, double* str, double* prevStr, const double* dstr,
                               const double* ddif, const double* dpan, int64_t m, double cref, double dt,
                               cudaStream_t s) {
    if (m > 0) k_vp_strength<<<nblk(m, 256), 256, 0, s>>>(pos, str, prevStr, dstr, ddif, dpan, m, cref, dt);
    return cudaGetLastError();
}
cudaError_t vp_launch_sigma(const double* rec, int64_t n, const double* vpart, const double* fil, int64_t nf,
                            const double vinf[3], double* sigma, cudaStream_t s) {
    if (n > 0) k_vp_sigma<<<nblk(n, 256), 256, 0, s>>>(rec, n, vpart, fil, nf, dv3{vinf[0], vinf[1], vinf[2]}, sigma);
    return cudaGetLastError();
}
cudaError_t vp_launch_rhs_c(const double* C, int64_t n, int64_t n2, const double* mu2, double* rhs, cudaStream_t s) {
    if (n > 0 && n2 > 0) k_vp_rhs_c<<<nblk(n, 256), 256, 0, s>>>(C, n, n2, mu2, rhs);
    return cudaGetLastError();
}
cudaError_t vp_launch_wake_mu(const double* mu, const int32_t* widx, const double* wcoef, int64_t n1, double* mu1,
                              double* prev1, int keep_prev, cudaStream_t s) {
    if (n1 > 0) k_vp_wake_mu<<<nblk(n1, 128), 128, 0, s>>>(mu, widx, wcoef, n1, mu1, prev1, keep_prev);
    return cudaGetLastError();
}
cudaError_t vp_launch_buffer(const double* mu1, const int32_t* parent, int64_t n2, double* mu2, double* prev2,
                             cudaStream_t s) {
    if (n2 > 0) k_vp_buffer<<<nblk(n2, 128), 128, 0, s>>>(mu1, parent, n2, mu2, prev2);
    return cudaGetLastError();
}

}  // namespace cpg
