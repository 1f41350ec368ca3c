// Kernels of the vortex-particle case that involve panels: buffer-wake assembly
// columns, the C matrix, panel and filament velocity at points, panel-to-particle
// stretching (FP64, or with the far field in FP32), and the per-step updates.  Compiled with --fmad=false so that every
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
                                                          double skip_r, double* __restrict__ part, int64_t sinv) {
    __shared__ double tile[TILE * R_STRIDE];
    __shared__ double ts[TILE], tm[TILE];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < m;
    const int64_t q = live ? (int64_t)(((uint64_t)t * (uint64_t)sinv) % (uint64_t)m) : 0;
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
    if (t >= m) return;
    double* o = part + ((int64_t)blockIdx.y * m + q) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
}

__device__ __forceinline__ dv3 warp_sum3(dv3 v) {  // fixed butterfly: deterministic
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
    }
    return v;
}

// one warp per point: lanes share the body chunks' partial sums and the quads and
// filaments, each set reduced by a fixed butterfly
__global__ void k_vp_panel_vel_fin(const double* __restrict__ part, int64_t nchunk, const double* __restrict__ q1,
                                   const double* __restrict__ mu1, int64_t n1, const double* __restrict__ q2,
                                   const double* __restrict__ mu2, int64_t n2, const double* __restrict__ fil,
                                   int64_t nf, const double* __restrict__ pts, int64_t m, double skip_r,
                                   double* __restrict__ out) {
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= m) return;  // uniform across the warp
    dv3 poi = ld3(pts + 3 * q);
    if (skip_r > 0 && norm3(poi) > skip_r) {
        if (lane == 0) out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = 0;
        return;
    }
    dv3 acc = mk3(0, 0, 0);
    for (int64_t j = lane; j < n1 + n2 + nf; j += 32) {
        if (j < n1) {
            acc = acc + mu1[j] * dub_v_inf_q(q1 + j * Q_STRIDE, poi);
        } else if (j < n1 + n2) {
            acc = acc + mu2[j - n1] * dub_v_inf_q(q2 + (j - n1) * Q_STRIDE, poi);
        } else {
            const double* f = fil + 8 * (j - n1 - n2);
            dv3 p1 = ld3(f), p2 = ld3(f + 3);
            acc = acc + (f[6] * vortex_v(poi - p1, poi - p2, p2 - p1)) / CPG_FOUR_PI;
        }
    }
    // body chunks: lane l adds chunks l, l+32, ... (then the same butterfly)
    dv3 body = mk3(0, 0, 0);
    for (int64_t c = lane; c < nchunk; c += 32) body = body + ld3(part + (c * m + q) * 3);
    body = warp_sum3(body);
    acc = warp_sum3(acc);
    if (lane != 0) return;
    const dv3 tot = body + acc;
    out[3 * q] = tot.x;
    out[3 * q + 1] = tot.y;
    out[3 * q + 2] = tot.z;
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
                                                        double* __restrict__ part, int64_t sinv) {
    __shared__ double tile[TILE * R_STRIDE];
    __shared__ double ts[TILE], tm[TILE];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < m;
    const int64_t q = live ? (int64_t)(((uint64_t)t * (uint64_t)sinv) % (uint64_t)m) : 0;
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
    if (t >= m) return;
    double* o = part + ((int64_t)blockIdx.y * m + q) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
}

// ---- FP32 far field (the mixed-precision form of the two panel kernels) ----
// Pairs beyond five panel lengths (the reference's point-source/point-doublet branch)
// are evaluated in FP32 from a float view of the tile: panel centre split into high
// and low floats, normal, sigma area / 4 pi, mu area / 4 pi and (5 longSide)^2.  The
// near/far decision compares the float squared distance with a relative margin of 1e-5
// and takes the FP64 test inside it, so every pair takes the same branch as in FP64;
// near pairs run the FP64 code above.  Far terms are summed with compensation in float.
constexpr float kBandLo = 1.0f - 1e-5f, kBandHi = 1.0f + 1e-5f;
enum { FT_CH = 0, FT_CL = 3, FT_N = 6, FT_AS = 9, FT_AD = 10, FT_T2 = 11, FT_STRIDE = 12 };

struct KSum3 {
    float x = 0, y = 0, z = 0, cx = 0, cy = 0, cz = 0;
    __device__ __forceinline__ static void add1(float& s, float& c, float v) {
        float y_ = v - c;
        float t = s + y_;
        c = (t - s) - y_;
        s = t;
    }
    __device__ __forceinline__ void add(float vx, float vy, float vz) {
        add1(x, cx, vx);
        add1(y, cy, vy);
        add1(z, cz, vz);
    }
    __device__ __forceinline__ dv3 value() const {
        return mk3((double)x - (double)cx, (double)y - (double)cy, (double)z - (double)cz);
    }
};

// float view of panel b + k (thread-strided fill of a tile)
__device__ __forceinline__ void fill_ftile(const double* __restrict__ r, double sigma, double mu, float* __restrict__ f) {
    const double inv4pi = 1.0 / CPG_FOUR_PI;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const double c = r[R_C + q];
        const float h = __double2float_rn(c);
        f[FT_CH + q] = h;
        f[FT_CL + q] = __double2float_rn(c - (double)h);
        f[FT_N + q] = __double2float_rn(r[R_N + q]);
    }
    f[FT_AS] = __double2float_rn(sigma * r[R_AREA] * inv4pi);
    f[FT_AD] = __double2float_rn(mu * r[R_AREA] * inv4pi);
    const double t = 5 * r[R_LONG];
    f[FT_T2] = __double2float_rn(t * t);
}

struct PtF {
    float hx, hy, hz, lx, ly, lz;
};
__device__ __forceinline__ PtF split_pt(dv3 p) {
    PtF f;
    f.hx = __double2float_rn(p.x);
    f.hy = __double2float_rn(p.y);
    f.hz = __double2float_rn(p.z);
    f.lx = __double2float_rn(p.x - (double)f.hx);
    f.ly = __double2float_rn(p.y - (double)f.hy);
    f.lz = __double2float_rn(p.z - (double)f.hz);
    return f;
}

// 1: far (point formulas), 0: near; p - centre in (dx, dy, dz), squared norm d2
__device__ __forceinline__ bool far_pair(const PtF& p, const float* __restrict__ f, const double* __restrict__ r,
                                         dv3 poi, float& dx, float& dy, float& dz, float& d2) {
    dx = (p.hx - f[FT_CH]) + (p.lx - f[FT_CL]);
    dy = (p.hy - f[FT_CH + 1]) + (p.ly - f[FT_CL + 1]);
    dz = (p.hz - f[FT_CH + 2]) + (p.lz - f[FT_CL + 2]);
    d2 = dx * dx + dy * dy + dz * dz;
    const float t2 = f[FT_T2];
    if (d2 > t2 * kBandHi) return true;
    if (d2 < t2 * kBandLo) return false;
    return norm3(poi - ld3(r + R_C)) / r[R_LONG] > 5;  // the FP64 test of panel_v_inf / stretching
}

// Per-warp queue of the FP64 near pairs of one panel tile: entries (panel << 5) | lane in
// tile order, then lane order; the warp evaluates them one per lane and each target adds
// its own results in queue order (the same order on every run).
struct NearQueue {
    unsigned short q[VT / 32][TILE * 32];
    double tgt[VT / 32][32][6];  // the warp's targets: position, strength
    double res[VT / 32][32][3];
    int own[VT / 32][32];
    __device__ __forceinline__ void put_target(int w, int lane, dv3 x, dv3 a) {
        tgt[w][lane][0] = x.x; tgt[w][lane][1] = x.y; tgt[w][lane][2] = x.z;
        tgt[w][lane][3] = a.x; tgt[w][lane][4] = a.y; tgt[w][lane][5] = a.z;
    }
    __device__ __forceinline__ dv3 tx(int w, int ln) const { return mk3(tgt[w][ln][0], tgt[w][ln][1], tgt[w][ln][2]); }
    __device__ __forceinline__ dv3 ta(int w, int ln) const { return mk3(tgt[w][ln][3], tgt[w][ln][4], tgt[w][ln][5]); }
    // all lanes call; returns the new (warp-uniform) length
    __device__ __forceinline__ int push(int w, int lane, bool near, int k, int qn) {
        const unsigned m = __ballot_sync(0xffffffffu, near);
        if (near) q[w][qn + __popc(m & ((1u << lane) - 1u))] = (unsigned short)((k << 5) | lane);
        return qn + __popc(m);
    }
    __device__ __forceinline__ bool take(int w, int e, int qn, int& k, int& ln) const {
        if (e >= qn) return false;
        const int ent = q[w][e];
        k = ent >> 5;
        ln = ent & 31;
        return true;
    }
    __device__ __forceinline__ void put_result(int w, int lane, int ln, dv3 v) {
        res[w][lane][0] = v.x; res[w][lane][1] = v.y; res[w][lane][2] = v.z;
        own[w][lane] = ln;
    }
    // all lanes call after their take/put_result: adds this chunk's results to their owners
    __device__ __forceinline__ dv3 gather(int w, int lane, int base, int qn, dv3 acc) {
        __syncwarp();
        const int cnt = min(32, qn - base);
        for (int j = 0; j < cnt; j++)
            if (own[w][j] == lane) acc = acc + mk3(res[w][j][0], res[w][j][1], res[w][j][2]);
        __syncwarp();
        return acc;
    }
};

__global__ void __launch_bounds__(VT) k_vp_panel_vel_part_f32(const double* __restrict__ rec,
                                                              const double* __restrict__ sigma,
                                                              const double* __restrict__ mu, int64_t nb,
                                                              int64_t chunk, const double* __restrict__ pts,
                                                              int64_t m, double skip_r, double* __restrict__ part, int64_t sinv) {
    __shared__ double tile[TILE * R_STRIDE];
    __shared__ double ts[TILE], tm[TILE];
    __shared__ float ft[TILE * FT_STRIDE];
    __shared__ NearQueue nq;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < m;
    const int64_t q = live ? (int64_t)(((uint64_t)t * (uint64_t)sinv) % (uint64_t)m) : 0;
    dv3 poi = live ? ld3(pts + 3 * q) : mk3(0, 0, 0);
    if (live && skip_r > 0 && norm3(poi) > skip_r) live = false;
    nq.put_target(w, lane, poi, mk3(0, 0, 0));
    const PtF pf = split_pt(poi);
    const int64_t jb = (int64_t)blockIdx.y * chunk, je = min(nb, jb + chunk);
    dv3 acc = mk3(0, 0, 0);
    KSum3 fa;
    for (int64_t b = jb; b < je; b += TILE) {
        int lim = (int)((je - b) < TILE ? (je - b) : TILE);
        __syncthreads();
        for (int k = threadIdx.x; k < lim * R_STRIDE; k += VT) tile[k] = rec[b * R_STRIDE + k];
        for (int k = threadIdx.x; k < lim; k += VT) {
            ts[k] = sigma[b + k];
            tm[k] = mu[b + k];
            fill_ftile(rec + (b + k) * R_STRIDE, ts[k], tm[k], ft + k * FT_STRIDE);
        }
        __syncthreads();
        int qn = 0;
        for (int k = 0; k < lim; k++) {
            bool near = false;
            if (live) {
                const float* f = ft + k * FT_STRIDE;
                float dx, dy, dz, d2;
                if (far_pair(pf, f, tile + k * R_STRIDE, poi, dx, dy, dz, d2)) {
                    // sigma vSrc + mu vDub = (3 ad pn / d^2 - as) / d^3 (p - c) - ad / d^3 n
                    const float inv = rsqrtf(d2), i2 = inv * inv, i3 = i2 * inv;
                    const float nx = f[FT_N], ny = f[FT_N + 1], nz = f[FT_N + 2];
                    const float pn = dx * nx + dy * ny + dz * nz;
                    const float ad = f[FT_AD];
                    const float cp = (3 * ad * pn * i2 - f[FT_AS]) * i3, cn = ad * i3;
                    fa.add(cp * dx - cn * nx, cp * dy - cn * ny, cp * dz - cn * nz);
                } else {
                    near = true;
                }
            }
            qn = nq.push(w, lane, near, k, qn);
        }
        __syncwarp();
        for (int base = 0; base < qn; base += 32) {  // FP64 near pairs, one per lane
            int kk, ln;
            if (nq.take(w, base + lane, qn, kk, ln)) {
                dv3 vs, vd;
                panel_v_inf(tile + kk * R_STRIDE, nq.tx(w, ln), vs, vd);
                nq.put_result(w, lane, ln, ts[kk] * vs + tm[kk] * vd);
            }
            acc = nq.gather(w, lane, base, qn, acc);
        }
    }
    if (t >= m) return;
    acc = acc + fa.value();
    double* o = part + ((int64_t)blockIdx.y * m + q) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
}

__global__ void __launch_bounds__(VT) k_vp_stretch_part_f32(const double* __restrict__ rec,
                                                            const double* __restrict__ sigma,
                                                            const double* __restrict__ mu, int64_t nb, int64_t chunk,
                                                            const double* __restrict__ pos,
                                                            const double* __restrict__ str, int64_t m,
                                                            double skip_x, double* __restrict__ part, int64_t sinv) {
    __shared__ double tile[TILE * R_STRIDE];
    __shared__ double ts[TILE], tm[TILE];
    __shared__ float ft[TILE * FT_STRIDE];
    __shared__ NearQueue nq;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = t < m;
    const int64_t q = live ? (int64_t)(((uint64_t)t * (uint64_t)sinv) % (uint64_t)m) : 0;
    dv3 x = live ? ld3(pos + 3 * q) : mk3(0, 0, 0);
    dv3 a = live ? ld3(str + 3 * q) : mk3(0, 0, 0);
    if (live && skip_x > 0 && fabs(x.x) > skip_x) live = false;
    nq.put_target(w, lane, x, a);
    const PtF pf = split_pt(x);
    const float ax = (float)a.x, ay = (float)a.y, az = (float)a.z;
    const int64_t jb = (int64_t)blockIdx.y * chunk, je = min(nb, jb + chunk);
    dv3 acc = mk3(0, 0, 0);
    KSum3 fa;
    for (int64_t b = jb; b < je; b += TILE) {
        int lim = (int)((je - b) < TILE ? (je - b) : TILE);
        __syncthreads();
        for (int k = threadIdx.x; k < lim * R_STRIDE; k += VT) tile[k] = rec[b * R_STRIDE + k];
        for (int k = threadIdx.x; k < lim; k += VT) {
            ts[k] = sigma[b + k];
            tm[k] = mu[b + k];
            fill_ftile(rec + (b + k) * R_STRIDE, ts[k], tm[k], ft + k * FT_STRIDE);
        }
        __syncthreads();
        int qn = 0;  // warp-uniform: near pairs of this warp in this tile
        for (int k = 0; k < lim; k++) {
            bool near = false;
            if (live) {
                const float* f = ft + k * FT_STRIDE;
                const double* r = tile + k * R_STRIDE;
                float ddx, ddy, ddz, d2;
                if (far_pair(pf, f, r, x, ddx, ddy, ddz, d2)) {
                    // velocityGradientPointSource + velocityGradientPointDoublet in FP32, with
                    // the reference's terms: dx = c.x - x, dy = c.y - y, z = c.z, z - z0 = c.z - x.z
                    const float dx = -ddx, dy = -ddy, zz = -ddz;
                    const float z = f[FT_CH + 2] + f[FT_CL + 2];
                    const float dx2 = dx * dx, dy2 = dy * dy, z2 = z * z;
                    const float bb = dx2 + dy2 + z2;
                    const float sb = sqrtf(bb);
                    const float is = f[FT_AS] / (bb * bb * sb);          // sigma area / 4 pi / sdd
                    const float id = 1.0f / (bb * bb * bb * sb);          // 1 / ddd
                    const float uv = 3 * f[FT_AD] * id, wd = -f[FT_AD] * id;
                    const float e = dx2 + dy2 - 4 * z2;
                    float G00 = is * (-2 * dx2 + dy2 + z2) + uv * z * (-4 * dx2 + dy2 + z2);
                    float G10 = is * (-3 * dx * dy) + uv * (-5) * z * dy * dx;
                    float G20 = is * (-3 * dx * z) + uv * dx * e;
                    float G01 = is * (-3 * dx * dy) + uv * (-5) * dx * dy * z;
                    float G11 = is * (dx2 - dy2 + z2) + uv * z * (dx2 - 4 * dy2 + z2);
                    float G21 = is * (-3 * z * dy) + uv * dy * e;
                    float G02 = is * (-3 * dx * zz) + wd * (-3) * dx * e;
                    float G12 = is * (-3 * dy * zz) + wd * (-3) * dy * e;
                    float G22 = is * (-3 * z * zz + bb) + wd * (-3) * z * (3 * dx2 + 3 * dy2 - 2 * z2);
                    fa.add(G00 * ax + G01 * ay + G02 * az, G10 * ax + G11 * ay + G12 * az,
                           G20 * ax + G21 * ay + G22 * az);
                } else {
                    near = true;
                }
            }
            qn = nq.push(w, lane, near, k, qn);
        }
        __syncwarp();
        // the warp's FP64 near pairs, one per lane (bodyPanel::partStretching near branch)
        for (int base = 0; base < qn; base += 32) {
            int kk, ln;
            if (nq.take(w, base + lane, qn, kk, ln)) {
                const double* r = tile + kk * R_STRIDE;
                const dv3 xe = nq.tx(w, ln), ae = nq.ta(w, ln);
                dv3 c = ld3(r + R_C);
                dm3 g1 = vel_grad_tri_source(r, ts[kk], xe);
                dm3 g2 = vel_grad_doublet(r, 3, c, ld3(r + R_N), ld3(r + R_L), ld3(r + R_M), r[R_LONG], tm[kk], xe);
                dm3 G;
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) G.a[i][j] = (0 + g1.a[i][j]) + g2.a[i][j];
                nq.put_result(w, lane, ln, mul_m3(G, ae));
            }
            acc = nq.gather(w, lane, base, qn, acc);
        }
    }
    if (t >= m) return;
    acc = acc + fa.value();
    double* o = part + ((int64_t)blockIdx.y * m + q) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
}

// A = A32 + Alo: the FP64 matrix as a float pair (the mixed-precision solve factors A32
// and refines against both)
__global__ void k_vp_split(const double* __restrict__ A, int64_t nn, float* __restrict__ A32, float* __restrict__ Alo) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    const double a = A[i];
    const float h = __double2float_rn(a);
    A32[i] = h;
    Alo[i] = __double2float_rn(a - (double)h);
}

__global__ void k_vp_add(double* __restrict__ y, const double* __restrict__ x, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = y[i] + x[i];
}

// one warp per particle: lanes share the first-row quads (wakePanel::partStretching)
__global__ void k_vp_stretch_fin(const double* __restrict__ part, int64_t nchunk, const double* __restrict__ q1,
                                 const double* __restrict__ mu1, int64_t n1, const double* __restrict__ pos,
                                 const double* __restrict__ str, int64_t m, double skip_x, double* __restrict__ out) {
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= m) return;  // uniform across the warp
    dv3 x = ld3(pos + 3 * q), a = ld3(str + 3 * q);
    if (skip_x > 0 && fabs(x.x) > skip_x) {
        if (lane == 0) out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = 0;
        return;
    }
    dv3 acc = mk3(0, 0, 0);
    for (int64_t j = lane; j < n1; j += 32) {
        const double* w = q1 + j * Q_STRIDE;
        dv3 c = ld3(w + Q_C);
        dm3 G = norm3(x - c) / w[Q_LONG] > 5
                    ? vel_grad_point_doublet(c, w[Q_AREA], mu1[j], x)
                    : vel_grad_doublet(w, 4, c, ld3(w + Q_N), ld3(w + Q_L), ld3(w + Q_M), w[Q_LONG], mu1[j], x);
        acc = acc + mul_m3(G, a);
    }
    // body chunks: lane l adds chunks l, l+32, ... (then the same butterfly)
    dv3 body = mk3(0, 0, 0);
    for (int64_t c = lane; c < nchunk; c += 32) body = body + ld3(part + (c * m + q) * 3);
    body = warp_sum3(body);
    acc = warp_sum3(acc);
    if (lane != 0) return;
    const dv3 tot = body + acc;
    out[3 * q] = tot.x;
    out[3 * q + 1] = tot.y;
    out[3 * q + 2] = tot.z;
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
// vtot (optional, n x 3): the same onset velocity summed as cpCaseVP::VinfPlusVecPot does
// (CPanel/cpCaseVP.cpp:601-623: free stream, then particles, then each filament), whose dot
// product with the centre gives the panel potential of solveVPmatrixEq
__global__ void k_vp_sigma(const double* __restrict__ rec, int64_t n, const double* __restrict__ vpart,
                           const double* __restrict__ fil, int64_t nf, dv3 vinf, double* __restrict__ sigma,
                           double* __restrict__ vtot) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dv3 c = ld3(rec + i * R_STRIDE + R_C), nn = ld3(rec + i * R_STRIDE + R_N);
    dv3 s = vpart ? ld3(vpart + 3 * i) : mk3(0, 0, 0);
    dv3 t = vinf + s;
    for (int64_t j = 0; j < nf; j++) {
        const double* f = fil + 8 * j;
        dv3 p1 = ld3(f), p2 = ld3(f + 3);
        dv3 term = (f[6] * vortex_v(c - p1, c - p2, p2 - p1)) / CPG_FOUR_PI;
        s = s + term;
        t = t + term;
    }
    sigma[i] = -dot3(vinf + s, nn) + 0;
    if (vtot) {
        vtot[3 * i] = t.x;
        vtot[3 * i + 1] = t.y;
        vtot[3 * i + 2] = t.z;
    }
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
cudaError_t vp_launch_add(double* y, const double* x, int64_t n, cudaStream_t s) {
    if (n > 0) k_vp_add<<<nblk(n, 256), 256, 0, s>>>(y, x, n);
    return cudaGetLastError();
}
cudaError_t vp_launch_split(const double* A, int64_t nn, float* A32, float* Alo, cudaStream_t s) {
    if (nn > 0) k_vp_split<<<nblk(nn, 256), 256, 0, s>>>(A, nn, A32, Alo);
    return cudaGetLastError();
}
cudaError_t vp_launch_cmat(const double* rec, int64_t n, const double* q2, int64_t n2, double* C, cudaStream_t s) {
    if (n > 0 && n2 > 0) k_vp_cmat<<<nblk(n * n2, 256), 256, 0, s>>>(rec, n, q2, n2, C);
    return cudaGetLastError();
}
// chunks of body panels along grid.y: enough blocks to fill the GPU several times over
// panel chunks along grid.y: about 4 blocks per SM in all, chunks of at least CHUNK_MIN
// panels (a handful of points then still spreads over the SMs)
constexpr int CHUNK_MIN = 16;
int64_t vp_chunks(int64_t m, int64_t nb) {
    int64_t bx = (m + VT - 1) / VT;
    int64_t maxc = (nb + CHUNK_MIN - 1) / CHUNK_MIN;
    int64_t c = (4 * 152 + bx - 1) / bx;
    return std::max<int64_t>(1, std::min(c, maxc));
}
int64_t vp_chunk_size(int64_t m, int64_t nb) {
    const int64_t nc = vp_chunks(m, nb);
    return nb > 0 ? ((nb + nc - 1) / nc + CHUNK_MIN - 1) / CHUNK_MIN * CHUNK_MIN : CHUNK_MIN;
}

int64_t vp_scratch_doubles(int64_t m, int64_t nb) { return vp_chunks(m, nb) * m * 3; }

// Target t of a panel kernel handles point (t * sinv) mod m, a bijection when sinv is
// prime to m: points with consecutive indices (a row of particles shed in one step, which
// meet the body panels' FP64 near field together) land in distant blocks, so that work
// spreads over all SMs.  Each point's sums are the same in any placement.
int64_t spread_inverse(int64_t m) {
    if (m <= 2) return 1;
    int64_t s = (int64_t)(0.6180339887498949 * (double)m);
    auto gcd = [](int64_t a, int64_t b) {
        while (b) {
            int64_t r = a % b;
            a = b;
            b = r;
        }
        return a;
    };
    while (gcd(s, m) != 1) s++;
    // inverse of s modulo m (extended Euclid)
    int64_t r0 = m, r1 = s, t0 = 0, t1 = 1;
    while (r1) {
        const int64_t qq = r0 / r1, r2 = r0 - qq * r1, t2 = t0 - qq * t1;
        r0 = r1;
        r1 = r2;
        t0 = t1;
        t1 = t2;
    }
    return t0 < 0 ? t0 + m : t0;
}

cudaError_t vp_launch_panel_vel(const double* rec, const double* sigma, const double* mu, int64_t nb, const double* q1,
                                const double* mu1, int64_t n1, const double* q2, const double* mu2, int64_t n2,
                                const double* fil, int64_t nf, const double* pts, int64_t m, double skip_r,
                                double* out, double* scratch, cudaStream_t s, bool far_f32) {
    if (m <= 0) return cudaSuccess;
    const int64_t chunk = vp_chunk_size(m, nb);
    const int64_t ncu = nb > 0 ? (nb + chunk - 1) / chunk : 0;
    if (ncu > 0 && far_f32)
        k_vp_panel_vel_part_f32<<<dim3(nblk(m, VT), (unsigned)ncu), VT, 0, s>>>(rec, sigma, mu, nb, chunk, pts, m,
                                                                               skip_r, scratch, spread_inverse(m));
    else if (ncu > 0)
        k_vp_panel_vel_part<<<dim3(nblk(m, VT), (unsigned)ncu), VT, 0, s>>>(rec, sigma, mu, nb, chunk, pts, m, skip_r,
                                                                           scratch, spread_inverse(m));
    k_vp_panel_vel_fin<<<nblk(32 * m, 128), 128, 0, s>>>(scratch, ncu, q1, mu1, n1, q2, mu2, n2, fil, nf, pts, m, skip_r,
                                                    out);
    return cudaGetLastError();
}
cudaError_t vp_launch_stretch_panels(const double* rec, const double* sigma, const double* mu, int64_t nb,
                                     const double* q1, const double* mu1, int64_t n1, const double* pos,
                                     const double* str, int64_t m, double skip_x, double* out, double* scratch,
                                     cudaStream_t s, bool far_f32) {
    if (m <= 0) return cudaSuccess;
    const int64_t chunk = vp_chunk_size(m, nb);
    const int64_t ncu = nb > 0 ? (nb + chunk - 1) / chunk : 0;
    if (ncu > 0 && far_f32)
        k_vp_stretch_part_f32<<<dim3(nblk(m, VT), (unsigned)ncu), VT, 0, s>>>(rec, sigma, mu, nb, chunk, pos, str, m,
                                                                             skip_x, scratch, spread_inverse(m));
    else if (ncu > 0)
        k_vp_stretch_part<<<dim3(nblk(m, VT), (unsigned)ncu), VT, 0, s>>>(rec, sigma, mu, nb, chunk, pos, str, m,
                                                                         skip_x, scratch, spread_inverse(m));
    k_vp_stretch_fin<<<nblk(32 * m, 128), 128, 0, s>>>(scratch, ncu, q1, mu1, n1, pos, str, m, skip_x, out);
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
                            const double vinf[3], double* sigma, double* vtot, cudaStream_t s) {
    if (n > 0)
        k_vp_sigma<<<nblk(n, 256), 256, 0, s>>>(rec, n, vpart, fil, nf, dv3{vinf[0], vinf[1], vinf[2]}, sigma, vtot);
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
