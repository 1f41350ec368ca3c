// Influence-matrix assembly (geometry::setInfCoeff, CPanel/geometry.cpp:809-891).
//
// Compiled with --fmad=false (see panel64.cuh).  Layout: A(i,j) at A[j*n + i]
// (column-major like the reference's Eigen::MatrixXd), i = target centroid,
// j = source panel.  A block owns 128 consecutive targets and a contiguous range of
// source panels, staged 32 at a time in shared memory; each store instruction of
// a warp writes 32 consecutive rows of one column.
#include <mutex>

#include "../../include/cpanel_gpu.h"
#include "assemble.h"
#include "df.cuh"
#include "panel64.cuh"
#include "particles.h"

namespace {

constexpr int TI = 128;   // targets per block (threads)
constexpr int TJ = 32;    // sources per shared-memory tile

__device__ __forceinline__ void load_tile(double* s_rec, const double* __restrict__ rec, int64_t j0, int64_t n) {
    const int tot = TJ * R_STRIDE;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        int64_t j = j0 + t / R_STRIDE;
        s_rec[t] = j < n ? rec[j0 * R_STRIDE + t] : 0.0;
    }
}

// Plain FP64: writes A and B for the body panels.
__global__ void __launch_bounds__(TI) k_assemble_fp64(const double* __restrict__ rec, int64_t n, int64_t jchunk,
                                                      double* __restrict__ A, double* __restrict__ B,
                                                      unsigned long long* __restrict__ near_count) {
    __shared__ double s_rec[TJ * R_STRIDE];
    int64_t i = (int64_t)blockIdx.x * TI + threadIdx.x;
    bool act = i < n;
    dv3 poi = act ? ld3(rec + i * R_STRIDE + R_C) : mk3(0, 0, 0);
    int64_t jb = (int64_t)blockIdx.y * jchunk, je = min(n, jb + jchunk);
    unsigned nnear = 0;
    for (int64_t j0 = jb; j0 < je; j0 += TJ) {
        __syncthreads();
        load_tile(s_rec, rec, j0, n);
        __syncthreads();
        int cnt = (int)min((int64_t)TJ, je - j0);
        if (!act) continue;
        for (int t = 0; t < cnt; t++) {
            int64_t j = j0 + t;
            double src = 0, dub = 0;
            nnear += panel_phi_inf(s_rec + t * R_STRIDE, poi, src, dub);
            A[j * n + i] = dub;
            B[j * n + i] = src;
        }
    }
    if (near_count) {
        for (int o = 16; o > 0; o >>= 1) nnear += __shfl_down_sync(0xffffffffu, nnear, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(near_count, (unsigned long long)nnear);
    }
}

// Mixed: double-float far field, FP64 near field (the reference's own near set,
// |pjk| <= 5 longSide).  A is stored as two FP32 matrices, hi and lo, whose sum
// carries about 44 bits; the Krylov iterations read hi only, the refinement
// residual reads both.  Instead of storing B, the source right-hand-side basis
// rb[c*n+i] = sum_j B(i,j) * n_j[c] is accumulated (double-float per tile, FP64
// across tiles and for near pairs).  Each column chunk writes its own partial sums
// (rbp[(chunk*3 + c)*n + i]); k_rb_reduce adds the chunks in order, so the result does
// not depend on block scheduling.
__global__ void __launch_bounds__(TI) k_assemble_mixed(const double* __restrict__ rec, const float* __restrict__ frec,
                                                       int64_t n, int64_t jchunk, float* __restrict__ A32,
                                                       float* __restrict__ Alo, double* __restrict__ rbp,
                                                       unsigned long long* __restrict__ near_count) {
    __shared__ double s_rec[TJ * R_STRIDE];
    __shared__ float s_f[TJ * F_STRIDE];
    int64_t i = (int64_t)blockIdx.x * TI + threadIdx.x;
    bool act = i < n;
    dv3 poi = act ? ld3(rec + i * R_STRIDE + R_C) : mk3(0, 0, 0);
    df32 ci[3] = {{0, 0}, {0, 0}, {0, 0}};
    if (act)
        for (int c = 0; c < 3; c++) ci[c] = df32{frec[i * F_STRIDE + F_CHI + c], frec[i * F_STRIDE + F_CLO + c]};
    int64_t jb = (int64_t)blockIdx.y * jchunk, je = min(n, jb + jchunk);
    double acc64[3] = {0, 0, 0};
    unsigned nnear = 0;
    const double q4 = 1.0 / CPG_FOUR_PI;
    const df32 inv4pi = df32{(float)q4, (float)(q4 - (double)(float)q4)};
    for (int64_t j0 = jb; j0 < je; j0 += TJ) {
        __syncthreads();
        load_tile(s_rec, rec, j0, n);
        for (int t = threadIdx.x; t < TJ * F_STRIDE; t += blockDim.x) {
            int64_t j = j0 + t / F_STRIDE;
            s_f[t] = j < n ? frec[j0 * F_STRIDE + t] : 0.f;
        }
        __syncthreads();
        int cnt = (int)min((int64_t)TJ, je - j0);
        if (!act) continue;
        df32 acc[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (int t = 0; t < cnt; t++) {
            int64_t j = j0 + t;
            const float* f = s_f + t * F_STRIDE;
            df32 d[3];
#pragma unroll
            for (int c = 0; c < 3; c++) d[c] = df_sub(ci[c], df32{f[F_CHI + c], f[F_CLO + c]});
            float r2f = __fmaf_rn(d[2].hi, d[2].hi, __fmaf_rn(d[1].hi, d[1].hi, __fmul_rn(d[0].hi, d[0].hi)));
            float L = f[F_LONG];
            float lim = __fmul_rn(25.f, __fmul_rn(L, L));
            bool far;
            if (r2f > __fmul_rn(lim, 1.00001f))
                far = true;
            else if (r2f < __fmul_rn(lim, 0.99999f))
                far = false;
            else {  // guard band: decide exactly as the FP64 reference does
                const double* r = s_rec + t * R_STRIDE;
                double dd = norm3(poi - ld3(r + R_C));
                far = dd / r[R_LONG] > 5;
            }
            if (far) {
                // pntSrcPhi / pntDubPhi (CPanel/bodyPanel.cpp:392-395, panel.cpp:737-740) in double-float
                df32 r2 = df_add(df_add(df_mul(d[0], d[0]), df_mul(d[1], d[1])), df_mul(d[2], d[2]));
                df32 rinv = df_rsqrt(r2);
                df32 src = df_mul(df_mul(df32{f[F_AHI], f[F_ALO]}, rinv), inv4pi);
                df32 nv[3] = {{f[F_NHI], f[F_NLO]}, {f[F_NHI + 1], f[F_NLO + 1]}, {f[F_NHI + 2], f[F_NLO + 2]}};
                df32 pn = df_add(df_add(df_mul(d[0], nv[0]), df_mul(d[1], nv[1])), df_mul(d[2], nv[2]));
                df32 dub = df_mul(df_mul(pn, df_mul(rinv, rinv)), src);
                A32[j * n + i] = dub.hi;
                Alo[j * n + i] = dub.lo;
#pragma unroll
                for (int c = 0; c < 3; c++) acc[c] = df_add(acc[c], df_mul(src, nv[c]));
            } else {
                double src = 0, dub = 0;
                const double* r = s_rec + t * R_STRIDE;
                panel_phi_inf(r, poi, src, dub);
                nnear++;
                float hi = (float)dub;
                A32[j * n + i] = hi;
                Alo[j * n + i] = (float)(dub - (double)hi);  // FP64 value = hi + lo to 2^-48
                acc64[0] += src * r[R_N + 0];
                acc64[1] += src * r[R_N + 1];
                acc64[2] += src * r[R_N + 2];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) acc64[c] += df_to_double(acc[c]);
    }
    if (act) {
        double* part = rbp + (int64_t)blockIdx.y * 3 * n;
        part[i] = acc64[0];
        part[n + i] = acc64[1];
        part[2 * n + i] = acc64[2];
    }
    if (near_count) {
        for (int o = 16; o > 0; o >>= 1) nnear += __shfl_down_sync(0xffffffffu, nnear, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(near_count, (unsigned long long)nnear);
    }
}

// Wake doublet columns, CPanel/geometry.cpp:853-873.  One thread per target row
// walks the wake panels in wPanels order, so each of the (at most four) columns a
// wake panel touches receives its contributions in the reference's order.
template <typename T>
__global__ void k_wake_columns(const double* __restrict__ rec, const double* __restrict__ wrec,
                               const int32_t* __restrict__ widx, const double* __restrict__ wcoef, int64_t n,
                               int64_t nw, T* __restrict__ A) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dv3 poi = ld3(rec + i * R_STRIDE + R_C);
    for (int64_t j = 0; j < nw; j++) {
        double infl = dub_phi_inf(wrec + j * R_STRIDE, poi);
        double c = wcoef[j];
        const int32_t* ix = widx + 4 * j;
        int64_t c0 = ix[0], c1 = ix[1], c2 = ix[2], c3 = ix[3];
        A[c0 * n + i] = (T)((double)A[c0 * n + i] + infl * (1 - c));
        A[c1 * n + i] = (T)((double)A[c1 * n + i] + infl * (c - 1));
        A[c2 * n + i] = (T)((double)A[c2 * n + i] + infl * c);
        A[c3 * n + i] = (T)((double)A[c3 * n + i] - infl * c);
    }
}

// Wake columns for the split (hi + lo) FP32 storage of the mixed path.
__global__ void k_wake_columns_split(const double* __restrict__ rec, const double* __restrict__ wrec,
                                     const int32_t* __restrict__ widx, const double* __restrict__ wcoef, int64_t n,
                                     int64_t nw, float* __restrict__ Ahi, float* __restrict__ Alo) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dv3 poi = ld3(rec + i * R_STRIDE + R_C);
    for (int64_t j = 0; j < nw; j++) {
        double infl = dub_phi_inf(wrec + j * R_STRIDE, poi);
        double c = wcoef[j];
        const int32_t* ix = widx + 4 * j;
        const double add[4] = {infl * (1 - c), infl * (c - 1), infl * c, -(infl * c)};
        for (int q = 0; q < 4; q++) {
            int64_t o = (int64_t)ix[q] * n + i;
            double v = ((double)Ahi[o] + (double)Alo[o]) + add[q];
            float hi = (float)v;
            Ahi[o] = hi;
            Alo[o] = (float)(v - (double)hi);
        }
    }
}

__global__ void k_rb_reduce(const double* __restrict__ rbp, int64_t n, int64_t chunks, double* __restrict__ rb) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    double acc = 0;
    for (int64_t y = 0; y < chunks; y++) acc += rbp[y * 3 * n + t];
    rb[t] = acc;
}

// panel::setGeom + getLocalSys on the device for free triangles (batched API).
__device__ void make_record(const double* v9, double* r) {
    dv3 p0 = ld3(v9), p1 = ld3(v9 + 3), p2 = ld3(v9 + 6);
    double ls = 0;
    dv3 pp[3] = {p0, p1, p2};
    for (int k = 0; k < 3; k++) {
        double l = norm3(pp[k == 2 ? 0 : k + 1] - pp[k]);
        if (l > ls) ls = l;
    }
    dv3 a = p1 - p0, b = p2 - p0;
    dv3 c = ((p0 + p1) + p2) / 3.0;
    double th = acos(dot3(a, b) / (norm3(a) * norm3(b)));
    double area = 0.5 * norm3(a) * norm3(b) * sin(th);
    dv3 nn = cross3(a, b);
    double z = dot3(nn, nn);
    dv3 n = z > 0 ? nn / sqrt(z) : nn;
    dv3 l0 = p0 - c;
    double zl = dot3(l0, l0);
    dv3 l = zl > 0 ? l0 / sqrt(zl) : l0;
    dv3 m = cross3(n, l);
    for (int k = 0; k < 9; k++) r[k] = v9[k];
    const dv3 f[4] = {c, n, l, m};
    for (int q = 0; q < 4; q++) {
        r[R_C + 3 * q] = f[q].x;
        r[R_C + 3 * q + 1] = f[q].y;
        r[R_C + 3 * q + 2] = f[q].z;
    }
    r[R_AREA] = area;
    r[R_LONG] = ls;
    r[23] = 0;
}

__global__ void k_phi_batch(const double* __restrict__ verts, const double* __restrict__ poi, int64_t m,
                            double* __restrict__ src, double* __restrict__ dub, int mode) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    double r[R_STRIDE];
    make_record(verts + 9 * t, r);
    dv3 p = ld3(poi + 3 * t);
    if (mode == 0) {
        double s = 0, d = 0;
        panel_phi_inf(r, p, s, d);
        src[t] = s;
        dub[t] = d;
    } else {
        dub[t] = dub_phi_inf(r, p);
    }
}

__global__ void k_v_batch(const double* __restrict__ verts, const double* __restrict__ poi, int64_t m,
                          double* __restrict__ vs, double* __restrict__ vd) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    double r[R_STRIDE];
    make_record(verts + 9 * t, r);
    dv3 a, b;
    panel_v_inf(r, ld3(poi + 3 * t), a, b);
    vs[3 * t] = a.x;
    vs[3 * t + 1] = a.y;
    vs[3 * t + 2] = a.z;
    vd[3 * t] = b.x;
    vd[3 * t + 1] = b.y;
    vd[3 * t + 2] = b.z;
}

// Trefftz-plane potential operator G(p, w) = dubPhiInf_w(p) (FP64, per mesh).
__global__ void k_wake_potential_op(const double* __restrict__ wrec, int64_t nw, const double* __restrict__ pts,
                                    int64_t np, double* __restrict__ G) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np * nw) return;
    int64_t p = t / nw, w = t % nw;
    G[t] = dub_phi_inf(wrec + w * R_STRIDE, ld3(pts + 3 * p));
}

__global__ void k_pack_records(const double* __restrict__ verts, int64_t m, double* __restrict__ rec) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m) make_record(verts + 9 * t, rec + t * R_STRIDE);
}

// Panel-induced velocity at points (the panel terms of cpCaseVP::velocityInflFromEverything,
// CPanel/cpCaseVP.cpp:713-731): sum_j sigma_j vSrc_j + mu_j vDub_j over body records
// (bodyPanel::panelV, bodyPanel.cpp:122-130), then mu_w dubVInf over wake records
// (wakePanel::panelV, wakePanel.cpp:89-92).  One thread per point; records are staged
// through shared memory in tiles shared by the block.
constexpr int PV_T = 128, PV_TILE = 64;
__global__ void __launch_bounds__(PV_T) k_panels_velocity(const double* __restrict__ rec, const double* __restrict__ sigma,
                                                          const double* __restrict__ mu, int64_t nb,
                                                          const double* __restrict__ wmu, int64_t nw,
                                                          const double* __restrict__ pts, int64_t m,
                                                          double* __restrict__ vel) {
    __shared__ double tile[PV_TILE * R_STRIDE];
    __shared__ double ts[PV_TILE], tm[PV_TILE];
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool live = q < m;
    dv3 poi = live ? ld3(pts + 3 * q) : mk3(0, 0, 0);
    dv3 acc = mk3(0, 0, 0);
    const int64_t tot = nb + nw;
    for (int64_t b = 0; b < tot; b += PV_TILE) {
        int lim = (int)((tot - b) < PV_TILE ? (tot - b) : PV_TILE);
        __syncthreads();
        for (int k = threadIdx.x; k < lim * R_STRIDE; k += PV_T) tile[k] = rec[b * R_STRIDE + k];
        for (int k = threadIdx.x; k < lim; k += PV_T) {
            int64_t j = b + k;
            ts[k] = j < nb ? sigma[j] : 0.0;
            tm[k] = j < nb ? mu[j] : wmu[j - nb];
        }
        __syncthreads();
        if (!live) continue;
        for (int k = 0; k < lim; k++) {
            const double* r = tile + k * R_STRIDE;
            if (b + k < nb) {
                dv3 vs, vd;
                panel_v_inf(r, poi, vs, vd);
                acc = acc + (ts[k] * vs + tm[k] * vd);
            } else {
                acc = acc + tm[k] * dub_v_inf(r, poi);
            }
        }
    }
    if (!live) return;
    vel[3 * q] = acc.x;
    vel[3 * q + 1] = acc.y;
    vel[3 * q + 2] = acc.z;
}

int64_t chunk_for(int64_t n) {
    // enough blocks in y to fill the 152 SMs several times over
    int64_t bx = (n + TI - 1) / TI;
    int64_t want = 152 * 16;
    int64_t by = (want + bx - 1) / bx;
    if (by < 1) by = 1;
    int64_t ch = (n + by - 1) / by;
    ch = ((ch + TJ - 1) / TJ) * TJ;
    return ch < TJ ? TJ : ch;
}

}  // namespace

namespace cpg {

cudaError_t launch_pack_records(const double* verts, int64_t m, double* rec, cudaStream_t s) {
    if (m > 0) k_pack_records<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(verts, m, rec);
    return cudaGetLastError();
}

cudaError_t launch_panels_velocity(const double* body_verts, const double* sigma, const double* mu, int64_t nb,
                                   const double* wake_verts, const double* wmu, int64_t nw, const double* pts,
                                   int64_t m, double* rec, double* vel, cudaStream_t s) {
    if (nb > 0) k_pack_records<<<(unsigned)((nb + 127) / 128), 128, 0, s>>>(body_verts, nb, rec);
    if (nw > 0) k_pack_records<<<(unsigned)((nw + 127) / 128), 128, 0, s>>>(wake_verts, nw, rec + nb * R_STRIDE);
    if (m > 0) k_panels_velocity<<<(unsigned)((m + PV_T - 1) / PV_T), PV_T, 0, s>>>(rec, sigma, mu, nb, wmu, nw, pts, m, vel);
    return cudaGetLastError();
}

cudaError_t launch_assemble_fp64(const double* rec, int64_t n, const double* wrec, const int32_t* widx,
                                 const double* wcoef, int64_t nw, double* A, double* B,
                                 unsigned long long* near_count, cudaStream_t s) {
    int64_t ch = chunk_for(n);
    dim3 grid((unsigned)((n + TI - 1) / TI), (unsigned)((n + ch - 1) / ch));
    {
        ProfScope ps(Prof::ASSEMBLE, s);
        k_assemble_fp64<<<grid, TI, 0, s>>>(rec, n, ch, A, B, near_count);
    }
    if (nw > 0) {
        ProfScope ps(Prof::WAKE_COLUMNS, s);
        k_wake_columns<double><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(rec, wrec, widx, wcoef, n, nw, A);
    }
    return cudaGetLastError();
}

cudaError_t launch_assemble_mixed(const double* rec, const float* frec, int64_t n, const double* wrec,
                                  const int32_t* widx, const double* wcoef, int64_t nw, float* A32, float* Alo,
                                  double* rb, double* rb_part, unsigned long long* near_count, cudaStream_t s) {
    int64_t ch = chunk_for(n);
    dim3 grid((unsigned)((n + TI - 1) / TI), (unsigned)((n + ch - 1) / ch));
    {
        ProfScope ps(Prof::ASSEMBLE, s);
        k_assemble_mixed<<<grid, TI, 0, s>>>(rec, frec, n, ch, A32, Alo, rb_part, near_count);
        k_rb_reduce<<<(unsigned)((3 * n + 255) / 256), 256, 0, s>>>(rb_part, n, (int64_t)grid.y, rb);
    }
    if (nw > 0) {
        ProfScope ps(Prof::WAKE_COLUMNS, s);
        k_wake_columns_split<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(rec, wrec, widx, wcoef, n, nw, A32, Alo);
    }
    return cudaGetLastError();
}

int64_t mixed_rb_part_doubles(int64_t n) {
    int64_t ch = chunk_for(n);
    return ((n + ch - 1) / ch) * 3 * n;
}

cudaError_t launch_phi_batch(const double* verts, const double* poi, int64_t m, double* src, double* dub, int mode,
                             cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    k_phi_batch<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(verts, poi, m, src, dub, mode);
    return cudaGetLastError();
}

cudaError_t launch_v_batch(const double* verts, const double* poi, int64_t m, double* vs, double* vd, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    k_v_batch<<<(unsigned)((m + 127) / 128), 128, 0, s>>>(verts, poi, m, vs, vd);
    return cudaGetLastError();
}

cudaError_t launch_wake_potential_op(const double* wrec, int64_t nw, const double* pts, int64_t np, double* G,
                                     cudaStream_t s) {
    int64_t tot = np * nw;
    if (tot <= 0) return cudaSuccess;
    k_wake_potential_op<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(wrec, nw, pts, np, G);
    return cudaGetLastError();
}

}  // namespace cpg

// ---------------------------------------------------------------------------
// Allocation-free assembly.
//
// Some callers cannot allocate device memory while they run this path: a host
// that records the influence assembly into a CUDA graph, a plug-in living inside
// another solver's memory pool, or a real-time loop that has forbidden allocation
// after start-up.  cpg_set_inf_coeff_noalloc serves them.  It runs the same FP64
// kernels as cpg_set_inf_coeff, but the one scratch table those kernels need (the
// packed 192-byte panel records, normally held by a cpg_geometry) lives in the
// fixed array below.  Every GPU that loads this library keeps that array
// (kNoAllocMaxPanels * 192 bytes, about 3 MB) until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocMaxPanels = 16384;  // body + wake panels per call
static __device__ __align__(256) double g_noalloc_records[kNoAllocMaxPanels * R_STRIDE];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the array on the current device.  The array's host-side name
// is only a stand-in, so the address is looked up once per device, with that
// device current.
cudaError_t noalloc_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_noalloc_records);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int cpg_set_inf_coeff_noalloc(const double* body_verts, int64_t n, const double* wake_verts,
                                         const int32_t* wake_idx4, const double* wake_coef, int64_t nw,
                                         double* A, double* B, void* stream) {
    if (n < 1 || nw < 0 || n + nw > kNoAllocMaxPanels) return CPG_E_INVALID;
    if (!body_verts || !A || !B || (nw > 0 && (!wake_verts || !wake_idx4 || !wake_coef))) return CPG_E_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    double* rec = nullptr;
    if (noalloc_scratch(&rec) != cudaSuccess) return CPG_E_CUDA;
    double* wrec = rec + n * R_STRIDE;
    // every record the kernels read is rewritten here, so no clearing is needed
    k_pack_records<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(body_verts, n, rec);
    if (nw > 0) k_pack_records<<<(unsigned)((nw + 127) / 128), 128, 0, s>>>(wake_verts, nw, wrec);
    int64_t ch = chunk_for(n);
    dim3 grid((unsigned)((n + TI - 1) / TI), (unsigned)((n + ch - 1) / ch));
    k_assemble_fp64<<<grid, TI, 0, s>>>(rec, n, ch, A, B, nullptr);
    if (nw > 0)
        k_wake_columns<double><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(rec, wrec, wake_idx4, wake_coef, n, nw, A);
    return cudaGetLastError() == cudaSuccess ? CPG_OK : CPG_E_CUDA;
}
