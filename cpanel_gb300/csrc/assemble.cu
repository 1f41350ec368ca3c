// Influence-matrix assembly (geometry::setInfCoeff, CPanel/geometry.cpp:809-891).
//
// Compiled with --fmad=false (see panel64.cuh).  Layout: A(i,j) at A[j*n + i]
// (column-major like the reference's Eigen::MatrixXd), i = target centroid,
// j = source panel.  A block owns 128 consecutive targets and a contiguous range of
// source panels, staged 32 at a time in shared memory; each store instruction of
// a warp writes 32 consecutive rows of one column.
#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/cpanel_gpu.h"
#include "assemble.h"
#include "mesh.h"
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

// panelPhiInf (CPanel/bodyPanel.cpp:132-190) for a target between 3 and 5 longSide of the
// source, in double-float.  The three edge angles of vortexPhi sum to minus the solid angle
// of the triangle, taken here as 2 atan(N / D) (Van Oosterom and Strackee, 1983) with
// N = -2 area PN and D = |a0||a1||a2| + (a0.a1)|a2| + (a0.a2)|a1| + (a1.a2)|a0| (a_k = poi - v_k);
// there |N / D| < 0.02, so atan is a short odd series.  Each edge's log term is
// log((A+B+S)/(A+B-S)) = 2 atanh(S / (A+B)) with S / (A+B) < 0.25, also a series.  The
// edge sum of the reference loses accuracy for nearly coplanar pairs (|N / D| < 1e-6: up
// to 3e-11 absolute on the test wings); those, and anything outside the series' ranges,
// return false and take the FP64 formula.  d: poi - centroid; f: the panel's record.
struct BandPhi {
    df32 src, dub;
    bool ok;
};
__device__ __noinline__ BandPhi band_phi_df(df32 d0, df32 d1, df32 d2, const float* __restrict__ f) {
    BandPhi out{{0, 0}, {0, 0}, false};
    const df32 d[3] = {d0, d1, d2};
    const df32 nv[3] = {{f[F_NHI], f[F_NLO]}, {f[F_NHI + 1], f[F_NLO + 1]}, {f[F_NHI + 2], f[F_NLO + 2]}};
    const df32 PN = df_add(df_add(df_mul(d[0], nv[0]), df_mul(d[1], nv[1])), df_mul(d[2], nv[2]));
    df32 a[3][3], A[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int c = 0; c < 3; c++) a[k][c] = df_sub(d[c], df32{f[F_VC + 2 * (3 * k + c)], f[F_VC + 2 * (3 * k + c) + 1]});
        A[k] = df_sqrt(df_add(df_add(df_mul(a[k][0], a[k][0]), df_mul(a[k][1], a[k][1])), df_mul(a[k][2], a[k][2])));
    }
    auto dot = [&](int i, int j) {
        return df_add(df_add(df_mul(a[i][0], a[j][0]), df_mul(a[i][1], a[j][1])), df_mul(a[i][2], a[j][2]));
    };
    df32 D = df_mul(df_mul(A[0], A[1]), A[2]);
    D = df_add(D, df_mul(dot(0, 1), A[2]));
    D = df_add(D, df_mul(dot(0, 2), A[1]));
    D = df_add(D, df_mul(dot(1, 2), A[0]));
    if (!(D.hi > 0.f)) return out;
    const df32 N = df_neg(df_mul(df32{2.f * f[F_AHI], 2.f * f[F_ALO]}, PN));
    const df32 x = df_div(N, D);
    const float ax = fabsf(x.hi);
    if (ax < 1e-6f || ax > 0.02f) return out;
    // atan(x) = x (1 - u/3 + u^2/5 - ... - u^5/11), u = x^2 (next term below 2e-20 x)
    const df32 u = df_mul(x, x);
    df32 p = CPG_DFK(-1.0 / 11);
    p = df_add(df_mul(p, u), CPG_DFK(1.0 / 9));
    p = df_add(df_mul(p, u), CPG_DFK(-1.0 / 7));
    p = df_add(df_mul(p, u), CPG_DFK(1.0 / 5));
    p = df_add(df_mul(p, u), CPG_DFK(-1.0 / 3));
    p = df_add(df_mul(p, u), df32{1.f, 0.f});
    const df32 at = df_mul(x, p);
    const df32 dubs = df32{-2.f * at.hi, -2.f * at.lo};  // sum of the three edge angles
    df32 ss = {0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int k1 = k == 2 ? 0 : k + 1;
        const df32 S = {f[F_S + 2 * k], f[F_S + 2 * k + 1]}, IS = {f[F_IS + 2 * k], f[F_IS + 2 * k + 1]};
        const df32 t = df_div(S, df_add(A[k], A[k1]));
        if (!(t.hi < 0.25f)) return out;
        // atanh(t) = t (1 + w/3 + w^2/5 + ... + w^12/25), w = t^2 (next term below 1e-16 t)
        const df32 w = df_mul(t, t);
        df32 q = CPG_DFK(1.0 / 25);
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 23));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 21));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 19));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 17));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 15));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 13));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 11));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 9));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 7));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 5));
        q = df_add(df_mul(q, w), CPG_DFK(1.0 / 3));
        q = df_add(df_mul(q, w), df32{1.f, 0.f});
        const df32 at2 = df_mul(t, q);
        const df32 ns[3] = {{f[F_NS + 2 * (3 * k)], f[F_NS + 2 * (3 * k) + 1]},
                            {f[F_NS + 2 * (3 * k + 1)], f[F_NS + 2 * (3 * k + 1) + 1]},
                            {f[F_NS + 2 * (3 * k + 2)], f[F_NS + 2 * (3 * k + 2) + 1]}};
        const df32 Al = df_add(df_add(df_mul(ns[0], a[k][0]), df_mul(ns[1], a[k][1])), df_mul(ns[2], a[k][2]));
        // Al * GL with GL = 2 atanh(t) / S
        ss = df_add(ss, df_mul(Al, df_mul(df32{2.f * at2.hi, 2.f * at2.lo}, IS)));
    }
    const double q4 = 1.0 / CPG_FOUR_PI;
    const df32 inv4pi = df32{(float)q4, (float)(q4 - (double)(float)q4)};
    out.src = df_mul(df_sub(ss, df_mul(PN, dubs)), inv4pi);
    out.dub = df_mul(dubs, inv4pi);
    out.ok = true;
    return out;
}

// Mixed assembly.  Per (target, source) pair: far field (beyond 5 longSide, decided
// exactly as the reference) in double-float; between 3 and 5 longSide the exact formulas
// in double-float (band_phi_df); nearer, the FP64 formulas.  A is stored as two FP32
// matrices, hi and lo, whose sum carries about 44 bits; the factorization reads hi, the
// refinement residual both.  Instead of storing B, the source right-hand-side basis
// rb[c*n+i] = sum_j B(i,j) * n_j[c] is accumulated (double-float per tile, FP64 across
// tiles and for near pairs).  Each source chunk writes its own partial sums
// (rbp[(chunk*3 + c)*n + i]); k_rb_reduce adds the chunks in order, so the result does
// not depend on block scheduling.  The FP64 pairs of a warp are
// queued per source tile (in tile order, then lane order) and evaluated by the whole warp,
// one pair per lane, so a warp with a few near lanes does not idle the others; each target
// then adds its own queued results in queue order (the same order on every run).
constexpr int WARPS_PER_BLOCK = TI / 32;
struct MixedSmem {
    double rec[TJ * R_STRIDE];
    float f[TJ * F_STRIDE];
    double e[TJ * E_STRIDE];
    unsigned short q[WARPS_PER_BLOCK][TJ * 32];  // (tile index << 5) | lane
    double res[WARPS_PER_BLOCK][32][3];
    int own[WARPS_PER_BLOCK][32];
    double poi[WARPS_PER_BLOCK][32][3];
};

// One (row block bx, source chunk by) of the mixed assembly: targets bx*TI .. bx*TI+TI-1,
// sources by*jchunk .. min(n, (by+1)*jchunk)-1.  Safe to call back to back from one block
// (every shared tile is refilled behind a barrier; the queue arrays are per warp).
__device__ __forceinline__ void mixed_block(MixedSmem& S, const double* __restrict__ rec,
                                            const float* __restrict__ frec, const double* __restrict__ erec,
                                            int64_t n, int64_t jchunk, int64_t bx, int64_t by,
                                            float* __restrict__ A32, float* __restrict__ Alo,
                                            double* __restrict__ rbp, unsigned long long* __restrict__ near_count) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    int64_t i = bx * TI + threadIdx.x;
    const int64_t iw = bx * TI + 32 * w;  // first target of this warp
    bool act = i < n;
    dv3 poi = act ? ld3(rec + i * R_STRIDE + R_C) : mk3(0, 0, 0);
    S.poi[w][lane][0] = poi.x;
    S.poi[w][lane][1] = poi.y;
    S.poi[w][lane][2] = poi.z;
    df32 ci[3] = {{0, 0}, {0, 0}, {0, 0}};
    if (act)
        for (int c = 0; c < 3; c++) ci[c] = df32{frec[i * F_STRIDE + F_CHI + c], frec[i * F_STRIDE + F_CLO + c]};
    int64_t jb = by * jchunk, je = min(n, jb + jchunk);
    double acc64[3] = {0, 0, 0};
    unsigned nnear = 0;
    const double q4 = 1.0 / CPG_FOUR_PI;
    const df32 inv4pi = df32{(float)q4, (float)(q4 - (double)(float)q4)};
    for (int64_t j0 = jb; j0 < je; j0 += TJ) {
        __syncthreads();
        load_tile(S.rec, rec, j0, n);
        for (int t = threadIdx.x; t < TJ * F_STRIDE; t += blockDim.x) {
            int64_t j = j0 + t / F_STRIDE;
            S.f[t] = j < n ? frec[j0 * F_STRIDE + t] : 0.f;
        }
        for (int t = threadIdx.x; t < TJ * E_STRIDE; t += blockDim.x) {
            int64_t j = j0 + t / E_STRIDE;
            S.e[t] = j < n ? erec[j0 * E_STRIDE + t] : 0.0;
        }
        __syncthreads();
        int cnt = (int)min((int64_t)TJ, je - j0);
        df32 acc[3] = {{0, 0}, {0, 0}, {0, 0}};
        int qn = 0, qfar = 0;  // warp-uniform queue lengths (front and back class)
        for (int t = 0; t < cnt; t++) {
            int64_t j = j0 + t;
            const float* f = S.f + t * F_STRIDE;
            bool near64 = false, close = false;
            if (act) {
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
                    const double* r = S.rec + t * R_STRIDE;
                    double dd = norm3(poi - ld3(r + R_C));
                    far = dd / r[R_LONG] > 5;
                }
                df32 nv[3] = {{f[F_NHI], f[F_NLO]}, {f[F_NHI + 1], f[F_NLO + 1]}, {f[F_NHI + 2], f[F_NLO + 2]}};
                if (far) {
                    // pntSrcPhi / pntDubPhi (CPanel/bodyPanel.cpp:392-395, panel.cpp:737-740) in double-float
                    df32 r2 = df_add(df_add(df_mul(d[0], d[0]), df_mul(d[1], d[1])), df_mul(d[2], d[2]));
                    df32 rinv = df_rsqrt(r2);
                    df32 src = df_mul(df_mul(df32{f[F_AHI], f[F_ALO]}, rinv), inv4pi);
                    df32 pn = df_add(df_add(df_mul(d[0], nv[0]), df_mul(d[1], nv[1])), df_mul(d[2], nv[2]));
                    df32 dub = df_mul(df_mul(pn, df_mul(rinv, rinv)), src);
                    A32[j * n + i] = dub.hi;
                    Alo[j * n + i] = dub.lo;
#pragma unroll
                    for (int c = 0; c < 3; c++) acc[c] = df_add(acc[c], df_mul(src, nv[c]));
                } else {
                    // beyond 3 longSide the exact formulas run in double-float (band_phi_df)
                    BandPhi bp{{0, 0}, {0, 0}, false};
                    if (r2f > __fmul_rn(9.f, __fmul_rn(L, L))) bp = band_phi_df(d[0], d[1], d[2], f);
                    if (bp.ok) {
                        A32[j * n + i] = bp.dub.hi;
                        Alo[j * n + i] = bp.dub.lo;
#pragma unroll
                        for (int c = 0; c < 3; c++) acc[c] = df_add(acc[c], df_mul(bp.src, nv[c]));
                    } else {
                        near64 = true;
                        close = r2f < __fmul_rn(L, L);
                    }
                }
            }
            // two classes, so that a chunk of the queue takes one branch of panel_phi_inf_pre:
            // within one longSide (edge sums) from the front, farther (one atan2) from the back
            const unsigned qc = __ballot_sync(0xffffffffu, close);
            const unsigned qf = __ballot_sync(0xffffffffu, near64 && !close);
            if (close) S.q[w][qn + __popc(qc & lt_mask)] = (unsigned short)((t << 5) | lane);
            if (near64 && !close) S.q[w][TJ * 32 - 1 - (qfar + __popc(qf & lt_mask))] = (unsigned short)((t << 5) | lane);
            qn += __popc(qc);
            qfar += __popc(qf);
        }
        __syncwarp();
        // the warp's FP64 pairs, one per lane: the front class, then the back class
        const int qtot = qn + qfar;
        for (int base = 0; base < qtot; base += 32) {
            const int e = base + lane;
            if (e < qtot) {
                const int ent = e < qn ? S.q[w][e] : S.q[w][TJ * 32 - 1 - (e - qn)];
                const int tt = ent >> 5, ln = ent & 31;
                const double* r = S.rec + tt * R_STRIDE;
                const dv3 pe = mk3(S.poi[w][ln][0], S.poi[w][ln][1], S.poi[w][ln][2]);
                double src = 0, dub = 0;
                panel_phi_inf_pre(r, S.e + tt * E_STRIDE, pe, src, dub);
                const int64_t ie = iw + ln, je_ = j0 + tt;
                float hi = (float)dub;
                A32[je_ * n + ie] = hi;
                Alo[je_ * n + ie] = (float)(dub - (double)hi);  // FP64 value = hi + lo to 2^-48
                S.res[w][lane][0] = src * r[R_N + 0];
                S.res[w][lane][1] = src * r[R_N + 1];
                S.res[w][lane][2] = src * r[R_N + 2];
                S.own[w][lane] = ln;
                nnear++;
            }
            __syncwarp();
            const int m = min(32, qtot - base);
            for (int k = 0; k < m; k++)
                if (S.own[w][k] == lane) {
                    acc64[0] += S.res[w][k][0];
                    acc64[1] += S.res[w][k][1];
                    acc64[2] += S.res[w][k][2];
                }
            __syncwarp();
        }
#pragma unroll
        for (int c = 0; c < 3; c++) acc64[c] += df_to_double(acc[c]);
    }
    if (act) {
        double* part = rbp + by * 3 * n;
        part[i] = acc64[0];
        part[n + i] = acc64[1];
        part[2 * n + i] = acc64[2];
    }
    if (near_count) {
        for (int o = 16; o > 0; o >>= 1) nnear += __shfl_down_sync(0xffffffffu, nnear, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(near_count, (unsigned long long)nnear);
    }
}

__global__ void __launch_bounds__(TI, 4) k_assemble_mixed(const double* __restrict__ rec,
                                                          const float* __restrict__ frec,
                                                          const double* __restrict__ erec, int64_t n, int64_t jchunk,
                                                          const int* __restrict__ order, float* __restrict__ A32,
                                                          float* __restrict__ Alo, double* __restrict__ rbp,
                                                          unsigned long long* __restrict__ near_count) {
    // block b works on row block order[2b] and source chunk order[2b+1] (the costly
    // near-diagonal blocks first, so that they do not form the tail)
    __shared__ MixedSmem S;
    mixed_block(S, rec, frec, erec, n, jchunk, order[2 * blockIdx.x], order[2 * blockIdx.x + 1], A32, Alo, rbp,
                near_count);
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

// Wake columns for the split (hi + lo) FP32 storage of the mixed path: the scatter of
// k_wake_columns for row i, one rounding to hi + lo per update, with the influences read
// from G[j * n + i] (k_wake_infl, all pairs in parallel) and added in wPanels order.
__device__ __forceinline__ void wake_row_split_table(const double* __restrict__ G, const int32_t* __restrict__ widx,
                                                     const double* __restrict__ wcoef, int64_t n, int64_t nw,
                                                     float* __restrict__ Ahi, float* __restrict__ Alo, int64_t i) {
    for (int64_t j = 0; j < nw; j++) {
        double infl = G[j * n + i];
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

// G[j * n + i] = dubPhiInf of wake panel j at body centroid i, all pairs in parallel
__global__ void k_wake_infl(const double* __restrict__ rec, const double* __restrict__ wrec, int64_t n,
                            double* __restrict__ G) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n) return;
    G[j * n + i] = dub_phi_inf(wrec + j * R_STRIDE, ld3(rec + i * R_STRIDE + R_C));
}

__global__ void k_wake_columns_split(const double* __restrict__ G, const int32_t* __restrict__ widx,
                                     const double* __restrict__ wcoef, int64_t n, int64_t nw,
                                     float* __restrict__ Ahi, float* __restrict__ Alo) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    wake_row_split_table(G, widx, wcoef, n, nw, Ahi, Alo, i);
}

__global__ void k_rb_reduce(const double* __restrict__ rbp, int64_t n, int64_t chunks, double* __restrict__ rb) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    double acc = 0;
    for (int64_t y = 0; y < chunks; y++) acc += rbp[y * 3 * n + t];
    rb[t] = acc;
}

// ---- grouped launch: the mixed assembly of many meshes at once.
// The work queue holds items (mesh, row block, first source chunk, chunk count); the
// chunk length of a mesh is the one its single-mesh launch uses (chunk_for), and every
// chunk still writes its own partial sums, so any queue order and any grouping of chunks
// into items gives the same bits as the single-mesh launch.  Persistent: each block
// takes the next item from a counter until the queue is empty.
__global__ void __launch_bounds__(TI, 4) k_assemble_mixed_grouped(const cpg::MixedMeshDesc* __restrict__ meshes,
                                                                  const int4* __restrict__ items, int nitems,
                                                                  int* __restrict__ next) {
    __shared__ MixedSmem S;
    __shared__ int s_item;
    for (;;) {
        __syncthreads();  // every thread has read the previous s_item
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) return;
        const int4 w = items[it];
        const cpg::MixedMeshDesc& d = meshes[w.x];
        for (int c = 0; c < w.w; c++)
            mixed_block(S, d.rec, d.frec, d.erec, d.n, d.jchunk, w.y, w.z + c, d.A32, d.Alo, d.rbp, d.near_count);
    }
}

// mesh of flattened row r (meshes sorted by row0)
__device__ __forceinline__ int mesh_of_row(const cpg::MixedMeshDesc* __restrict__ meshes, int m, int64_t r) {
    int lo = 0, hi = m - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (meshes[mid].row0 <= r) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// k_rb_reduce for every mesh of a group (same order of additions)
__global__ void k_rb_reduce_grouped(const cpg::MixedMeshDesc* __restrict__ meshes, int m, int64_t rows) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const cpg::MixedMeshDesc& d = meshes[mesh_of_row(meshes, m, r)];
    const int64_t i = r - d.row0, n = d.n, chunks = (n + d.jchunk - 1) / d.jchunk;
    for (int c = 0; c < 3; c++) {
        double acc = 0;
        for (int64_t y = 0; y < chunks; y++) acc += d.rbp[y * 3 * n + c * n + i];
        d.rb[c * n + i] = acc;
    }
}

// k_wake_infl for every mesh of a group into its partial-sum buffer (free after the reduction)
__global__ void k_wake_infl_grouped(const cpg::MixedMeshDesc* __restrict__ meshes, int m, int64_t rows) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (r >= rows) return;
    const cpg::MixedMeshDesc& d = meshes[mesh_of_row(meshes, m, r)];
    if (j >= d.nw) return;
    const int64_t i = r - d.row0;
    d.rbp[j * d.n + i] = dub_phi_inf(d.wrec + j * R_STRIDE, ld3(d.rec + i * R_STRIDE + R_C));
}

__global__ void k_wake_columns_grouped(const cpg::MixedMeshDesc* __restrict__ meshes, int m, int64_t rows) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const cpg::MixedMeshDesc& d = meshes[mesh_of_row(meshes, m, r)];
    if (d.nw > 0) wake_row_split_table(d.rbp, d.widx, d.wcoef, d.n, d.nw, d.A32, d.Alo, r - d.row0);
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
    // short source chunks (96 on the 19k wing): the FP64 near field concentrates in the few blocks
    // whose targets and sources are neighbours, and one such block of 128 x 1,152 pairs had run for
    // the whole kernel (27.8 of 28.5 ms, the SMs 52% occupied); 128 x 96 blocks spread it out
    int64_t bx = (n + TI - 1) / TI;
    int64_t want = 152 * 256;
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

cudaError_t launch_panels_velocity_rec(const double* rec, const double* sigma, const double* mu, int64_t nb,
                                       const double* wmu, int64_t nw, const double* pts, int64_t m, double* vel,
                                       cudaStream_t s) {
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

void mixed_block_order(int64_t n, const double* cent, int64_t cstride, const double* longside, int64_t lstride,
                       std::vector<int>& out) {
    const int64_t ch = chunk_for(n);
    const int64_t nbx = (n + TI - 1) / TI, nby = (n + ch - 1) / ch, ntj = (n + TJ - 1) / TJ;
    // bounding boxes of the row blocks' and the source tiles' centroids, the tiles' longest side
    std::vector<double> rb(6 * nbx), sb(6 * ntj), sl(ntj, 0.0);
    auto box = [&](int64_t i0, int64_t i1, double* b) {
        for (int d = 0; d < 3; d++) b[d] = 1e300, b[3 + d] = -1e300;
        for (int64_t i = i0; i < i1; i++)
            for (int d = 0; d < 3; d++) {
                const double v = cent[i * cstride + d];
                b[d] = std::min(b[d], v);
                b[3 + d] = std::max(b[3 + d], v);
            }
    };
    for (int64_t bx = 0; bx < nbx; bx++) box(bx * TI, std::min(n, (bx + 1) * TI), &rb[6 * bx]);
    for (int64_t t = 0; t < ntj; t++) {
        box(t * TJ, std::min(n, (t + 1) * TJ), &sb[6 * t]);
        for (int64_t j = t * TJ; j < std::min(n, (t + 1) * TJ); j++) sl[t] = std::max(sl[t], longside[j * lstride]);
    }
    // a block's cost: per source tile of its chunk, 64 when the boxes come within 3 long sides (FP64
    // near pairs, run at 1/64 of the FP32 rate), 8 within 5 (the double-float band), else 1
    std::vector<int32_t> cost_of(nbx * nby);
    host_parallel((size_t)(nbx * nby), [&](unsigned, size_t lo, size_t hi) {
        for (int64_t blk = (int64_t)lo; blk < (int64_t)hi; blk++) {
            const int64_t by = blk / nbx, bx = blk % nbx;
            int64_t cost = 0;
            const double* r = &rb[6 * bx];
            for (int64_t t = by * ch / TJ; t < std::min(ntj, (by + 1) * ch / TJ); t++) {
                const double* q = &sb[6 * t];
                double d2 = 0;
                for (int d = 0; d < 3; d++) {
                    const double gap = std::max(0.0, std::max(q[d] - r[3 + d], r[d] - q[3 + d]));
                    d2 += gap * gap;
                }
                cost += d2 < 9 * sl[t] * sl[t] ? 64 : d2 < 25 * sl[t] * sl[t] ? 8 : 1;
            }
            cost_of[blk] = (int32_t)cost;
        }
    });
    int32_t cmax = 0;
    for (int32_t c : cost_of) cmax = std::max(cmax, c);
    // costliest first, blocks of equal cost in index order (a counting sort over the small integer costs)
    std::vector<int64_t> start(cmax + 2, 0);
    for (int32_t c : cost_of) start[cmax - c + 1]++;
    for (int32_t c = 1; c <= cmax + 1; c++) start[c] += start[c - 1];
    std::vector<std::pair<int64_t, int64_t>> key(cost_of.size());
    for (int64_t blk = 0; blk < (int64_t)cost_of.size(); blk++) key[start[cmax - cost_of[blk]]++] = {-cost_of[blk], blk};
    out.resize(2 * key.size());
    for (size_t b = 0; b < key.size(); b++) {
        out[2 * b] = (int)(key[b].second % nbx);
        out[2 * b + 1] = (int)(key[b].second / nbx);
    }
}

cudaError_t launch_assemble_mixed(const double* rec, const float* frec, const double* erec, int64_t n,
                                  const double* wrec, const int32_t* widx, const double* wcoef, int64_t nw,
                                  const int* order, float* A32, float* Alo, double* rb, double* rb_part,
                                  unsigned long long* near_count, cudaStream_t s) {
    int64_t ch = chunk_for(n);
    const int64_t nbx = (n + TI - 1) / TI, nby = (n + ch - 1) / ch;
    {
        ProfScope ps(Prof::ASSEMBLE, s);
        k_assemble_mixed<<<(unsigned)(nbx * nby), TI, 0, s>>>(rec, frec, erec, n, ch, order, A32, Alo, rb_part,
                                                              near_count);
        k_rb_reduce<<<(unsigned)((3 * n + 255) / 256), 256, 0, s>>>(rb_part, n, nby, rb);
    }
    if (nw > 65535) return cudaErrorInvalidValue;  // one grid row per wake panel below
    if (nw > 0) {  // the chunk partial sums are reduced: their buffer holds the wake table
        ProfScope ps(Prof::WAKE_COLUMNS, s);
        k_wake_infl<<<dim3((unsigned)((n + 127) / 128), (unsigned)nw), 128, 0, s>>>(rec, wrec, n, rb_part);
        k_wake_columns_split<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(rb_part, widx, wcoef, n, nw, A32, Alo);
    }
    return cudaGetLastError();
}

int64_t mixed_rb_part_doubles(int64_t n, int64_t nw) {
    int64_t ch = chunk_for(n);
    return std::max(((n + ch - 1) / ch) * 3 * n, nw * n);
}

int64_t mixed_chunk(int64_t n) { return chunk_for(n); }

int64_t group_schedule(const int64_t* n, int m, int chunks_per_item, int near_band, std::vector<int>& items) {
    // an item's cost estimate: its pairs, weighted 16x when the row and source index
    // ranges lie within near_band chunk lengths of each other (near-diagonal items hold
    // most of the FP64 near field); near items keep one chunk each, the rest are grouped
    // chunks_per_item at a time, and the queue runs from the costliest item down
    struct It {
        double cost;
        int q, bx, by, g;
    };
    std::vector<It> v;
    if (chunks_per_item < 1) chunks_per_item = 1;
    for (int q = 0; q < m; q++) {
        const int64_t nn = n[q];
        if (nn <= 0) continue;
        const int64_t ch = chunk_for(nn), nbx = (nn + TI - 1) / TI, nby = (nn + ch - 1) / ch;
        const int64_t band = (int64_t)near_band * ch;
        for (int64_t bx = 0; bx < nbx; bx++) {
            const int64_t r0 = bx * TI, r1 = std::min(nn, r0 + TI);
            int64_t by = 0;
            while (by < nby) {
                const int64_t c0 = by * ch, c1 = std::min(nn, c0 + ch);
                const int64_t gap = c0 >= r1 ? c0 - r1 : (r0 >= c1 ? r0 - c1 : 0);
                const bool near_item = gap <= band;
                int g = 1;
                if (!near_item) {
                    while (g < chunks_per_item && by + g < nby) {  // extend while the next chunk is far too
                        const int64_t d0 = (by + g) * ch, d1 = std::min(nn, d0 + ch);
                        const int64_t gp = d0 >= r1 ? d0 - r1 : (r0 >= d1 ? r0 - d1 : 0);
                        if (gp <= band) break;
                        g++;
                    }
                }
                const int64_t e1 = std::min(nn, (by + g) * ch);
                const double pairs = (double)(r1 - r0) * (double)(e1 - c0);
                v.push_back({pairs * (near_item ? 16.0 : 1.0), q, (int)bx, (int)by, g});
                by += g;
            }
        }
    }
    std::stable_sort(v.begin(), v.end(), [](const It& a, const It& b) { return a.cost > b.cost; });
    items.resize(4 * v.size());
    for (size_t t = 0; t < v.size(); t++) {
        items[4 * t] = v[t].q;
        items[4 * t + 1] = v[t].bx;
        items[4 * t + 2] = v[t].by;
        items[4 * t + 3] = v[t].g;
    }
    return (int64_t)v.size();
}

cudaError_t launch_assemble_mixed_grouped_core(const MixedMeshDesc* meshes, const int* items, int nitems,
                                               int blocks, int* next, cudaStream_t s) {
    if (nitems <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(next, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    ProfScope ps(Prof::ASSEMBLE, s);
    k_assemble_mixed_grouped<<<(unsigned)blocks, TI, 0, s>>>(meshes, (const int4*)items, nitems, next);
    return cudaGetLastError();
}

cudaError_t launch_assemble_mixed_grouped_finish(const MixedMeshDesc* meshes, int m, int64_t rows, int64_t max_nw,
                                                 cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    const unsigned g = (unsigned)((rows + 127) / 128);
    {
        ProfScope ps(Prof::ASSEMBLE, s);
        k_rb_reduce_grouped<<<g, 128, 0, s>>>(meshes, m, rows);
    }
    if (max_nw > 0) {
        ProfScope ps(Prof::WAKE_COLUMNS, s);
        k_wake_infl_grouped<<<dim3(g, (unsigned)max_nw), 128, 0, s>>>(meshes, m, rows);
        k_wake_columns_grouped<<<g, 128, 0, s>>>(meshes, m, rows);
    }
    return cudaGetLastError();
}

int assemble_mixed_grouped_max_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_assemble_mixed_grouped, TI, 0) != cudaSuccess) return 1;
    return nb < 1 ? 1 : nb;
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
    // an error left by earlier work is not this call's: report it without clearing it
    if (cudaPeekAtLastError() != cudaSuccess) return CPG_E_CUDA;
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
