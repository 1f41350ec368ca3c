// Direct FP32 solve of the mixed path: blocked right-looking LU without pivoting,
// then iterative refinement against the double-float matrix (hi + lo).
//
// The panel matrix has a -0.5 self term on the diagonal; measured pivot growth of
// the unpivoted factorization is 1.00003 on the synthetic wings, and refinement
// with an exact-product residual reaches 1e-14 relative in three to four steps.
// Diagonal blocks and the two triangular block solves are hand-written kernels;
// the trailing update A22 -= L21 U12 is a plain GEMM issued through cuBLAS in
// FP32 (or its BF16x9 tensor-core emulation, which keeps FP32 accuracy).
#include <cublas_v2.h>

#include "tc_gemm.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "assemble.h"

namespace {

constexpr int NB = 128;   // panel width
constexpr int SB = 8 * NB; // blocks of the substitutions' combined inverses
constexpr int P = NB + 1; // padded smem pitch (no bank conflicts on row access)

constexpr int DT = 512;    // threads of the diagonal-block kernel
constexpr int BS = 32;     // inner block of the diagonal kernel
constexpr int TP = BS + 1; // pitch of its 32 x 32 scratch
constexpr int DIAG_SMEM = (3 * NB * P + 6 * BS * TP) * 4;

// In-place LU (unit lower L, upper U) of the b x b block at A + K*n + K, then the
// inverses of both triangles into Dinv (L11^{-1} then U11^{-1}, column-major, ld NB).
// A block smaller than NB is padded with the identity, which factors and inverts to
// itself without touching the real entries.  Every phase below is a set of
// independent items spread over the 512 threads; barriers separate the phases.
//
// LU: four 32-column steps (below); the inverses of the four 32 x 32 diagonal blocks come out
// of them, and the off-diagonal blocks of the inverses follow by distance d = 1..3 from the
// diagonal:
// Linv[I][J] = -Linv[I][I] sum_{K=J}^{I-1} L[I][K] Linv[K][J] and
// Uinv[I][J] = -Uinv[I][I] sum_{K=I+1}^{J} U[I][K] Uinv[K][J].
// The 32 x 32 diagonal block of one blocked-LU step in one warp's registers, lane i holding
// row i (template recursion keeps every register index static).
// fact_step: step k of the elimination; the multipliers replace the entries below the pivot.
template <int k>
__device__ __forceinline__ void fact_step(float (&r)[32], int lane, int* bad) {
    float u[32];
#pragma unroll
    for (int c = k; c < 32; c++) u[c] = __shfl_sync(0xffffffffu, r[c], k);
    float piv = u[k];
    if (piv == 0.f) {
        if (lane == 0) atomicExch(bad, 1);
        piv = 1.f;
    }
    const float rp = __frcp_rn(piv);  // the correctly rounded 1 / piv
    // rows at or above the pivot take a zero multiplier (no branch: r + (-0) u is r)
    const float l = lane > k ? r[k] * rp : 0.f;
    r[k] = lane > k ? l : r[k];
#pragma unroll
    for (int c = k + 1; c < 32; c++) r[c] = __fmaf_rn(-l, u[c], r[c]);
    if constexpr (k + 1 < 32) fact_step<k + 1>(r, lane, bad);
}
// X = L^{-1} (L unit lower, multipliers in r): row i of X is e_i - sum_{k<i} L[i][k] X[k],
// and row k is final once steps 0..k-1 have run
template <int k>
__device__ __forceinline__ void linv_step(const float (&r)[32], float (&x)[32], int lane) {
    const float m = lane > k ? r[k] : 0.f;
#pragma unroll
    for (int c = 0; c <= k; c++) x[c] = __fmaf_rn(-m, __shfl_sync(0xffffffffu, x[c], k), x[c]);
    if constexpr (k + 1 < 31) linv_step<k + 1>(r, x, lane);
}
// Y = U^{-1}: from the last row up, row k = (e_k - sum_{j>k} U[k][j] Y[j]) / U[k][k]
template <int k>
__device__ __forceinline__ void uinv_step(const float (&r)[32], float (&y)[32], int lane) {
    const float rd = __frcp_rn(__shfl_sync(0xffffffffu, r[k], k));  // 1 / U[k][k], once a step
    const float sc = lane == k ? rd : 1.f, m = lane < k ? r[k] : 0.f;
#pragma unroll
    for (int c = k; c < 32; c++) y[c] *= sc;
#pragma unroll
    for (int c = k; c < 32; c++) y[c] = __fmaf_rn(-m, __shfl_sync(0xffffffffu, y[c], k), y[c]);
    if constexpr (k > 0) uinv_step<k - 1>(r, y, lane);
}

__device__ __forceinline__ void lu_diag_body(float* sm, float* __restrict__ A, int64_t n, int64_t K, int b,
                                             float* __restrict__ Dinv, int* bad) {
    float* S = sm;                 // S[r*P + c]
    float* ZL = sm + NB * P;       // L^{-1}, row-major
    float* ZU = sm + 2 * NB * P;   // U^{-1}, row-major
    float* Tb = sm + 3 * NB * P;   // 6 scratch blocks, Tb[slot*BS*TP + r*TP + c]
    const int t = threadIdx.x;
    {  // all 32 loads of a thread in flight together
        float v[NB * NB / DT];
#pragma unroll
        for (int q = 0; q < NB * NB / DT; q++) {
            const int idx = t + q * DT, c = idx / NB, r = idx % NB;
            v[q] = (r < b && c < b) ? A[(K + c) * n + K + r] : (r == c ? 1.f : 0.f);
        }
#pragma unroll
        for (int q = 0; q < NB * NB / DT; q++) {
            const int idx = t + q * DT, c = idx / NB, r = idx % NB;
            S[r * P + c] = v[q];
            ZL[r * P + c] = r == c ? 1.f : 0.f;
            ZU[r * P + c] = r == c ? 1.f : 0.f;
        }
    }
    __syncthreads();
    // ---- blocked LU by 32-column steps o = 0, 32, 64, 96:
    //  1. warp 0 factors the 32 x 32 diagonal block D, then warps 0 and 1 invert its unit lower
    //     and upper triangles into the diagonal blocks of ZL and ZU, in registers (lane i: row i);
    //  2. the block column below becomes L = A U_D^{-1} and the block row to the right
    //     U = L_D^{-1} A (4 x 4 register tiles, written after a barrier: the products read
    //     the rows they replace);
    //  3. the trailing block loses L U.
    const int w = t >> 5, lane = t & 31;
    for (int o = 0; o < NB; o += BS) {
        if (w < 2) {  // warp 0 factors; then warp 0 inverts L_D and warp 1 U_D, side by side
            float r[32], x[32];
            if (w == 0) {
#pragma unroll
                for (int c = 0; c < 32; c++) r[c] = S[(o + lane) * P + o + c];
                fact_step<0>(r, lane, bad);
#pragma unroll
                for (int c = 0; c < 32; c++) S[(o + lane) * P + o + c] = r[c];
            }
            asm volatile("bar.sync 1, 64;" ::: "memory");
            if (w == 1) {
#pragma unroll
                for (int c = 0; c < 32; c++) r[c] = S[(o + lane) * P + o + c];
            }
#pragma unroll
            for (int c = 0; c < 32; c++) x[c] = c == lane ? 1.f : 0.f;
            if (w == 0) {
                linv_step<0>(r, x, lane);
#pragma unroll
                for (int c = 0; c < 32; c++) ZL[(o + lane) * P + o + c] = x[c];
            } else {
                uinv_step<31>(r, x, lane);
#pragma unroll
                for (int c = 0; c < 32; c++) ZU[(o + lane) * P + o + c] = x[c];
            }
        }
        __syncthreads();
        const int nr = NB - o - BS;  // rows below and columns to the right
        if (nr == 0) break;
        // 2. block column (2 nr tiles) and block row (2 nr tiles)
        float acc[4][4];
        int tr = 0, tc = 0;
        const bool col = t < 2 * nr, row = !col && t < 4 * nr;
        if (col) {
            tr = o + BS + 4 * (t >> 3);
            tc = o + 4 * (t & 7);
        } else if (row) {
            tr = o + 4 * ((t - 2 * nr) & 7);
            tc = o + BS + 4 * ((t - 2 * nr) >> 3);
        }
        if (col || row) {
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 4; x++) acc[i][x] = 0.f;
            const float* Pa = col ? S : ZL;
            const float* Pb = col ? ZU : S;
            for (int k = 0; k < BS; k++) {
                float a[4], bb[4];
#pragma unroll
                for (int i = 0; i < 4; i++) a[i] = Pa[(tr + i) * P + o + k];
#pragma unroll
                for (int x = 0; x < 4; x++) bb[x] = Pb[(o + k) * P + tc + x];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int x = 0; x < 4; x++) acc[i][x] = __fmaf_rn(a[i], bb[x], acc[i][x]);
            }
        }
        __syncthreads();
        if (col || row) {
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 4; x++) S[(tr + i) * P + tc + x] = acc[i][x];
        }
        __syncthreads();
        // 3. trailing update, (nr / 4)^2 tiles
        const int q4 = nr >> 2;
        for (int q = t; q < q4 * q4; q += DT) {
            const int rr = o + BS + 4 * (q % q4), cc = o + BS + 4 * (q / q4);
            float u[4][4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 4; x++) u[i][x] = 0.f;
            for (int k = 0; k < BS; k++) {
                float a[4], bb[4];
#pragma unroll
                for (int i = 0; i < 4; i++) a[i] = S[(rr + i) * P + o + k];
#pragma unroll
                for (int x = 0; x < 4; x++) bb[x] = S[(o + k) * P + cc + x];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int x = 0; x < 4; x++) u[i][x] = __fmaf_rn(a[i], bb[x], u[i][x]);
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 4; x++) S[(rr + i) * P + cc + x] -= u[i][x];
        }
        __syncthreads();
    }
    // ---- off-diagonal blocks, by distance from the diagonal
    for (int d = 1; d < NB / BS; d++) {
        const int nL = NB / BS - d;
        for (int w = t; w < 2 * nL * 64; w += DT) {
            const bool isU = w >= nL * 64;
            const int ww = w % (nL * 64), q = ww / 64, tile = ww % 64, tr = tile / 8, tc = tile % 8;
            const int I = isU ? q : d + q, J = isU ? q + d : q;
            const int kb = isU ? I + 1 : J, ke = isU ? J + 1 : I;
            const float* Z = isU ? ZU : ZL;
            float acc[4][4] = {};
            for (int Kb = kb; Kb < ke; Kb++)
                for (int k = 0; k < BS; k++) {
                    const int kk = BS * Kb + k;
                    float a[4], bb[4];
#pragma unroll
                    for (int i = 0; i < 4; i++) a[i] = S[(BS * I + 4 * tr + i) * P + kk];
#pragma unroll
                    for (int x = 0; x < 4; x++) bb[x] = Z[kk * P + BS * J + 4 * tc + x];
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int x = 0; x < 4; x++) acc[i][x] = __fmaf_rn(a[i], bb[x], acc[i][x]);
                }
            float* Tq = Tb + (isU ? 3 + q : q) * BS * TP;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 4; x++) Tq[(4 * tr + i) * TP + 4 * tc + x] = acc[i][x];
        }
        __syncthreads();
        for (int w = t; w < 2 * nL * 64; w += DT) {
            const bool isU = w >= nL * 64;
            const int ww = w % (nL * 64), q = ww / 64, tile = ww % 64, tr = tile / 8, tc = tile % 8;
            const int I = isU ? q : d + q, J = isU ? q + d : q;
            float* Z = isU ? ZU : ZL;
            const float* Tq = Tb + (isU ? 3 + q : q) * BS * TP;
            float acc[4][4] = {};
            for (int k = 0; k < BS; k++) {
                float a[4], bb[4];
#pragma unroll
                for (int i = 0; i < 4; i++) a[i] = Z[(BS * I + 4 * tr + i) * P + BS * I + k];
#pragma unroll
                for (int x = 0; x < 4; x++) bb[x] = Tq[k * TP + 4 * tc + x];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int x = 0; x < 4; x++) acc[i][x] = __fmaf_rn(a[i], bb[x], acc[i][x]);
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 4; x++) Z[(BS * I + 4 * tr + i) * P + BS * J + 4 * tc + x] = -acc[i][x];
        }
        __syncthreads();
    }
    float* Li = Dinv + (K / NB) * 2 * NB * NB;
    float* Ui = Li + NB * NB;
    for (int idx = t; idx < NB * NB; idx += DT) {
        int c = idx / NB, rr = idx % NB;
        Li[idx] = ZL[rr * P + c];
        Ui[idx] = ZU[rr * P + c];
        if (rr < b && c < b) A[(K + c) * n + K + rr] = S[rr * P + c];
    }
}

__global__ void __launch_bounds__(DT) k_lu_diag(float* __restrict__ A, int64_t n, int64_t K, int b,
                                                float* __restrict__ Dinv, int* bad) {
    extern __shared__ float sm[];
    lu_diag_body(sm, A, n, K, b, Dinv, bad);
}

// ---- lockstep factorization of many matrices (the batch path) ----
// Every kernel below takes work items of LB_ITEM ints: mesh, r0, r1, c0, c1, K, b, unused.
// The matrices are column-major with their own order n (LU[c*n + r]).
constexpr int LB_ITEM = 8;

// diagonal block K of every listed mesh, one block of DT threads each
__global__ void __launch_bounds__(DT) k_lu_diag_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                        const int* __restrict__ items) {
    extern __shared__ float sm[];
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    lu_diag_body(sm, d.LU, d.n, it[5], it[6], d.dinv, d.bad);
}

// L21 = A21 U_KK^{-1} in place for rows [r0, r1), columns K..K+b.  256 threads: thread t
// owns row t % 64 and the 32 columns 32 (t / 64) ..; U^{-1} staged 16 rows at a time.
constexpr int CS_R = 64;
__global__ void __launch_bounds__(256) k_col_solve_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                           const int* __restrict__ items) {
    __shared__ float X[CS_R][NB + 1];
    __shared__ __align__(16) float U[16][NB];
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    const int64_t n = d.n, r0 = it[1], r1 = it[2], K = it[5];
    const int b = it[6];
    float* A = d.LU;
    const float* Ui = d.dinv + (K / NB) * 2 * NB * NB + NB * NB;  // column-major, ld NB
    const int t = threadIdx.x, r = t % CS_R, cg = t / CS_R;
    for (int idx = t; idx < CS_R * NB; idx += 256) {
        const int c = idx / CS_R, rr = idx % CS_R;
        X[rr][c] = (r0 + rr < r1 && c < b) ? A[(K + c) * n + r0 + rr] : 0.f;
    }
    float acc[32];
#pragma unroll
    for (int j = 0; j < 32; j++) acc[j] = 0.f;
    for (int k0 = 0; k0 < b; k0 += 16) {
        __syncthreads();
        for (int idx = t; idx < 16 * NB; idx += 256) {
            const int kk = idx % 16, c = idx / 16;
            U[kk][c] = (k0 + kk < b && c < b) ? Ui[(k0 + kk) + (int64_t)c * NB] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; kk++) {
            const float a = X[r][k0 + kk];
            const float4* u4 = reinterpret_cast<const float4*>(&U[kk][32 * cg]);
#pragma unroll
            for (int j4 = 0; j4 < 8; j4++) {
                const float4 u = u4[j4];
                acc[4 * j4] = __fmaf_rn(a, u.x, acc[4 * j4]);
                acc[4 * j4 + 1] = __fmaf_rn(a, u.y, acc[4 * j4 + 1]);
                acc[4 * j4 + 2] = __fmaf_rn(a, u.z, acc[4 * j4 + 2]);
                acc[4 * j4 + 3] = __fmaf_rn(a, u.w, acc[4 * j4 + 3]);
            }
        }
    }
    if (r0 + r < r1) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int c = 32 * cg + j;
            if (c < b) A[(K + c) * n + r0 + r] = acc[j];
        }
    }
}

// U12 = L_KK^{-1} A12 in place for rows K..K+b, columns [c0, c1) (at most 64).  256
// threads: thread t owns row t % 128 and the 32 columns 32 (t / 128) ..; L^{-1} staged 16
// columns at a time.
constexpr int RS_C = 64;
__global__ void __launch_bounds__(256) k_row_solve_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                           const int* __restrict__ items) {
    __shared__ __align__(16) float X[NB][RS_C + 4];
    __shared__ float L[16][NB + 1];
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    const int64_t n = d.n, c0 = it[3], c1 = it[4], K = it[5];
    const int b = it[6];
    float* A = d.LU;
    const float* Li = d.dinv + (K / NB) * 2 * NB * NB;  // column-major, ld NB
    const int t = threadIdx.x, r = t % NB, cg = t / NB;
    for (int idx = t; idx < NB * RS_C; idx += 256) {
        const int c = idx / NB, k = idx % NB;
        X[k][c] = (k < b && c0 + c < c1) ? A[(c0 + c) * n + K + k] : 0.f;
    }
    float acc[32];
#pragma unroll
    for (int j = 0; j < 32; j++) acc[j] = 0.f;
    for (int k0 = 0; k0 < b; k0 += 16) {
        __syncthreads();
        for (int idx = t; idx < 16 * NB; idx += 256) {
            const int kk = idx / NB, rr = idx % NB;
            L[kk][rr] = (k0 + kk < b && rr < b) ? Li[rr + (int64_t)(k0 + kk) * NB] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; kk++) {
            const float a = L[kk][r];
            const float4* x4 = reinterpret_cast<const float4*>(&X[k0 + kk][32 * cg]);
#pragma unroll
            for (int j4 = 0; j4 < 8; j4++) {
                const float4 x = x4[j4];
                acc[4 * j4] = __fmaf_rn(a, x.x, acc[4 * j4]);
                acc[4 * j4 + 1] = __fmaf_rn(a, x.y, acc[4 * j4 + 1]);
                acc[4 * j4 + 2] = __fmaf_rn(a, x.z, acc[4 * j4 + 2]);
                acc[4 * j4 + 3] = __fmaf_rn(a, x.w, acc[4 * j4 + 3]);
            }
        }
    }
    if (r < b) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int64_t c = c0 + 32 * cg + j;
            if (c < c1) A[c * n + K + r] = acc[j];
        }
    }
}

// C -= L(:, K..K+b) U(K..K+b, :) on the tile rows [r0, min(r0 + 128, r1)) x columns
// [c0, min(c0 + 64, c1)).  128 threads, each an 8 x 8 block of C in registers (rows
// 8 (t % 16) .., columns 8 (t / 16) ..); L and U staged GS_K columns / rows at a time and
// read as float4 (two loads each per k for 64 FMAs).
constexpr int GS_R = 128, GS_C = 64, GS_K = 32;
__global__ void __launch_bounds__(128) k_gemm_sub_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                          const int* __restrict__ items) {
    __shared__ __align__(16) float Ls[GS_K][GS_R];
    __shared__ __align__(16) float Us[GS_K][GS_C];
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    const int64_t n = d.n, r0 = it[1], r1 = it[2], c0 = it[3], c1 = it[4], K = it[5];
    const int b = it[6];
    float* A = d.LU;
    const int t = threadIdx.x, tr = t % 16, tc = t / 16;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < b; k0 += GS_K) {
        __syncthreads();
        for (int idx = t; idx < GS_K * GS_R; idx += 128) {
            const int kk = idx / GS_R, rr = idx % GS_R;
            Ls[kk][rr] = (k0 + kk < b && r0 + rr < r1) ? A[(K + k0 + kk) * n + r0 + rr] : 0.f;
        }
        for (int idx = t; idx < GS_K * GS_C; idx += 128) {
            const int kk = idx % GS_K, c = idx / GS_K;
            Us[kk][c] = (k0 + kk < b && c0 + c < c1) ? A[(c0 + c) * n + K + k0 + kk] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < GS_K; kk++) {
            const float4 a0 = *reinterpret_cast<const float4*>(&Ls[kk][8 * tr]);
            const float4 a1 = *reinterpret_cast<const float4*>(&Ls[kk][8 * tr + 4]);
            const float4 u0 = *reinterpret_cast<const float4*>(&Us[kk][8 * tc]);
            const float4 u1 = *reinterpret_cast<const float4*>(&Us[kk][8 * tc + 4]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float u[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(a[i], u[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int64_t c = c0 + 8 * tc + j;
        if (c >= c1) continue;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int64_t r = r0 + 8 * tr + i;
            if (r < r1) {
                float* p = A + c * n + r;
                *p = *p - acc[i][j];
            }
        }
    }
}

// ---- lockstep block substitutions (the batch path's refined solves) ----
// X and Y are n x k (ld n); items of LB_ITEM ints: mesh, r0, r1, -, -, K, b, -.
struct SubstMesh {
    const float* LU;
    const float* dinv;
    float* X;
    float* Y;
    int64_t n;
    int k;
    int pad;
};
// KC right-hand sides per pass over the block (8, 16 or 32: the smallest that holds k,
// or 32 in passes); the staged block Z is read as float4.

// forward (dir 0): Y_K = L_KK^{-1} X_K; backward (dir 1): X_K = U_KK^{-1} Y_K.  One block of
// NB threads per system, thread r computing row r.
template <int KC>
__global__ void __launch_bounds__(NB) k_subst_diag_batched(const SubstMesh* __restrict__ ms,
                                                           const int* __restrict__ items,
                                                           const int* __restrict__ active, int dir) {
    __shared__ __align__(16) float Z[NB][KC];
    const int* it = items + LB_ITEM * blockIdx.x;
    if (!active[it[0]]) return;
    const SubstMesh d = ms[it[0]];
    const int64_t n = d.n, K = it[5];
    const int b = it[6], r = threadIdx.x;
    const float* Mi = d.dinv + (K / NB) * 2 * NB * NB + (dir ? NB * NB : 0);  // column-major, ld NB
    const float* src = dir ? d.Y : d.X;
    float* dst = dir ? d.X : d.Y;
    for (int c0 = 0; c0 < d.k; c0 += KC) {
        const int kc = min(KC, d.k - c0);
        __syncthreads();
        for (int idx = r; idx < NB * KC; idx += NB) {
            const int c = idx / NB, j = idx % NB;
            Z[j][c] = (j < b && c < kc) ? src[(int64_t)(c0 + c) * n + K + j] : 0.f;
        }
        __syncthreads();
        float acc[KC];
#pragma unroll
        for (int c = 0; c < KC; c++) acc[c] = 0.f;
#pragma unroll 4
        for (int j = 0; j < b; j++) {
            const float a = Mi[r + j * NB];
            const float4* z4 = reinterpret_cast<const float4*>(&Z[j][0]);
#pragma unroll
            for (int c4 = 0; c4 < KC / 4; c4++) {
                const float4 z = z4[c4];
                acc[4 * c4] = __fmaf_rn(a, z.x, acc[4 * c4]);
                acc[4 * c4 + 1] = __fmaf_rn(a, z.y, acc[4 * c4 + 1]);
                acc[4 * c4 + 2] = __fmaf_rn(a, z.z, acc[4 * c4 + 2]);
                acc[4 * c4 + 3] = __fmaf_rn(a, z.w, acc[4 * c4 + 3]);
            }
        }
        if (r < b) {
#pragma unroll
            for (int c = 0; c < KC; c++)
                if (c < kc) dst[(int64_t)(c0 + c) * n + K + r] = acc[c];
        }
    }
}

// forward (dir 0): X_i -= L(i, K..K+b) Y_K for the rows i in [r0, min(r0 + NB, r1)) below the
// block; backward (dir 1): Y_i -= U(i, K..K+b) X_K for rows above it.  Thread r owns row r0 + r.
template <int KC>
__global__ void __launch_bounds__(NB) k_subst_update_batched(const SubstMesh* __restrict__ ms,
                                                             const int* __restrict__ items,
                                                             const int* __restrict__ active, int dir) {
    __shared__ __align__(16) float Z[NB][KC];
    const int* it = items + LB_ITEM * blockIdx.x;
    if (!active[it[0]]) return;
    const SubstMesh d = ms[it[0]];
    const int64_t n = d.n, r0 = it[1], r1 = it[2], K = it[5];
    const int b = it[6], r = threadIdx.x;
    const int64_t i = r0 + r;
    const float* src = dir ? d.X : d.Y;
    float* dst = dir ? d.Y : d.X;
    for (int c0 = 0; c0 < d.k; c0 += KC) {
        const int kc = min(KC, d.k - c0);
        __syncthreads();
        for (int idx = r; idx < NB * KC; idx += NB) {
            const int c = idx / NB, j = idx % NB;
            Z[j][c] = (j < b && c < kc) ? src[(int64_t)(c0 + c) * n + K + j] : 0.f;
        }
        __syncthreads();
        if (i < r1) {
            float acc[KC];
#pragma unroll
            for (int c = 0; c < KC; c++) acc[c] = 0.f;
            const float* Lp = d.LU + K * n + i;
#pragma unroll 4
            for (int j = 0; j < b; j++) {
                const float a = Lp[(int64_t)j * n];
                const float4* z4 = reinterpret_cast<const float4*>(&Z[j][0]);
#pragma unroll
                for (int c4 = 0; c4 < KC / 4; c4++) {
                    const float4 z = z4[c4];
                    acc[4 * c4] = __fmaf_rn(a, z.x, acc[4 * c4]);
                    acc[4 * c4 + 1] = __fmaf_rn(a, z.y, acc[4 * c4 + 1]);
                    acc[4 * c4 + 2] = __fmaf_rn(a, z.z, acc[4 * c4 + 2]);
                    acc[4 * c4 + 3] = __fmaf_rn(a, z.w, acc[4 * c4 + 3]);
                }
            }
#pragma unroll
            for (int c = 0; c < KC; c++)
                if (c < kc) {
                    float* p = dst + (int64_t)(c0 + c) * n + i;
                    *p = *p - acc[c];
                }
        }
    }
}

template <int KC>
void subst_launch(int kind, unsigned g, const SubstMesh* d, const int* it, const int* act, int dir, cudaStream_t s) {
    if (kind == 0)
        k_subst_diag_batched<KC><<<g, NB, 0, s>>>(d, it, act, dir);
    else
        k_subst_update_batched<KC><<<g, NB, 0, s>>>(d, it, act, dir);
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, int64_t m) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m) b[t] = (float)a[t];
}
__global__ void k_addf(double* __restrict__ x, const float* __restrict__ d, int64_t m) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m) x[t] += (double)d[t];
}

inline unsigned nb256(int64_t m) { return (unsigned)((m + 255) / 256); }

// once per device, also when several host threads start at the same time
void set_attrs() {
    static std::once_flag once[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::call_once(once[dev & 63],
                   [] {
                       cudaFuncSetAttribute(k_lu_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM);
                       cudaFuncSetAttribute(k_lu_diag_batched, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            DIAG_SMEM);
                   });
}

// GEMM arithmetic of the factorization: the rank-OB updates in the BF16x9 emulation of FP32
// on the tensor cores; the panel-sized GEMMs (inner dimension 128) in FP32 on the CUDA cores
// (one kernel each, where the emulation launches three)
cublasComputeType_t lu_compute() { return CUBLAS_COMPUTE_32F_EMULATED_16BFX9; }
cublasComputeType_t lu_compute_small() { return CUBLAS_COMPUTE_32F; }

}  // namespace

namespace cpg {

namespace {

// The blocked loops below issue ~4 launches (plus cuBLAS calls) per 128 columns;
// replayed from a CUDA graph they run back to back on the device instead of
// waiting on the host.  cuBLAS gets a fixed workspace so that it never allocates
// while a stream is being captured.
constexpr size_t kBlasWorkspace = size_t(256) << 20;

cudaError_t prepare_blas(cublasHandle_t h, LuGraphs* G, cudaStream_t s) {
    if (!G->workspace) {
        cudaError_t e = cudaMalloc(&G->workspace, kBlasWorkspace);
        if (e != cudaSuccess) return e;
    }
    if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
    if (cublasSetWorkspace(h, G->workspace, kBlasWorkspace) != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
    return cudaSuccess;
}

// L21 = A21 U_KK^{-1} for all rows below block K, as a GEMM through W (copied back).
cudaError_t column_solve(cublasHandle_t h, float* LU, const float* Dinv, float* W, int64_t n, int64_t K,
                         cudaStream_t s) {
    const float one = 1.f, zero = 0.f;
    int b = (int)std::min<int64_t>(NB, n - K);
    const float* Ui = Dinv + (K / NB) * 2 * NB * NB + NB * NB;
    int64_t rest = n - K - b;
    if (rest <= 0) return cudaSuccess;
    if (cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)rest, b, b, &one, LU + K * n + K + b, CUDA_R_32F, (int)n, Ui,
                     CUDA_R_32F, NB, &zero, W, CUDA_R_32F, (int)rest, lu_compute_small(), CUBLAS_GEMM_DEFAULT) !=
        CUBLAS_STATUS_SUCCESS)
        return cudaErrorUnknown;
    return cudaMemcpy2DAsync(LU + K * n + K + b, n * sizeof(float), W, rest * sizeof(float), rest * sizeof(float), b,
                             cudaMemcpyDeviceToDevice, s);
}

// U(K..K+b, c0..c0+nc) = L_KK^{-1} A(K..K+b, c0..c0+nc), as a GEMM through W (copied back).
cudaError_t row_solve(cublasHandle_t h, float* LU, const float* Dinv, float* W, int64_t n, int64_t K, int64_t c0,
                      int64_t nc, cudaStream_t s) {
    if (nc <= 0) return cudaSuccess;
    const float one = 1.f, zero = 0.f;
    int b = (int)std::min<int64_t>(NB, n - K);
    const float* Li = Dinv + (K / NB) * 2 * NB * NB;
    if (cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, b, (int)nc, b, &one, Li, CUDA_R_32F, NB, LU + c0 * n + K,
                     CUDA_R_32F, (int)n, &zero, W, CUDA_R_32F, b, lu_compute_small(), CUBLAS_GEMM_DEFAULT) !=
        CUBLAS_STATUS_SUCCESS)
        return cudaErrorUnknown;
    return cudaMemcpy2DAsync(LU + c0 * n + K, n * sizeof(float), W, b * sizeof(float), b * sizeof(float), nc,
                             cudaMemcpyDeviceToDevice, s);
}

// A22 block [r0, r0+m) x [c0, c0+nc) -= L(r0.., K..K+b) U(K..K+b, c0..)
cudaError_t trailing(cublasHandle_t h, float* LU, int64_t n, int64_t K, int b, int64_t r0, int64_t m, int64_t c0,
                     int64_t nc) {
    if (m <= 0 || nc <= 0) return cudaSuccess;
    const float one = 1.f, mone = -1.f;
    cublasStatus_t st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)m, (int)nc, b, &mone, LU + K * n + r0,
                                     CUDA_R_32F, (int)n, LU + c0 * n + K, CUDA_R_32F, (int)n, &one, LU + c0 * n + r0,
                                     CUDA_R_32F, (int)n, b <= NB ? lu_compute_small() : lu_compute(),
                                     CUBLAS_GEMM_DEFAULT);
    return st == CUBLAS_STATUS_SUCCESS ? cudaSuccess : cudaErrorUnknown;
}

// Two-level right-looking blocked LU.  Inner blocks of NB columns are factored within an
// outer panel of OB columns: per inner block the diagonal kernel, L21 for all rows
// below, U12 and the trailing update only inside the outer panel (an (n - K) x < OB
// update that stays in L2).  After the panel, its U rows right of it come from a
// blocked forward substitution and the rest of the matrix from one rank-OB update, so the
// large trailing matrix is read and written once per OB columns instead of once per NB.
// Look-ahead: the rank-OB update is split into the next panel's columns and the rest;
// the next panel is factored on a high-priority stream while the rest of the update
// runs.  (Measured: about 1 ms of 56 on the 19k wing.  cuBLAS's large GEMM holds every
// SM until it ends, and keeping 8-32 SMs out of it for the panel measured 0.6-5 ms
// slower.)
// outer panel width: OB_BLOCKS inner blocks.  The lockstep factorization of many matrices
// uses OB_BLOCKS_BATCHED: its rank-128 panel updates run in FP32 on the CUDA cores and its
// rank-OB updates on the tensor cores, and on the 64-wing batch 512 columns measured 220 ms
// against 269 ms for 1,024 (256: 224 ms; 2,048: 379 ms).
constexpr int OB_BLOCKS = 8;
constexpr int OB_BLOCKS_BATCHED = 4;
// SMs the rank-OB update of the columns past the next panel leaves to that panel's
// factorization on its own stream (19k wing: LU 38.6 ms with 0, 37.5 with 8, 37.4 with 16,
// 36.8 with 32)
constexpr int kPanelSms = 32;
int64_t outer_width(int blocks = OB_BLOCKS) { return (int64_t)NB * blocks; }

struct Streams {  // where the next cuBLAS calls go
    cublasHandle_t h;
    cudaStream_t main, panel;
    void *ws_main, *ws_panel;
    cudaError_t use(bool on_panel) const {
        if (cublasSetStream(h, on_panel ? panel : main) != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
        if (cublasSetWorkspace(h, on_panel ? ws_panel : ws_main, kBlasWorkspace) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        return cudaSuccess;
    }
};

// factorization of the outer panel [KO, KE) (on st.panel)
cudaError_t factor_panel(const Streams& st, float* LU, float* Dinv, float* W, int64_t n, int* bad, int64_t KO,
                         int64_t KE) {
    cudaError_t e;
    if ((e = st.use(true)) != cudaSuccess) return e;
    for (int64_t K = KO; K < KE; K += NB) {
        const int b = (int)std::min<int64_t>(NB, n - K);
        k_lu_diag<<<1, DT, DIAG_SMEM, st.panel>>>(LU, n, K, b, Dinv, bad);
        if ((e = column_solve(st.h, LU, Dinv, W, n, K, st.panel)) != cudaSuccess) return e;
        const int64_t K1 = K + b;
        if ((e = row_solve(st.h, LU, Dinv, W, n, K, K1, KE - K1, st.panel)) != cudaSuccess) return e;
        if ((e = trailing(st.h, LU, n, K, b, K1, n - K1, K1, KE - K1)) != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

cudaError_t factor_body(const Streams& st, LuGraphs* G, float* LU, float* Dinv, float* W, int64_t n, int* bad) {
    cudaError_t e;
    const int64_t OB = outer_width();
    // first panel
    if ((e = cudaEventRecord(G->ev_update, st.main)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st.panel, G->ev_update, 0)) != cudaSuccess) return e;
    if ((e = factor_panel(st, LU, Dinv, W, n, bad, 0, std::min<int64_t>(OB, n))) != cudaSuccess) return e;
    for (int64_t KO = 0; KO < n; KO += OB) {
        const int64_t KE = std::min<int64_t>(KO + OB, n);
        // this panel done (the main stream has finished the rest of the previous update)
        if ((e = cudaEventRecord(G->ev_panel, st.panel)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(st.main, G->ev_panel, 0)) != cudaSuccess) return e;
        if (KE >= n) break;
        if ((e = st.use(false)) != cudaSuccess) return e;
        for (int64_t K = KO; K < KE; K += NB) {  // U(KO..KE, KE..n): forward substitution by blocks
            const int b = (int)std::min<int64_t>(NB, n - K);
            if ((e = row_solve(st.h, LU, Dinv, W, n, K, KE, n - KE, st.main)) != cudaSuccess) return e;
            if ((e = trailing(st.h, LU, n, K, b, K + b, KE - K - b, KE, n - KE)) != cudaSuccess) return e;
        }
        const int64_t KE2 = std::min<int64_t>(KE + OB, n);
        // rank-OB update A22 -= L21 U12 on the tensor cores: both operands split once, then the
        // next panel's columns, then the next panel on its stream beside the update of the
        // remaining columns
        TcOperand tA, tB;
        const int64_t rows = n - KE;
        tc_operand_bind(tA, G->tc_mem, rows, OB);
        tc_operand_bind(tB, (char*)G->tc_mem + tc_operand_bytes(rows, OB), rows, OB);
        if ((e = tc_split(LU + KO * n + KE, 1, n, rows, KE - KO, tA, bad, st.main)) != cudaSuccess) return e;
        if ((e = tc_split(LU + KE * n + KO, n, 1, rows, KE - KO, tB, bad, st.main)) != cudaSuccess) return e;
        const int sms = tc_num_sms();
        if ((e = tc_gemm(tA, rows, tB, KE2 - KE, -1.f, 1.f, LU + KE * n + KE, n, sms, bad, st.main)) != cudaSuccess)
            return e;
        if ((e = cudaEventRecord(G->ev_update, st.main)) != cudaSuccess) return e;
        if ((e = tc_gemm(tA, rows, tc_rows(tB, KE2 - KE), n - KE2, -1.f, 1.f, LU + KE2 * n + KE, n,
                         sms - kPanelSms, bad, st.main)) != cudaSuccess)
            return e;
        if ((e = cudaStreamWaitEvent(st.panel, G->ev_update, 0)) != cudaSuccess) return e;
        if ((e = factor_panel(st, LU, Dinv, W, n, bad, KE, KE2)) != cudaSuccess) return e;
    }
    if ((e = st.use(false)) != cudaSuccess) return e;
    return cudaGetLastError();
}

// Blocked forward and backward substitution with the diagonal-block inverses, two
// GEMMs per block and direction and no copies: forward, Y_K = inv(L_KK) X_K and
// X_below -= L_below,K Y_K; backward, X_K = inv(U_KK) Y_K and Y_above -= U_above,K X_K.
// X (n x k, ld n) ends with the solution; Y is an n x k scratch array.  The first nsup
// SB-column blocks use their combined inverses (Dinv4), so a pass takes an eighth of the
// dependent steps there; the rest of the matrix goes by 128-column blocks.
cudaError_t solve_body(cublasHandle_t h, const float* LU, const float* Dinv, const float* Dinv4, int64_t nsup,
                       int64_t n, float* X, float* Y, int k) {
    const float one = 1.f, mone = -1.f, zero = 0.f;
    const int64_t nblk = (n + NB - 1) / NB, blk0 = nsup * (SB / NB);
    for (int64_t sb = 0; sb < nsup; sb++) {
        const int64_t K = sb * SB;
        const float* Li = Dinv4 + sb * 2 * SB * SB;
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, SB, k, SB, &one, Li, SB, X + K, (int)n, &zero, Y + K, (int)n) !=
            CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        const int64_t rest = n - K - SB;
        if (rest > 0 && cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)rest, k, SB, &mone, LU + K * n + K + SB, (int)n,
                                    Y + K, (int)n, &one, X + K + SB, (int)n) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
    }
    for (int64_t blk = blk0; blk < nblk; blk++) {
        int64_t K = blk * NB;
        int b = (int)std::min<int64_t>(NB, n - K);
        const float* Li = Dinv + blk * 2 * NB * NB;
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, b, k, b, &one, Li, NB, X + K, (int)n, &zero, Y + K, (int)n) !=
            CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        int64_t rest = n - K - b;
        if (rest > 0 && cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)rest, k, b, &mone, LU + K * n + K + b, (int)n,
                                    Y + K, (int)n, &one, X + K + b, (int)n) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
    }
    for (int64_t blk = nblk - 1; blk >= blk0; blk--) {
        int64_t K = blk * NB;
        int b = (int)std::min<int64_t>(NB, n - K);
        const float* Ui = Dinv + blk * 2 * NB * NB + NB * NB;
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, b, k, b, &one, Ui, NB, Y + K, (int)n, &zero, X + K, (int)n) !=
            CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        if (K > 0 && cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)K, k, b, &mone, LU + K * n, (int)n, X + K, (int)n,
                                 &one, Y, (int)n) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
    }
    for (int64_t sb = nsup - 1; sb >= 0; sb--) {
        const int64_t K = sb * SB;
        const float* Ui = Dinv4 + sb * 2 * SB * SB + SB * SB;
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, SB, k, SB, &one, Ui, SB, Y + K, (int)n, &zero, X + K, (int)n) !=
            CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        if (K > 0 && cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)K, k, SB, &mone, LU + K * n, (int)n, X + K, (int)n,
                                 &one, Y, (int)n) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
    }
    return cudaGetLastError();
}

// Inverses of the full SB-column diagonal blocks from the 128-column ones inside each, by
// block-triangular doublings (128 -> 256 -> 512 -> 1024):
//   [[A, 0], [C, B]]^{-1} = [[A^{-1}, 0], [-B^{-1} C A^{-1}, B^{-1}]]   (L, unit lower)
//   [[A, C], [0, B]]^{-1} = [[A^{-1}, -A^{-1} C B^{-1}], [0, B^{-1}]]   (U)
// Every step is one strided-batched FP32 GEMM over all the 512-column blocks (their
// diagonal blocks of LU, their inverses and their scratch all lie at fixed strides).
// Layout: Dinv4 + s * 2 * SB^2 holds L^{-1} then U^{-1} of block s, column-major, ld SB.
__global__ void k_super_init(const float* __restrict__ Dinv, float* __restrict__ Dinv4, int64_t nsup) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsup * 2 * SB * SB) return;
    const int64_t s = t / (2 * SB * SB);
    const int64_t w = t % (2 * SB * SB);
    const int u = (int)(w / (SB * SB));  // 0: L, 1: U
    const int64_t e = w % (SB * SB);
    const int r = (int)(e % SB), c = (int)(e / SB);
    float v = 0.f;
    if (r / NB == c / NB) {
        const int64_t blk = s * (SB / NB) + r / NB;
        v = Dinv[blk * 2 * NB * NB + u * NB * NB + (r % NB) + (int64_t)(c % NB) * NB];
    }
    Dinv4[t] = v;
}

cudaError_t build_super_inverses(cublasHandle_t h, LuGraphs* G, const float* LU, int64_t n, cudaStream_t s) {
    const int64_t nsup = n / SB;
    G->super_n = 0;
    if (nsup == 0) return cudaSuccess;
    cudaError_t e;
    if (!G->dinv4 || G->super_cap != nsup) {  // same buffers for every factorization of this size,
        if (G->solve) cudaGraphExecDestroy(G->solve);  // so a captured substitution stays valid
        G->solve = nullptr;
        if (G->dinv4) cudaFree(G->dinv4);
        if (G->super_tmp) cudaFree(G->super_tmp);
        G->dinv4 = G->super_tmp = nullptr;
        G->super_cap = 0;
        if ((e = cudaMalloc(&G->dinv4, sizeof(float) * nsup * 2 * SB * SB)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&G->super_tmp, sizeof(float) * nsup * (SB / 2) * (SB / 2))) != cudaSuccess) return e;
        G->super_cap = nsup;
    }
    const int64_t tot = nsup * 2 * SB * SB;
    k_super_init<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(G->dinv, G->dinv4, nsup);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const float one = 1.f, mone = -1.f, zero = 0.f;
    const int ni = (int)n, bc = (int)nsup;
    const long long sLU = (long long)SB * (n + 1), sD = 2LL * SB * SB, sT = (long long)(SB / 2) * (SB / 2);
    float* T = G->super_tmp;
    auto gemm = [&](int m, int nn, int kk, float alpha, const float* A, int lda, long long sA, const float* B, int ldb,
                    long long sB, float* C, int ldc) -> cudaError_t {
        return cublasSgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, m, nn, kk, &alpha, A, lda, sA, B, ldb, sB, &zero,
                                         C, ldc, C == T ? sT : sD, bc) == CUBLAS_STATUS_SUCCESS
                   ? cudaSuccess
                   : cudaErrorUnknown;
    };
    for (int w = NB; w < SB; w *= 2) {  // size of the two blocks combined at this level
        for (int p = 0; p < SB / (2 * w); p++) {
            const int o = 2 * w * p;  // offset of the pair inside the 512-column block
            float* Linv = G->dinv4;
            float* Uinv = G->dinv4 + SB * SB;
            // L: T = C A^{-1}, then -B^{-1} T into the lower-left block
            if ((e = gemm(w, w, w, one, LU + (o + w) + (int64_t)o * n, ni, sLU, Linv + o + (int64_t)o * SB, SB, sD, T,
                          w)) != cudaSuccess)
                return e;
            if ((e = gemm(w, w, w, mone, Linv + (o + w) + (int64_t)(o + w) * SB, SB, sD, T, w, sT,
                          Linv + (o + w) + (int64_t)o * SB, SB)) != cudaSuccess)
                return e;
            // U: T = C B^{-1}, then -A^{-1} T into the upper-right block
            if ((e = gemm(w, w, w, one, LU + o + (int64_t)(o + w) * n, ni, sLU, Uinv + (o + w) + (int64_t)(o + w) * SB,
                          SB, sD, T, w)) != cudaSuccess)
                return e;
            if ((e = gemm(w, w, w, mone, Uinv + o + (int64_t)o * SB, SB, sD, T, w, sT, Uinv + o + (int64_t)(o + w) * SB,
                          SB)) != cudaSuccess)
                return e;
        }
    }
    G->super_n = n;
    return cudaSuccess;
}

// Capture body() on s into a graph (no profiler events inside the capture).
template <class F>
cudaError_t capture(cudaStream_t s, cudaGraphExec_t* out, F body, unsigned long long flags = 0) {
    Prof* saved = g_prof;
    g_prof = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        g_prof = saved;
        return e;
    }
    cudaError_t eb = body();
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    g_prof = saved;
    if (eb != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return eb;
    }
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiateWithFlags(out, graph, flags);
    cudaGraphDestroy(graph);
    return e;
}

}  // namespace

void LuGraphs::release() {
    if (solve) cudaGraphExecDestroy(solve);
    if (workspace && !shared_ws) cudaFree(workspace);
    if (workspace2 && !shared_ws) cudaFree(workspace2);
    workspace = nullptr;
    shared_ws = false;
    if (panel_stream) cudaStreamDestroy(panel_stream);
    if (ev_update) cudaEventDestroy(ev_update);
    if (ev_panel) cudaEventDestroy(ev_panel);
    workspace2 = nullptr;
    panel_stream = nullptr;
    ev_update = ev_panel = nullptr;
    if (dinv) cudaFree(dinv);
    if (panel) cudaFree(panel);
    if (tmp) cudaFree(tmp);
    if (dinv4) cudaFree(dinv4);
    if (super_tmp) cudaFree(super_tmp);
    if (tc_mem) cudaFree(tc_mem);
    tc_mem = nullptr;
    tc_bytes = 0;
    dinv4 = super_tmp = nullptr;
    super_n = super_cap = 0;
    solve = nullptr;
    workspace = nullptr;
    dinv = panel = tmp = nullptr;
    tmp_floats = 0;
    solve_X = nullptr;
    solve_k = 0;
    factor_n = 0;
}

// Launched directly (not from a graph): a geometry is factored once, and its ~3,000
// launches are each longer than their host-side cost, so a captured graph would only
// add the capture and instantiation to every new geometry.
cudaError_t lu_factor_fp32(void* blas, LuGraphs* G, float* LU, int64_t n, int* bad, cudaStream_t s) {
    set_attrs();
    cublasHandle_t h = (cublasHandle_t)blas;
    cudaError_t e = prepare_blas(h, G, s);
    if (e != cudaSuccess) return e;
    if (G->factor_n != n || !G->dinv) {
        if (G->solve) cudaGraphExecDestroy(G->solve);  // it holds the old Dinv
        G->solve = nullptr;
        if (G->dinv) cudaFree(G->dinv);
        if (G->panel) cudaFree(G->panel);
        G->dinv = G->panel = nullptr;
        size_t nb = (size_t)((n + NB - 1) / NB);
        if ((e = cudaMalloc(&G->dinv, sizeof(float) * nb * 2 * NB * NB)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&G->panel, sizeof(float) * (size_t)n * NB)) != cudaSuccess) return e;
        G->factor_n = n;
    }
    const size_t tcb = 2 * tc_operand_bytes(n, outer_width());
    if (G->tc_bytes < tcb) {
        if (G->tc_mem) cudaFree(G->tc_mem);
        G->tc_mem = nullptr;
        G->tc_bytes = 0;
        if ((e = cudaMalloc(&G->tc_mem, tcb)) != cudaSuccess) return e;
        G->tc_bytes = tcb;
    }
    if (!G->panel_stream) {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if ((e = cudaStreamCreateWithPriority(&G->panel_stream, cudaStreamNonBlocking, greatest)) != cudaSuccess)
            return e;
        if ((e = cudaEventCreateWithFlags(&G->ev_update, cudaEventDisableTiming)) != cudaSuccess) return e;
        if ((e = cudaEventCreateWithFlags(&G->ev_panel, cudaEventDisableTiming)) != cudaSuccess) return e;
        if (!G->workspace2 && (e = cudaMalloc(&G->workspace2, kBlasWorkspace)) != cudaSuccess) return e;
    }
    const Streams st{h, s, G->panel_stream, G->workspace, G->workspace2};
    ProfScope ps(Prof::LU_FACTOR, s);
    if ((e = factor_body(st, G, LU, G->dinv, G->panel, n, bad)) != cudaSuccess) return e;
    return build_super_inverses(h, G, LU, n, s);
}

// Lockstep factorization of m matrices: the same two-level blocked LU as factor_body
// (inner blocks of NB columns inside outer panels of outer_width() columns), with each
// step taken for every matrix at once.  Block step K is one launch of the diagonal
// kernel with one thread block per matrix that still has a block at K, then one launch
// each of the column solve, the in-panel row solve and the in-panel update over all
// matrices; after an outer panel, the U rows right of it by blocked forward substitution
// (two launches per inner block), then the rank-OB update of each matrix through cuBLAS
// (BF16x9).  The work items of every launch are planned on the host and uploaded once.
// No look-ahead stream: the diagonal blocks of all matrices run side by side instead.
cudaError_t lu_factor_batched(void* blas, LuGraphs* const* Gs, float* const* LUs, const int64_t* ns,
                              int* const* bads, int m, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    set_attrs();
    cublasHandle_t h = (cublasHandle_t)blas;
    cudaError_t e = prepare_blas(h, Gs[0], s);
    if (e != cudaSuccess) return e;
    std::vector<LuBatchMesh> desc(m);
    int64_t nmax = 0;
    for (int q = 0; q < m; q++) {
        LuGraphs* G = Gs[q];
        const int64_t n = ns[q];
        G->super_n = 0;  // no combined inverses for these factors: substitute by 128 columns
        if (G->solve) cudaGraphExecDestroy(G->solve);
        G->solve = nullptr;
        if (G->factor_n != n || !G->dinv) {
            if (G->solve) cudaGraphExecDestroy(G->solve);  // it holds the old Dinv
            G->solve = nullptr;
            if (G->dinv) cudaFree(G->dinv);
            G->dinv = nullptr;
            const size_t nb = (size_t)((n + NB - 1) / NB);
            if ((e = cudaMalloc(&G->dinv, sizeof(float) * nb * 2 * NB * NB)) != cudaSuccess) return e;
            G->factor_n = n;
        }
        desc[q] = LuBatchMesh{LUs[q], G->dinv, n, bads[q]};
        nmax = std::max(nmax, n);
    }
    // ---- plan
    enum { DIAG = 0, COLS = 1, ROWS = 2, GEMM = 3, RANK = 4 };
    struct Step {
        int kind;
        int64_t off, cnt;
        int q;
        int64_t KO, KE;
    };
    std::vector<Step> plan;
    std::vector<int> items;
    auto add = [&](int q, int64_t r0, int64_t r1, int64_t c0, int64_t c1, int64_t K, int b) {
        const int v[LB_ITEM] = {q, (int)r0, (int)r1, (int)c0, (int)c1, (int)K, b, 0};
        items.insert(items.end(), v, v + LB_ITEM);
    };
    int64_t mark = 0;
    auto open = [&]() { mark = (int64_t)items.size() / LB_ITEM; };
    auto close = [&](int kind) {
        const int64_t now = (int64_t)items.size() / LB_ITEM;
        if (now > mark) plan.push_back(Step{kind, mark, now - mark, -1, 0, 0});
    };
    const int64_t OB = outer_width(OB_BLOCKS_BATCHED);
    for (int64_t KO = 0; KO < nmax; KO += OB) {
        for (int64_t K = KO; K < KO + OB && K < nmax; K += NB) {
            open();
            for (int q = 0; q < m; q++)
                if (K < ns[q]) add(q, 0, 0, 0, 0, K, (int)std::min<int64_t>(NB, ns[q] - K));
            close(DIAG);
            open();
            for (int q = 0; q < m; q++) {
                const int64_t n = ns[q];
                if (K >= n) continue;
                const int b = (int)std::min<int64_t>(NB, n - K);
                for (int64_t r0 = K + b; r0 < n; r0 += CS_R) add(q, r0, n, 0, 0, K, b);
            }
            close(COLS);
            open();
            for (int q = 0; q < m; q++) {
                const int64_t n = ns[q], KE = std::min(KO + OB, n);
                if (K >= n) continue;
                const int b = (int)std::min<int64_t>(NB, n - K);
                for (int64_t c0 = K + b; c0 < KE; c0 += RS_C) add(q, 0, 0, c0, KE, K, b);
            }
            close(ROWS);
            open();
            for (int q = 0; q < m; q++) {
                const int64_t n = ns[q], KE = std::min(KO + OB, n);
                if (K >= n) continue;
                const int b = (int)std::min<int64_t>(NB, n - K);
                for (int64_t r0 = K + b; r0 < n; r0 += GS_R)
                    for (int64_t c0 = K + b; c0 < KE; c0 += GS_C) add(q, r0, n, c0, KE, K, b);
            }
            close(GEMM);
        }
        // U rows right of the panel: forward substitution by inner blocks
        for (int64_t K = KO; K < KO + OB; K += NB) {
            open();
            for (int q = 0; q < m; q++) {
                const int64_t n = ns[q], KE = KO + OB;
                if (KE >= n) continue;  // no columns right of the panel
                for (int64_t c0 = KE; c0 < n; c0 += RS_C) add(q, 0, 0, c0, n, K, NB);
            }
            close(ROWS);
            open();
            for (int q = 0; q < m; q++) {
                const int64_t n = ns[q], KE = KO + OB;
                if (KE >= n) continue;
                for (int64_t r0 = K + NB; r0 < KE; r0 += GS_R)
                    for (int64_t c0 = KE; c0 < n; c0 += GS_C) add(q, r0, KE, c0, n, K, NB);
            }
            close(GEMM);
        }
        for (int q = 0; q < m; q++)
            if (KO + OB < ns[q]) plan.push_back(Step{RANK, 0, 0, q, KO, KO + OB});
    }
    // ---- upload and issue
    LuBatchMesh* ddesc = nullptr;
    int* ditems = nullptr;
    if ((e = cudaMallocAsync((void**)&ddesc, sizeof(LuBatchMesh) * m, s)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync((void**)&ditems, sizeof(int) * std::max<size_t>(1, items.size()), s)) != cudaSuccess) {
        cudaFreeAsync(ddesc, s);
        return e;
    }
    e = cudaMemcpyAsync(ddesc, desc.data(), sizeof(LuBatchMesh) * m, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpyAsync(ditems, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, s);
    {
        ProfScope ps(Prof::LU_FACTOR, s);
        for (size_t t = 0; t < plan.size() && e == cudaSuccess; t++) {
            const Step& st = plan[t];
            const int* it = ditems + st.off * LB_ITEM;
            const unsigned g = (unsigned)st.cnt;
            switch (st.kind) {
                case DIAG: k_lu_diag_batched<<<g, DT, DIAG_SMEM, s>>>(ddesc, it); break;
                case COLS: k_col_solve_batched<<<g, 256, 0, s>>>(ddesc, it); break;
                case ROWS: k_row_solve_batched<<<g, 256, 0, s>>>(ddesc, it); break;
                case GEMM: k_gemm_sub_batched<<<g, 128, 0, s>>>(ddesc, it); break;
                default: {
                    const int64_t n = ns[st.q];
                    e = trailing(h, LUs[st.q], n, st.KO, (int)(st.KE - st.KO), st.KE, n - st.KE, st.KE, n - st.KE);
                }
            }
            if (e == cudaSuccess) e = cudaGetLastError();
        }
    }
    cudaFreeAsync(ditems, s);
    cudaFreeAsync(ddesc, s);
    return e;
}

cudaError_t solve_lu_refined_batched(const RefineMesh* ms, int m, double tol, int max_steps, SolveStats* st,
                                     cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    struct Bufs {
        double *r64, *P64, *part, *dd;
        float *d32, *y32;
    };
    std::vector<Bufs> B(m);
    std::vector<SubstMesh> desc(m);
    int64_t maxnb = 0;
    int kmax = 1;
    // each system's own work (conversions, residuals, norms) on its own stream; the
    // substitutions of all of them on s between a join and a fork
    std::vector<cudaStream_t> own;
    for (int q = 0; q < m; q++) {
        cudaStream_t t = ms[q].stream ? ms[q].stream : s;
        if (t != s && std::find(own.begin(), own.end(), t) == own.end()) own.push_back(t);
    }
    auto sq = [&](int q) { return ms[q].stream ? ms[q].stream : s; };
    std::vector<cudaEvent_t> evs(own.size() + 1);
    for (auto& ev : evs)
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return cudaErrorUnknown;
    struct EvFree {
        std::vector<cudaEvent_t>& v;
        ~EvFree() {
            for (auto ev : v) cudaEventDestroy(ev);
        }
    } evf{evs};
    auto join = [&]() -> cudaError_t {  // s waits for every system stream
        for (size_t j = 0; j < own.size(); j++) {
            cudaError_t ee = cudaEventRecord(evs[j], own[j]);
            if (ee == cudaSuccess) ee = cudaStreamWaitEvent(s, evs[j], 0);
            if (ee != cudaSuccess) return ee;
        }
        return cudaSuccess;
    };
    auto fork = [&]() -> cudaError_t {  // every system stream waits for s
        cudaError_t ee = cudaEventRecord(evs.back(), s);
        for (size_t j = 0; j < own.size() && ee == cudaSuccess; j++) ee = cudaStreamWaitEvent(own[j], evs.back(), 0);
        return ee;
    };
    auto sync_all = [&]() -> cudaError_t {
        cudaError_t ee = cudaStreamSynchronize(s);
        for (size_t j = 0; j < own.size() && ee == cudaSuccess; j++) ee = cudaStreamSynchronize(own[j]);
        return ee;
    };
    for (int q = 0; q < m; q++) {
        const RefineMesh& R = ms[q];
        if (R.k < 1 || R.k > 4096) return cudaErrorInvalidValue;
        char* p = (char*)R.work;
        auto take = [&](size_t bytes) {
            char* r = p;
            p += (bytes + 255) & ~size_t(255);
            return r;
        };
        const size_t kn = (size_t)R.k * R.n;  // the carving of solve_lu_refined
        B[q].r64 = (double*)take(sizeof(double) * kn);
        B[q].d32 = (float*)take(sizeof(float) * kn);
        B[q].y32 = (float*)take(sizeof(float) * kn);
        B[q].P64 = (double*)take(sizeof(double) * (size_t)residual_chunks(R.n) * 17 * R.n);
        B[q].part = (double*)take(sizeof(double) * 2 * R.k * 64);
        B[q].dd = (double*)take(sizeof(double) * 2 * R.k);
        desc[q] = SubstMesh{R.LU, R.dinv, B[q].d32, B[q].y32, R.n, R.k, 0};
        maxnb = std::max(maxnb, (R.n + NB - 1) / NB);
        kmax = std::max(kmax, R.k);
    }
    // the substitution plan (the same for every pass)
    struct Step {
        int kind, dir;
        int64_t off, cnt;
    };
    std::vector<Step> plan;
    std::vector<int> items;
    auto add = [&](int q, int64_t r0, int64_t r1, int64_t K, int b) {
        const int v[LB_ITEM] = {q, (int)r0, (int)r1, 0, 0, (int)K, b, 0};
        items.insert(items.end(), v, v + LB_ITEM);
    };
    auto step = [&](int kind, int dir, int64_t t) {
        const int64_t off = (int64_t)items.size() / LB_ITEM;
        for (int q = 0; q < m; q++) {
            const int64_t n = ms[q].n, K = t * NB;
            if (K >= n) continue;
            const int b = (int)std::min<int64_t>(NB, n - K);
            if (kind == 0) {
                add(q, 0, 0, K, b);
            } else if (dir == 0) {
                for (int64_t r0 = K + b; r0 < n; r0 += NB) add(q, r0, n, K, b);
            } else {
                for (int64_t r0 = 0; r0 < K; r0 += NB) add(q, r0, K, K, b);
            }
        }
        const int64_t cnt = (int64_t)items.size() / LB_ITEM - off;
        if (cnt > 0) plan.push_back(Step{kind, dir, off, cnt});
    };
    for (int64_t t = 0; t < maxnb; t++) {
        step(0, 0, t);
        step(1, 0, t);
    }
    for (int64_t t = maxnb - 1; t >= 0; t--) {
        step(0, 1, t);
        step(1, 1, t);
    }
    cudaError_t e;
    SubstMesh* ddesc = nullptr;
    int *ditems = nullptr, *dact = nullptr;
    if ((e = cudaMallocAsync((void**)&ddesc, sizeof(SubstMesh) * m, s)) != cudaSuccess) return e;
    if ((e = cudaMallocAsync((void**)&ditems, sizeof(int) * std::max<size_t>(1, items.size()), s)) != cudaSuccess) {
        cudaFreeAsync(ddesc, s);
        return e;
    }
    if ((e = cudaMallocAsync((void**)&dact, sizeof(int) * m, s)) != cudaSuccess) {
        cudaFreeAsync(ditems, s);
        cudaFreeAsync(ddesc, s);
        return e;
    }
    struct Free {
        void *a, *b, *c;
        cudaStream_t s;
        ~Free() {
            cudaFreeAsync(a, s);
            cudaFreeAsync(b, s);
            cudaFreeAsync(c, s);
        }
    } fr{ddesc, ditems, dact, s};
    if ((e = cudaMemcpyAsync(ddesc, desc.data(), sizeof(SubstMesh) * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    if (!items.empty() &&
        (e = cudaMemcpyAsync(ditems, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, s)) !=
            cudaSuccess)
        return e;
    // start: x = 0, r = b, and the right-hand sides' norms
    std::vector<std::vector<double>> hd(m);
    if ((e = fork()) != cudaSuccess) return e;  // the plan's uploads before any system's work
    for (int q = 0; q < m; q++) {
        const RefineMesh& R = ms[q];
        const size_t kn = (size_t)R.k * R.n;
        hd[q].assign(2 * R.k, 0.0);
        cudaMemsetAsync(R.x, 0, sizeof(double) * kn, sq(q));
        cudaMemcpyAsync(B[q].r64, R.rhs, sizeof(double) * kn, cudaMemcpyDeviceToDevice, sq(q));
        if ((e = column_norms2_device(R.rhs, R.n, R.k, B[q].part, B[q].dd, sq(q))) != cudaSuccess) return e;
    }
    // hd is pageable host memory: each copy returns when it is done, so the systems' copies
    // are issued after all their kernels, stream by stream
    auto read_norms = [&](const std::vector<int>& act) -> cudaError_t {
        for (int q = 0; q < m; q++)
            if (act[q]) {
                cudaError_t ee = cudaMemcpyAsync(hd[q].data(), B[q].dd, sizeof(double) * ms[q].k,
                                                 cudaMemcpyDeviceToHost, sq(q));
                if (ee != cudaSuccess) return ee;
            }
        return sync_all();
    };
    std::vector<int> act(m, 1);
    if ((e = read_norms(act)) != cudaSuccess) return e;
    std::vector<std::vector<double>> bn(m);
    for (int q = 0; q < m; q++) {
        bn[q].resize(ms[q].k);
        for (int c = 0; c < ms[q].k; c++) bn[q][c] = std::sqrt(hd[q][c]);
        st[q].refinements = 0;
        st[q].residual_max = 1;
    }
    for (int pass = 0; pass < max_steps; pass++) {
        int nact = 0;
        for (int q = 0; q < m; q++) nact += act[q];
        if (nact == 0) break;
        // every stream is idle here (after read_norms), so this small pageable copy costs
        // no overlap
        if ((e = cudaMemcpyAsync(dact, act.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return e;
        if ((e = fork()) != cudaSuccess) return e;
        for (int q = 0; q < m; q++)
            if (act[q]) {
                const size_t kn = (size_t)ms[q].k * ms[q].n;
                k_d2f<<<nb256(kn), 256, 0, sq(q)>>>(B[q].r64, B[q].d32, kn);
            }
        if ((e = join()) != cudaSuccess) return e;
        {
            ProfScope ps(Prof::LU_SOLVE, s);
            for (const Step& stp : plan) {
                const int* it = ditems + stp.off * LB_ITEM;
                if (kmax <= 8)
                    subst_launch<8>(stp.kind, (unsigned)stp.cnt, ddesc, it, dact, stp.dir, s);
                else if (kmax <= 16)
                    subst_launch<16>(stp.kind, (unsigned)stp.cnt, ddesc, it, dact, stp.dir, s);
                else
                    subst_launch<32>(stp.kind, (unsigned)stp.cnt, ddesc, it, dact, stp.dir, s);
            }
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = fork()) != cudaSuccess) return e;
        for (int q = 0; q < m; q++)
            if (act[q]) {
                const RefineMesh& R = ms[q];
                const size_t kn = (size_t)R.k * R.n;
                k_addf<<<nb256(kn), 256, 0, sq(q)>>>(R.x, B[q].d32, kn);
                if ((e = residual_df(R.A32, R.Alo, R.n, R.k, R.x, R.rhs, B[q].r64, B[q].P64, sq(q))) != cudaSuccess)
                    return e;
                if ((e = column_norms2_device(B[q].r64, R.n, R.k, B[q].part, B[q].dd, sq(q))) != cudaSuccess)
                    return e;
            }
        if ((e = read_norms(act)) != cudaSuccess) return e;
        for (int q = 0; q < m; q++)
            if (act[q]) {
                double worst = 0;
                for (int c = 0; c < ms[q].k; c++)
                    worst = std::max(worst, bn[q][c] > 0 ? std::sqrt(hd[q][c]) / bn[q][c] : 0.0);
                st[q].refinements++;
                st[q].residual_max = worst;
                if (worst <= tol) act[q] = 0;
            }
    }
    return cudaGetLastError();
}

size_t lu_blas_workspace_bytes() { return kBlasWorkspace; }

// X (n x k, ld n) <- U^{-1} L^{-1} X
cudaError_t lu_solve_fp32(void* blas, LuGraphs* G, const float* LU, int64_t n, float* X, int k, cudaStream_t s) {
    set_attrs();
    cublasHandle_t h = (cublasHandle_t)blas;
    cudaError_t e = prepare_blas(h, G, s);
    if (e != cudaSuccess) return e;
    if (!G->dinv) return cudaErrorInvalidValue;  // factor first
    if (!G->solve || G->solve_X != X || G->solve_k != k || G->solve_LU != LU) {
        if (G->solve) cudaGraphExecDestroy(G->solve);
        G->solve = nullptr;
        if (G->tmp_floats < (size_t)n * k) {
            if (G->tmp) cudaFree(G->tmp);
            G->tmp = nullptr;
            if ((e = cudaMalloc(&G->tmp, sizeof(float) * n * k)) != cudaSuccess) return e;
            G->tmp_floats = (size_t)n * k;
        }
        const int64_t nsup = (G->super_n == n && G->dinv4) ? n / SB : 0;
        e = capture(s, &G->solve, [&] { return solve_body(h, LU, G->dinv, G->dinv4, nsup, n, X, G->tmp, k); });
        if (e != cudaSuccess) return e;
        G->solve_X = X;
        G->solve_k = k;
        G->solve_LU = LU;
    }
    ProfScope ps(Prof::LU_SOLVE, s);
    return cudaGraphLaunch(G->solve, s);
}

__global__ void k_identity(float* __restrict__ X, int64_t n) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n * n) X[t] = (t / n == t % n) ? 1.f : 0.f;
}

cudaError_t lu_invert_fp32(void* blas, LuGraphs* G, const float* LU, int64_t n, float* Ainv, cudaStream_t s) {
    k_identity<<<nb256(n * n), 256, 0, s>>>(Ainv, n);
    cudaError_t e = lu_solve_fp32(blas, G, LU, n, Ainv, (int)n, s);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    // the n-column substitution graph and its n x n scratch are not needed again
    if (G->solve) cudaGraphExecDestroy(G->solve);
    G->solve = nullptr;
    G->solve_X = nullptr;
    G->solve_k = 0;
    if (G->tmp) cudaFree(G->tmp);
    G->tmp = nullptr;
    G->tmp_floats = 0;
    return cudaSuccess;
}

size_t solve_lu_work_bytes(int64_t n, int k) {
    size_t kn = (size_t)k * n;
    return sizeof(double) * (2 * kn + 2 * (size_t)k * 64 + 2 * (size_t)k) + 2 * sizeof(float) * kn +
           sizeof(double) * (size_t)residual_chunks(n) * 17 * (size_t)n + 64 * 1024;
}

cudaError_t solve_lu_refined(void* blas, LuGraphs* G, const float* A32, const float* Alo, const float* LU, int64_t n,
                             int k, const double* rhs, double* x, void* work, double tol, int max_steps,
                             SolveStats* st, cudaStream_t s, const float* Ainv) {
    char* p = (char*)work;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    const size_t kn = (size_t)k * n;
    double* r64 = (double*)take(sizeof(double) * kn);
    float* d32 = (float*)take(sizeof(float) * kn);
    float* e32 = (float*)take(sizeof(float) * kn);  // Ainv r
    double* P64 = (double*)take(sizeof(double) * (size_t)residual_chunks(n) * 17 * n);
    double* part = (double*)take(sizeof(double) * 2 * k * 64);
    double* dd = (double*)take(sizeof(double) * 2 * k);
    std::vector<double> hd(2 * k), bn(k);
    cudaError_t e;
    cudaMemsetAsync(x, 0, sizeof(double) * kn, s);
    cudaMemcpyAsync(r64, rhs, sizeof(double) * kn, cudaMemcpyDeviceToDevice, s);
    if ((e = column_norms2(rhs, n, k, part, dd, hd.data(), s)) != cudaSuccess) return e;
    for (int c = 0; c < k; c++) bn[c] = std::sqrt(hd[c]);
    double worst = 1;
    int steps = 0;
    for (; steps < max_steps; steps++) {
        k_d2f<<<nb256(kn), 256, 0, s>>>(r64, d32, kn);
        if (Ainv) {  // correction = Ainv r (one product instead of the two substitutions)
            cublasHandle_t h = (cublasHandle_t)blas;
            if ((e = prepare_blas(h, G, s)) != cudaSuccess) return e;
            const float one = 1.f, zero = 0.f;
            cublasStatus_t bs = k == 1 ? cublasSgemv(h, CUBLAS_OP_N, (int)n, (int)n, &one, Ainv, (int)n, d32, 1, &zero,
                                                     e32, 1)
                                       : cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)n, k, (int)n, &one, Ainv,
                                                     (int)n, d32, (int)n, &zero, e32, (int)n);
            if (bs != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
            k_addf<<<nb256(kn), 256, 0, s>>>(x, e32, kn);
        } else {
            if ((e = lu_solve_fp32(blas, G, LU, n, d32, k, s)) != cudaSuccess) return e;
            k_addf<<<nb256(kn), 256, 0, s>>>(x, d32, kn);
        }
        if ((e = residual_df(A32, Alo, n, k, x, rhs, r64, P64, s)) != cudaSuccess) return e;
        if ((e = column_norms2(r64, n, k, part, dd, hd.data(), s)) != cudaSuccess) return e;
        worst = 0;
        for (int c = 0; c < k; c++) worst = std::max(worst, bn[c] > 0 ? std::sqrt(hd[c]) / bn[c] : 0.0);
        if (worst <= tol) {
            steps++;
            break;
        }
    }
    if (st) {
        st->refinements += steps;
        st->residual_max = std::max(st->residual_max, worst);
    }
    return cudaGetLastError();
}

}  // namespace cpg
