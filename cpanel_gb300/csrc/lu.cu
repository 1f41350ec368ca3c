// Direct FP32 solve of the mixed path: blocked right-looking LU without pivoting,
// then iterative refinement against the double-float matrix (hi + lo).
//
// The panel matrix has a -0.5 self term on the diagonal; measured pivot growth of
// the unpivoted factorization is 1.00003 on the synthetic wings, and refinement
// with an exact-product residual reaches 1e-12 relative in three passes.
// Every kernel is hand-written: the diagonal blocks and the block steps inside them on the
// CUDA cores, the panel products and the trailing updates on the tensor cores (tc_gemm.cu),
// the substitutions as skinny products on the CUDA cores (skinny.cu).
#include "tc_gemm.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "assemble.h"
#include "skinny.h"

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

// PRE: before factoring, the block takes the update of the 128-column step before it,
// A_KK -= L(K.., K-NB..K) U(K-NB..K, K..): the caller's update of the rest of the trailing matrix
// then skips this block, and this kernel is the only launch between two diagonal steps.
template <bool PRE>
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
            if constexpr (!PRE) {
                ZL[r * P + c] = r == c ? 1.f : 0.f;
                ZU[r * P + c] = r == c ? 1.f : 0.f;
            }
        }
    }
    if constexpr (PRE) {
        // the previous step's L rows of this block (into ZL) and U columns of it (into ZU), zero
        // outside the block's b rows and columns
        float vl[NB * NB / DT], vu[NB * NB / DT];
#pragma unroll
        for (int q = 0; q < NB * NB / DT; q++) {
            const int idx = t + q * DT, c = idx / NB, r = idx % NB;
            vl[q] = r < b ? A[(K - NB + c) * n + K + r] : 0.f;
            vu[q] = c < b ? A[(K + c) * n + K - NB + r] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < NB * NB / DT; q++) {
            const int idx = t + q * DT, c = idx / NB, r = idx % NB;
            ZL[r * P + c] = vl[q];
            ZU[r * P + c] = vu[q];
        }
        __syncthreads();
        // S -= ZL ZU: thread t takes rows 4 (t / 16) .. + 3 and columns t % 16 + 16 x (x < 8)
        const int tr = t / 16, tc = t % 16;
        float acc[4][8];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int x = 0; x < 8; x++) acc[i][x] = 0.f;
        for (int k = 0; k < NB; k++) {
            float a[4], u[8];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = ZL[(4 * tr + i) * P + k];
#pragma unroll
            for (int x = 0; x < 8; x++) u[x] = ZU[k * P + tc + 16 * x];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int x = 0; x < 8; x++) acc[i][x] = __fmaf_rn(a[i], u[x], acc[i][x]);
        }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int x = 0; x < 8; x++) S[(4 * tr + i) * P + tc + 16 * x] -= acc[i][x];
        __syncthreads();
        for (int idx = t; idx < NB * NB; idx += DT) {
            const int c = idx / NB, r = idx % NB;
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

template <bool PRE>
__global__ void __launch_bounds__(DT) k_lu_diag(float* __restrict__ A, int64_t n, int64_t K, int b,
                                                float* __restrict__ Dinv, int* bad) {
    extern __shared__ float sm[];
    lu_diag_body<PRE>(sm, A, n, K, b, Dinv, bad);
}

// ---- block steps of the factorization, shared by the single-matrix and the lockstep kernels ----
// The matrices are column-major with their own order n (LU[c*n + r]).

// L21 = A21 U_KK^{-1} in place for rows [r0, min(r0 + 64, r1)), columns K..K+b.  256 threads:
// thread t owns row t % 64 and the 32 columns 32 (t / 64) ..; U^{-1} staged 16 rows at a time, or
// (FULL, the single-matrix chain kernel, one thread block per SM at most) all of it at once, with
// one barrier instead of sixteen.  The products are summed in the same order either way.
constexpr int CS_R = 64;
constexpr int CS_SMEM = (CS_R * (NB + 1) + 16 * NB) * 4;
constexpr int CS_FULL_SMEM = (CS_R * (NB + 1) + NB * (NB + 4)) * 4;
template <bool FULL>
__device__ __forceinline__ void col_solve_body(float* __restrict__ A, int64_t n, const float* __restrict__ dinv,
                                               int64_t r0, int64_t r1, int64_t K, int b, float* smem) {
    float (*X)[NB + 1] = reinterpret_cast<float (*)[NB + 1]>(smem);
    float (*U)[NB] = reinterpret_cast<float (*)[NB]>(smem + CS_R * (NB + 1));  // 16-byte aligned
    const float* Ui = dinv + (K / NB) * 2 * NB * NB + NB * NB;  // column-major, ld NB
    const int t = threadIdx.x, r = t % CS_R, cg = t / CS_R;
    {
        float v[CS_R * NB / 256];
#pragma unroll
        for (int q = 0; q < CS_R * NB / 256; q++) {
            const int idx = t + 256 * q, c = idx / CS_R, rr = idx % CS_R;
            v[q] = (r0 + rr < r1 && c < b) ? A[(K + c) * n + r0 + rr] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < CS_R * NB / 256; q++) {
            const int idx = t + 256 * q;
            X[idx % CS_R][idx / CS_R] = v[q];
        }
    }
    float acc[32];
#pragma unroll
    for (int j = 0; j < 32; j++) acc[j] = 0.f;
    if constexpr (FULL) {
        float (*Uf)[NB + 4] = reinterpret_cast<float (*)[NB + 4]>(smem + CS_R * (NB + 1));  // 16-byte aligned
        for (int idx = t; idx < NB * NB; idx += 256) {
            const int kk = idx % NB, c = idx / NB;
            Uf[kk][c] = (kk < b && c < b) ? Ui[kk + (int64_t)c * NB] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < b; kk++) {
            const float a = X[r][kk];
            const float4* u4 = reinterpret_cast<const float4*>(&Uf[kk][32 * cg]);
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
    for (int k0 = 0; !FULL && k0 < b; k0 += 16) {
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

// U12 = L_KK^{-1} A12 in place for rows K..K+b, columns [c0, min(c0 + 64, c1)).  256 threads:
// thread t owns row t % 128 and the 32 columns 32 (t / 128) ..; L^{-1} staged 16 columns at a
// time, or (FULL) all of it at once.
constexpr int RS_C = 64;
constexpr int RS_SMEM = (NB * (RS_C + 4) + 16 * (NB + 1)) * 4;
constexpr int RS_FULL_SMEM = (NB * (RS_C + 4) + NB * (NB + 1)) * 4;
constexpr int CR_FULL_SMEM = CS_FULL_SMEM > RS_FULL_SMEM ? CS_FULL_SMEM : RS_FULL_SMEM;
template <bool FULL>
__device__ __forceinline__ void row_solve_body(float* __restrict__ A, int64_t n, const float* __restrict__ dinv,
                                               int64_t c0, int64_t c1, int64_t K, int b, float* smem) {
    float (*X)[RS_C + 4] = reinterpret_cast<float (*)[RS_C + 4]>(smem);  // rows of 272 bytes
    float (*L)[NB + 1] = reinterpret_cast<float (*)[NB + 1]>(smem + NB * (RS_C + 4));
    const float* Li = dinv + (K / NB) * 2 * NB * NB;  // column-major, ld NB
    const int t = threadIdx.x, r = t % NB, cg = t / NB;
    {
        float v[NB * RS_C / 256];
#pragma unroll
        for (int q = 0; q < NB * RS_C / 256; q++) {
            const int idx = t + 256 * q, c = idx / NB, k = idx % NB;
            v[q] = (k < b && c0 + c < c1) ? A[(c0 + c) * n + K + k] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < NB * RS_C / 256; q++) {
            const int idx = t + 256 * q;
            X[idx % NB][idx / NB] = v[q];
        }
    }
    float acc[32];
#pragma unroll
    for (int j = 0; j < 32; j++) acc[j] = 0.f;
    if constexpr (FULL) {
        for (int idx = t; idx < NB * NB; idx += 256) {
            const int kk = idx / NB, rr = idx % NB;
            L[kk][rr] = (kk < b && rr < b) ? Li[rr + (int64_t)kk * NB] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < b; kk++) {
            const float a = L[kk][r];
            const float4* x4 = reinterpret_cast<const float4*>(&X[kk][32 * cg]);
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
    for (int k0 = 0; !FULL && k0 < b; k0 += 16) {
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

// acc = sum_k A[i + k lda] B[k + j ldb] for the TR x (8192 / TR) tile i < m, j < nc (A and B
// already offset to the tile's first row and column), k < kk_n; TR = 128 or 64.  128 threads, each
// an 8 x 8 block of the tile in registers (rows 8 (t % (TR / 8)) .., columns 8 (t / (TR / 8)) ..);
// A and B copied GS_K columns / rows at a time into one of two shared-memory stages by cp.async
// (the next chunk is in flight while the current one is multiplied) and read as float4 (two
// loads each per k for 64 FMAs).  Elements outside the tile or past kk_n are zero-filled.
constexpr int GS_R = 128, GS_C = 64, GS_K = 32;
constexpr int GS_STAGE = GS_K * (GS_R + GS_C);
__shared__ __align__(16) float s_tile[2 * GS_STAGE];
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
template <int TR>
__device__ __forceinline__ void tile_mm(const float* A, int64_t lda, const float* B, int64_t ldb, int64_t m,
                                        int64_t nc, int kk_n, float (&acc)[8][8]) {
    constexpr int TC = 8192 / TR, GR = TR / 8;
    const int t = threadIdx.x, tr = t % GR, tc = t / GR;
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
    auto stage = [&](int st, int k0) {
        float* Ls = s_tile + st * GS_STAGE;  // [GS_K][TR]
        float* Us = Ls + GS_K * TR;          // [GS_K][TC]
        for (int idx = t; idx < GS_K * TR; idx += 128) {
            const int kk = idx / TR, rr = idx % TR;
            const bool v = k0 + kk < kk_n && rr < m;
            cp_async4(Ls + idx, v ? A + (int64_t)(k0 + kk) * lda + rr : A, v);
        }
        for (int idx = t; idx < GS_K * TC; idx += 128) {
            const int kk = idx % GS_K, c = idx / GS_K;
            const bool v = k0 + kk < kk_n && c < nc;
            cp_async4(Us + kk * TC + c, v ? B + (int64_t)c * ldb + k0 + kk : B, v);
        }
    };
    if (kk_n > 0) stage(0, 0);
    cp_async_commit();
    for (int k0 = 0, st = 0; k0 < kk_n; k0 += GS_K, st ^= 1) {
        if (k0 + GS_K < kk_n) stage(st ^ 1, k0 + GS_K);
        cp_async_commit();
        cp_async_wait1();  // this chunk's copies (all but the group just committed) have landed
        __syncthreads();
        const float* Ls = s_tile + st * GS_STAGE;
        const float* Us = Ls + GS_K * TR;
#pragma unroll 4
        for (int kk = 0; kk < GS_K; kk++) {
            const float4 a0 = *reinterpret_cast<const float4*>(&Ls[kk * TR + 8 * tr]);
            const float4 a1 = *reinterpret_cast<const float4*>(&Ls[kk * TR + 8 * tr + 4]);
            const float4 u0 = *reinterpret_cast<const float4*>(&Us[kk * TC + 8 * tc]);
            const float4 u1 = *reinterpret_cast<const float4*>(&Us[kk * TC + 8 * tc + 4]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float u[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = __fmaf_rn(a[i], u[j], acc[i][j]);
        }
        __syncthreads();  // the stage is free for the chunk after next
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// C -= L(:, K..K+b) U(K..K+b, :) on the tile rows [r0, min(r0 + 128, r1)) x columns
// [c0, min(c0 + 64, c1)).
__device__ __forceinline__ void gemm_sub_body(float* __restrict__ A, int64_t n, int64_t r0, int64_t r1, int64_t c0,
                                              int64_t c1, int64_t K, int b) {
    float acc[8][8];
    tile_mm<GS_R>(A + K * n + r0, n, A + c0 * n + K, n, r1 - r0, c1 - c0, b, acc);
    const int t = threadIdx.x, tr = t % 16, tc = t / 16;
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

// single matrix: the column solve of block K for rows [rb, re) (the first ceil((re - rb) / 64)
// thread blocks, 64 rows each) and its row solve for columns [cb, ce) (the others, 64 columns
// each), in one launch
__global__ void __launch_bounds__(256) k_colrow_solve(float* __restrict__ A, int64_t n, const float* __restrict__ dinv,
                                                      int64_t rb, int64_t re, int64_t cb, int64_t ce, int64_t K,
                                                      int b) {
    extern __shared__ __align__(16) float dsm[];
    const int64_t nrt = (re - rb + CS_R - 1) / CS_R;
    if ((int64_t)blockIdx.x < nrt)
        col_solve_body<true>(A, n, dinv, rb + (int64_t)blockIdx.x * CS_R, re, K, b, dsm);
    else
        row_solve_body<true>(A, n, dinv, cb + ((int64_t)blockIdx.x - nrt) * RS_C, ce, K, b, dsm);
}
// single matrix: the update of rows [rb, re) x columns [cb, ce) by block K, one 128 x 64 tile
// per thread block, except the 128 x 128 block at (rb, cb), which the next diagonal kernel updates
__global__ void __launch_bounds__(128) k_gemm_sub(float* __restrict__ A, int64_t n, int64_t rb, int64_t re,
                                                  int64_t cb, int64_t ce, int64_t K, int b) {
    if (blockIdx.x == 0 && blockIdx.y < NB / GS_C) return;
    gemm_sub_body(A, n, rb + (int64_t)blockIdx.x * GS_R, re, cb + (int64_t)blockIdx.y * GS_C, ce, K, b);
}

// ---- lockstep factorization of many matrices (the batch path) ----
// Every kernel below takes work items of LB_ITEM ints: mesh, r0, r1, c0, c1, K, b, unused.
constexpr int LB_ITEM = 8;

// diagonal block K of every listed mesh, one block of DT threads each
__global__ void __launch_bounds__(DT) k_lu_diag_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                        const int* __restrict__ items) {
    extern __shared__ float sm[];
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    lu_diag_body<false>(sm, d.LU, d.n, it[5], it[6], d.dinv, d.bad);
}
__global__ void __launch_bounds__(256) k_col_solve_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                           const int* __restrict__ items) {
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    extern __shared__ __align__(16) float dsm[];
    col_solve_body<false>(d.LU, d.n, d.dinv, it[1], it[2], it[5], it[6], dsm);
}
__global__ void __launch_bounds__(256) k_row_solve_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                           const int* __restrict__ items) {
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    extern __shared__ __align__(16) float dsm[];
    row_solve_body<false>(d.LU, d.n, d.dinv, it[3], it[4], it[5], it[6], dsm);
}
__global__ void __launch_bounds__(128) k_gemm_sub_batched(const cpg::LuBatchMesh* __restrict__ ms,
                                                          const int* __restrict__ items) {
    const int* it = items + LB_ITEM * blockIdx.x;
    const cpg::LuBatchMesh d = ms[it[0]];
    gemm_sub_body(d.LU, d.n, it[1], it[2], it[3], it[4], it[5], it[6]);
}

// ---- inverses of the SB-column diagonal blocks, one 128-column step at a time ----
// Step j of the inverses of the SB-column diagonal block at KO (D4: L^{-1} then U^{-1},
// column-major, ld SB), once its 128-column block j is factored (inverses in Dinv) and the
// L^{-1} rows and U^{-1} columns of the blocks before it are final:
//   L^{-1}[j, c] = -L_jj^{-1} sum_{c <= k < j} L[j, k] L^{-1}[k, c]    (64-column tiles, c < j)
//   U^{-1}[r, j] = -(sum_{r <= k < j} U^{-1}[r, k] U[k, j]) U_jj^{-1}    (64-row tiles, r < j)
// (block indices of 128; the sums run over the columns and rows that are not zero), then the
// rest of L^{-1}'s block row j (L_jj^{-1}, zeros to its right) and of U^{-1}'s block column j
// (U_jj^{-1}, zeros below).  Thread blocks of 128 threads.  The sum of a tile runs in K chunks of
// at most INV_KCH, one thread block each, so that the step takes about as long as its shortest
// tiles: each chunk's product goes to its own 8,192 floats of T, and the last chunk of a tile to
// arrive (counter cnt[tile], returned to 0) adds them in chunk order and applies the diagonal
// block's inverse.  Blocks: the chunks of the 2j L tiles, then of the 2j U tiles, then 2 fill.
constexpr int INV_KCH = 256;
__host__ __device__ constexpr int inv_chunks(int j, int q) { return (64 * (2 * j - q) + INV_KCH - 1) / INV_KCH; }
int inv_step_blocks(int j) {
    int c = 0;
    for (int q = 0; q < 2 * j; q++) c += inv_chunks(j, q);
    return 2 * c + 2;
}
__global__ void __launch_bounds__(128) k_inv_step(const float* __restrict__ LU, int64_t n, int64_t KO, int j,
                                                  const float* __restrict__ Dinv, float* D4, float* T,
                                                  unsigned* __restrict__ cnt) {
    __shared__ int s_last;
    const int nt = 2 * j, t = threadIdx.x;
    float* Linv = D4;
    float* Uinv = D4 + SB * SB;
    const int64_t J = (int64_t)NB * j;  // first row and column of block j inside the SB block
    const float* Ljj = Dinv + (KO / NB + j) * 2 * NB * NB;  // ld NB
    const float* Ujj = Ljj + NB * NB;
    // this block's tile (side 0: L, 1: U; q), chunk ch of nch, and its first slot of T
    int b = blockIdx.x, side = 0, q = 0, slot = 0;
    for (; side < 2; side++) {
        for (q = 0; q < nt; q++) {
            const int c = inv_chunks(j, q);
            if (b < c) break;
            b -= c;
            slot += c;
        }
        if (q < nt) break;
    }
    if (side == 2) {  // the fill blocks
        if (b == 0) {  // L^{-1}[J.., J..SB): L_jj^{-1}, then zeros
            for (int idx = t; idx < NB * (SB - (int)J); idx += 128) {
                const int64_t c = J + idx / NB;
                const int r = idx % NB;
                Linv[(J + r) + c * SB] = c < J + NB ? Ljj[r + (c - J) * NB] : 0.f;
            }
        } else {  // U^{-1}[J..SB, J..): U_jj^{-1}, then zeros
            const int h = SB - (int)J;
            for (int idx = t; idx < NB * h; idx += 128) {
                const int c = idx / h;
                const int64_t r = J + idx % h;
                Uinv[r + (J + c) * SB] = r < J + NB ? Ujj[(r - J) + (int64_t)c * NB] : 0.f;
            }
        }
        return;
    }
    const int ch = b, nch = inv_chunks(j, q);
    const int64_t o0 = 64 * (int64_t)q;  // c0 (L) or r0 (U)
    const int kt = (int)(J - o0), k0 = ch * INV_KCH, kn = min(INV_KCH, kt - k0);
    float* Tq = T + (int64_t)(slot + ch) * 8192;
    float acc[8][8];
    if (side == 0) {  // partial of L^{-1}[J.., c0..c0+64): 128 x 64, ld 128
        const int tr = t % 16, tc = t / 16;
        tile_mm<128>(LU + (KO + o0 + k0) * n + KO + J, n, Linv + o0 + k0 + o0 * SB, SB, 128, 64, kn, acc);
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int jj = 0; jj < 8; jj++) Tq[(8 * tc + jj) * 128 + 8 * tr + i] = acc[i][jj];
    } else {  // partial of U^{-1}[r0..r0+64, J..): 64 x 128, ld 64
        const int tr = t % 8, tc = t / 8;
        tile_mm<64>(Uinv + o0 + (o0 + k0) * SB, SB, LU + (KO + J) * n + KO + o0 + k0, n, 64, 128, kn, acc);
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int jj = 0; jj < 8; jj++) Tq[(8 * tc + jj) * 64 + 8 * tr + i] = acc[i][jj];
    }
    float* T0 = T + (int64_t)slot * 8192;  // the tile's sum (chunk 0's slot)
    if (nch > 1) {
        __threadfence();
        __syncthreads();
        const int tile = side * nt + q;
        if (t == 0) s_last = atomicAdd(cnt + tile, 1u) == (unsigned)(nch - 1);
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        if (t == 0) cnt[tile] = 0u;
        for (int e = t; e < 8192; e += 128) {
            float v = __ldcg(T0 + e);
            for (int c = 1; c < nch; c++) v += __ldcg(T0 + (int64_t)c * 8192 + e);
            T0[e] = v;
        }
    }
    __syncthreads();
    if (side == 0) {
        const int tr = t % 16, tc = t / 16;
        tile_mm<128>(Ljj, NB, T0, 128, 128, 64, NB, acc);
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int jj = 0; jj < 8; jj++) Linv[(J + 8 * tr + i) + (o0 + 8 * tc + jj) * SB] = -acc[i][jj];
    } else {
        const int tr = t % 8, tc = t / 8;
        tile_mm<64>(T0, 64, Ujj, NB, 64, 128, NB, acc);
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int jj = 0; jj < 8; jj++) Uinv[(o0 + 8 * tr + i) + (J + 8 * tc + jj) * SB] = -acc[i][jj];
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
                       cudaFuncSetAttribute(k_lu_diag<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM);
                       cudaFuncSetAttribute(k_lu_diag<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM);
                       cudaFuncSetAttribute(k_lu_diag_batched, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            DIAG_SMEM);
                       cudaFuncSetAttribute(k_colrow_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            CR_FULL_SMEM);
                   });
}

}  // namespace

namespace cpg {

namespace {

// Right-looking blocked LU by outer panels of SB = 1,024 columns.  Per panel [KO, KE):
//   1. its diagonal block is factored in place by 128-column steps restricted to the block
//      (k_lu_diag, then one launch of the column and row solves and one of the update inside
//      the block); after each step's k_lu_diag a third stream extends L11^{-1} and U11^{-1} of
//      the whole block by that step (k_inv_step), so the inverses are ready one step after
//      the factors;
//   2. L21 = A21 U11^{-1} and U12 = L11^{-1} A12 on the tensor cores (no pivoting, so the
//      panel's off-diagonal factors are these products);
//   3. A22 -= L21 U12 on the tensor cores.
// Look-ahead: the rows of L21 and the columns of U12 that meet the next diagonal block come
// first (1,024-wide products), then that block's update; it is factored on a high-priority
// stream while the rest of L21, U12 and the update run with kPanelSms SMs left to it.  The
// serial chain is the diagonal blocks and these three small products.
// (the 19,272-panel wing's factorization: 26.0 ms with 24 SMs, 26.2-26.3 ms with 16, 20 or 32,
// 26.7 ms with 12 or 40)
constexpr int kPanelSms = 24;
// tile scratch of k_inv_step: the chunks of step 7 (32 L and 32 U), then its per-tile counters
constexpr int64_t kInvScratch = 4 * (SB / 64) * 8192;
constexpr int64_t kInvCounters = 32;

// factorization of the diagonal block [KO, KE) x [KO, KE) in place on s (the updates of the
// earlier panels applied), the inverses of its 128-column blocks into G->dinv; for a full SB
// block also its combined inverses into G->dinv4 on G->inv_stream, joined back into s at the end.
// Look-ahead inside the block: step j's column and row solves, then the next diagonal kernel on s,
// which first applies step j's update to its own block; step j's update of the rest of the block
// runs on G->rest_stream beside it, and step j + 1's solves wait for it.
cudaError_t factor_diag_block(LuGraphs* G, float* LU, int64_t n, int* bad, int64_t KO, int64_t KE, cudaStream_t s) {
    cudaError_t e;
    const bool inv = KE - KO == SB;
    float* D4 = inv ? G->dinv4 + (KO / SB) * 2 * SB * SB : nullptr;
    for (int64_t K = KO; K < KE; K += NB) {
        const int b = (int)std::min<int64_t>(NB, KE - K);
        if (K == KO)
            k_lu_diag<false><<<1, DT, DIAG_SMEM, s>>>(LU, n, K, b, G->dinv, bad);
        else
            k_lu_diag<true><<<1, DT, DIAG_SMEM, s>>>(LU, n, K, b, G->dinv, bad);
        if (inv) {
            const int j = (int)((K - KO) / NB);
            if ((e = cudaEventRecord(G->ev_diag, s)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(G->inv_stream, G->ev_diag, 0)) != cudaSuccess) return e;
            k_inv_step<<<inv_step_blocks(j), 128, 0, G->inv_stream>>>(LU, n, KO, j, G->dinv, D4, G->super_tmp,
                                                                      (unsigned*)(G->super_tmp + kInvScratch));
        }
        const int64_t K1 = K + b, rest = KE - K1;
        if (rest <= 0) break;
        if (K > KO) {  // the previous step's update of the rest of the block
            if ((e = cudaStreamWaitEvent(s, G->ev_rest, 0)) != cudaSuccess) return e;
        }
        const unsigned g = (unsigned)((rest + CS_R - 1) / CS_R + (rest + RS_C - 1) / RS_C);
        k_colrow_solve<<<g, 256, CR_FULL_SMEM, s>>>(LU, n, G->dinv, K1, KE, K1, KE, K, b);
        if (rest > NB) {  // beyond the next diagonal block
            if ((e = cudaEventRecord(G->ev_solve, s)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(G->rest_stream, G->ev_solve, 0)) != cudaSuccess) return e;
            dim3 gg((unsigned)((rest + GS_R - 1) / GS_R), (unsigned)((rest + GS_C - 1) / GS_C));
            k_gemm_sub<<<gg, 128, 0, G->rest_stream>>>(LU, n, K1, KE, K1, KE, K, b);
            if ((e = cudaEventRecord(G->ev_rest, G->rest_stream)) != cudaSuccess) return e;
        }
    }
    if (inv) {
        if ((e = cudaEventRecord(G->ev_inv, G->inv_stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(s, G->ev_inv, 0)) != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// bytes of the split operands: two of n rows (panel columns and rows), two of SB rows for the
// products that meet the next diagonal block and two for the diagonal block's inverses, each SB
// halves long
size_t tc_bytes_for(int64_t n) { return 2 * tc_operand_bytes(n, SB) + 4 * tc_operand_bytes(SB, SB); }

cudaError_t factor_body(LuGraphs* G, float* LU, int64_t n, int* bad, cudaStream_t main, cudaStream_t panel) {
    cudaError_t e;
    // A21 / L21 rows, A12 / U12 columns (all of them, and the SB that meet the next diagonal
    // block), L11^{-1} rows, U11^{-1} columns
    TcOperand rowsA, colsB, nearA, nearB, invA, invB;
    char* mem = (char*)G->tc_mem;
    for (TcOperand* op : {&rowsA, &colsB}) {
        tc_operand_bind(*op, mem, n, SB);
        mem += tc_operand_bytes(n, SB);
    }
    for (TcOperand* op : {&nearA, &nearB, &invA, &invB}) {
        tc_operand_bind(*op, mem, SB, SB);
        mem += tc_operand_bytes(SB, SB);
    }
    const int sms = tc_num_sms();
    // first diagonal block
    if ((e = cudaEventRecord(G->ev_update, main)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(panel, G->ev_update, 0)) != cudaSuccess) return e;
    if ((e = factor_diag_block(G, LU, n, bad, 0, std::min<int64_t>(SB, n), panel)) != cudaSuccess) return e;
    for (int64_t KO = 0; KO < n; KO += SB) {
        const int64_t KE = std::min<int64_t>(KO + SB, n);
        const int64_t rows = n - KE, KE2 = std::min<int64_t>(KE + SB, n), w2 = KE2 - KE, far = rows - w2;
        float* A21 = LU + KO * n + KE;  // rows KE.., columns KO..KE (ld n)
        float* A12 = LU + KE * n + KO;  // rows KO..KE, columns KE.. (ld n)
        float* A22 = LU + KE * n + KE;
        // operand rows: A21's rows (K along its columns), U11^{-1}'s columns, L11^{-1}'s rows, A12's
        // columns.  The strips that meet the next diagonal block (A21 rows KE..KE2, A12 columns
        // KE..KE2) are final once the previous panel's update is queued: split them beside this
        // diagonal block, which does not touch them.
        if (KE < n) {
            if ((e = tc_split(A21, 1, n, w2, SB, nearA, bad, main)) != cudaSuccess) return e;
            if ((e = tc_split(A12, n, 1, w2, SB, nearB, bad, main)) != cudaSuccess) return e;
        }
        // this diagonal block factored and inverted (the main stream has finished the rest of
        // the previous update)
        if ((e = cudaEventRecord(G->ev_panel, panel)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(main, G->ev_panel, 0)) != cudaSuccess) return e;
        if (KE >= n) break;  // a panel that ends short of n is the last one, so KE - KO == SB below
        const float* Li = G->dinv4 + (KO / SB) * 2 * SB * SB;
        const float* Ui = Li + SB * SB;
        // the next diagonal block: L21 rows KE..KE2 on the main stream and U12 columns KE..KE2 on
        // the in-block update stream (idle between two diagonal blocks) side by side, each with its
        // inverse's split before and its own split after, then its update
        if ((e = cudaEventRecord(G->ev_fork, main)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(G->rest_stream, G->ev_fork, 0)) != cudaSuccess) return e;
        if ((e = tc_split(Ui, SB, 1, SB, SB, invB, bad, main)) != cudaSuccess) return e;
        if ((e = tc_split(Li, 1, SB, SB, SB, invA, bad, G->rest_stream)) != cudaSuccess) return e;
        if ((e = tc_gemm(nearA, w2, invB, SB, 1.f, 0.f, A21, n, sms, bad, main)) != cudaSuccess) return e;
        if ((e = tc_gemm(invA, SB, nearB, w2, 1.f, 0.f, A12, n, sms, bad, G->rest_stream)) != cudaSuccess) return e;
        if ((e = tc_split(A21, 1, n, w2, SB, nearA, bad, main)) != cudaSuccess) return e;
        if ((e = tc_split(A12, n, 1, w2, SB, nearB, bad, G->rest_stream)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(G->ev_join, G->rest_stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(main, G->ev_join, 0)) != cudaSuccess) return e;
        if ((e = tc_gemm(nearA, w2, nearB, w2, -1.f, 1.f, A22, n, sms, bad, main)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(G->ev_update, main)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(panel, G->ev_update, 0)) != cudaSuccess) return e;
        if ((e = factor_diag_block(G, LU, n, bad, KE, KE2, panel)) != cudaSuccess) return e;
        if (far <= 0) continue;
        // beside it: the rest of L21 and U12, then every other part of the update
        const int rest_sms = sms - kPanelSms;
        if ((e = tc_split(A21 + w2, 1, n, far, SB, rowsA, bad, main)) != cudaSuccess) return e;
        if ((e = tc_gemm(rowsA, far, invB, SB, 1.f, 0.f, A21 + w2, n, rest_sms, bad, main)) != cudaSuccess) return e;
        if ((e = tc_split(A12 + w2 * n, n, 1, far, SB, colsB, bad, main)) != cudaSuccess) return e;
        if ((e = tc_gemm(invA, SB, colsB, far, 1.f, 0.f, A12 + w2 * n, n, rest_sms, bad, main)) != cudaSuccess)
            return e;
        if ((e = tc_split(A21, 1, n, rows, SB, rowsA, bad, main)) != cudaSuccess) return e;
        if ((e = tc_split(A12, n, 1, rows, SB, colsB, bad, main)) != cudaSuccess) return e;
        // below the next diagonal block in its columns, then every column right of it
        if ((e = tc_gemm(tc_rows(rowsA, w2), far, colsB, w2, -1.f, 1.f, A22 + w2, n, rest_sms, bad, main)) !=
            cudaSuccess)
            return e;
        if ((e = tc_gemm(rowsA, rows, tc_rows(colsB, w2), far, -1.f, 1.f, A22 + w2 * n, n, rest_sms, bad, main)) !=
            cudaSuccess)
            return e;
    }
    return cudaGetLastError();
}

// Blocked forward and backward substitution with the diagonal-block inverses, two skinny
// products per block and direction and no copies: forward, Y_K = inv(L_KK) X_K and
// X_below -= L_below,K Y_K; backward, X_K = inv(U_KK) Y_K and Y_above -= U_above,K X_K.
// X (n x k, ld n) ends with the solution; Y is an n x k scratch array.  The first nsup
// SB-column blocks use their combined inverses (Dinv4), so a pass takes an eighth of the
// dependent steps there; the rest of the matrix goes by 128-column blocks.
cudaError_t solve_body(const float* LU, const float* Dinv, const float* Dinv4, int64_t nsup, int64_t n, float* X,
                       float* Y, int k, const SkinnySplit* sp, cudaStream_t s) {
    cudaError_t e;
    const int64_t nblk = (n + NB - 1) / NB, blk0 = nsup * (SB / NB);
    auto fwd = [&](int64_t K, int64_t b, const float* Li, int64_t ldi) -> cudaError_t {
        cudaError_t ee = skinny(Li, ldi, X + K, n, Y + K, n, b, b, k, 1.f, false, s, sp);
        if (ee != cudaSuccess) return ee;
        return skinny(LU + K * n + K + b, n, Y + K, n, X + K + b, n, n - K - b, b, k, -1.f, true, s, sp);
    };
    auto bwd = [&](int64_t K, int64_t b, const float* Ui, int64_t ldi) -> cudaError_t {
        cudaError_t ee = skinny(Ui, ldi, Y + K, n, X + K, n, b, b, k, 1.f, false, s, sp);
        if (ee != cudaSuccess) return ee;
        return skinny(LU + K * n, n, X + K, n, Y, n, K, b, k, -1.f, true, s, sp);
    };
    for (int64_t sb = 0; sb < nsup; sb++)
        if ((e = fwd(sb * SB, SB, Dinv4 + sb * 2 * SB * SB, SB)) != cudaSuccess) return e;
    for (int64_t blk = blk0; blk < nblk; blk++) {
        const int64_t K = blk * NB;
        if ((e = fwd(K, std::min<int64_t>(NB, n - K), Dinv + blk * 2 * NB * NB, NB)) != cudaSuccess) return e;
    }
    for (int64_t blk = nblk - 1; blk >= blk0; blk--) {
        const int64_t K = blk * NB;
        if ((e = bwd(K, std::min<int64_t>(NB, n - K), Dinv + blk * 2 * NB * NB + NB * NB, NB)) != cudaSuccess)
            return e;
    }
    for (int64_t sb = nsup - 1; sb >= 0; sb--)
        if ((e = bwd(sb * SB, SB, Dinv4 + sb * 2 * SB * SB + SB * SB, SB)) != cudaSuccess) return e;
    return cudaGetLastError();
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
    if (panel_stream) cudaStreamDestroy(panel_stream);
    if (inv_stream) cudaStreamDestroy(inv_stream);
    if (rest_stream) cudaStreamDestroy(rest_stream);
    for (cudaEvent_t ev : {ev_update, ev_panel, ev_diag, ev_inv, ev_solve, ev_rest, ev_fork, ev_join})
        if (ev) cudaEventDestroy(ev);
    panel_stream = inv_stream = rest_stream = nullptr;
    ev_update = ev_panel = ev_diag = ev_inv = ev_solve = ev_rest = ev_fork = ev_join = nullptr;
    if (dinv) cudaFree(dinv);
    if (tmp) cudaFree(tmp);
    if (dinv4) cudaFree(dinv4);
    if (super_tmp) cudaFree(super_tmp);
    if (split_ws) cudaFree(split_ws);
    if (split_cnt) cudaFree(split_cnt);
    split_ws = nullptr;
    split_cnt = nullptr;
    if (tc_mem) cudaFree(tc_mem);
    tc_mem = nullptr;
    tc_bytes = 0;
    dinv4 = super_tmp = nullptr;
    super_n = super_cap = 0;
    solve = nullptr;
    dinv = tmp = nullptr;
    tmp_floats = 0;
    solve_X = nullptr;
    solve_k = 0;
    factor_n = 0;
}

size_t lu_factor_bytes(int64_t n) {
    const size_t nb = (size_t)((n + NB - 1) / NB), nsup = (size_t)(n / SB);
    return sizeof(float) * (nb * 2 * NB * NB + nsup * 2 * SB * SB + (size_t)(kInvScratch + kInvCounters) + kSkinnyWsFloats) +
           tc_bytes_for(n) + sizeof(unsigned) * kSkinnyCounters + 4 * 256;
}

// Launched directly (not from a graph): a geometry is factored once, and its launches are
// each longer than their host-side cost, so a captured graph would only add the capture and
// instantiation to every new geometry.
cudaError_t lu_factor_fp32(LuGraphs* G, float* LU, int64_t n, int* bad, cudaStream_t s) {
    set_attrs();
    cudaError_t e;
    const int64_t nsup = n / SB;
    if (G->factor_n != n || !G->dinv || G->super_cap != nsup) {
        if (G->solve) cudaGraphExecDestroy(G->solve);  // it holds the old inverses
        G->solve = nullptr;
        if (G->dinv) cudaFree(G->dinv);
        if (G->dinv4) cudaFree(G->dinv4);
        if (G->super_tmp) cudaFree(G->super_tmp);
        G->dinv = G->dinv4 = G->super_tmp = nullptr;
        G->super_cap = 0;
        G->factor_n = 0;
        const size_t nb = (size_t)((n + NB - 1) / NB);
        if ((e = cudaMalloc(&G->dinv, sizeof(float) * nb * 2 * NB * NB)) != cudaSuccess) return e;
        if (nsup > 0) {
            if ((e = cudaMalloc(&G->dinv4, sizeof(float) * nsup * 2 * SB * SB)) != cudaSuccess) return e;
            if ((e = cudaMalloc(&G->super_tmp, sizeof(float) * (kInvScratch + kInvCounters))) != cudaSuccess) return e;
            if ((e = cudaMemset(G->super_tmp + kInvScratch, 0, sizeof(float) * kInvCounters)) != cudaSuccess) return e;
        }
        G->super_cap = nsup;
        G->factor_n = n;
    }
    const size_t tcb = tc_bytes_for(n);
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
        if ((e = cudaStreamCreateWithPriority(&G->inv_stream, cudaStreamNonBlocking, greatest)) != cudaSuccess)
            return e;
        if ((e = cudaStreamCreateWithPriority(&G->rest_stream, cudaStreamNonBlocking, greatest)) != cudaSuccess)
            return e;
        for (cudaEvent_t* ev : {&G->ev_update, &G->ev_panel, &G->ev_diag, &G->ev_inv, &G->ev_solve, &G->ev_rest,
                                &G->ev_fork, &G->ev_join})
            if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess) return e;
    }
    ProfScope ps(Prof::LU_FACTOR, s);
    if ((e = factor_body(G, LU, n, bad, s, G->panel_stream)) != cudaSuccess) return e;
    G->super_n = nsup > 0 ? n : 0;
    return cudaSuccess;
}

// Lockstep factorization of m matrices: blocked right-looking LU by outer panels of
// outer_width() columns, each step taken for every matrix at once.  Block step K is one
// launch of the diagonal kernel with one thread block per matrix that still has a block at K,
// then one launch each of the column solve, the in-panel row solve and the in-panel update
// over all matrices; after an outer panel, the U rows right of it by blocked forward
// substitution (two launches per inner block), then the rank-OB update of each matrix on the
// tensor cores.  The work items of every launch are planned on the host and uploaded once.
// No look-ahead stream: the diagonal blocks of all matrices run side by side instead.
// Outer panel width 512 columns: its rank-128 panel updates run in FP32 on the CUDA cores and
// its rank-512 updates on the tensor cores; on the 64-wing batch 512 columns measured 220 ms
// against 269 ms for 1,024 (256: 224 ms; 2,048: 379 ms).
constexpr int64_t OB_BATCHED = 4 * NB;
cudaError_t lu_factor_batched(LuGraphs* const* Gs, float* const* LUs, const int64_t* ns, int* const* bads, int m,
                              cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    set_attrs();
    cudaError_t e;
    std::vector<LuBatchMesh> desc(m);
    int64_t nmax = 0;
    for (int q = 0; q < m; q++) {
        LuGraphs* G = Gs[q];
        const int64_t n = ns[q];
        G->super_n = 0;  // no combined inverses for these factors: substitute by 128 columns
        if (G->solve) cudaGraphExecDestroy(G->solve);
        G->solve = nullptr;
        if (G->factor_n != n || !G->dinv) {
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
    const int64_t OB = OB_BATCHED;
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
    void* tcm = nullptr;
    const size_t opb = tc_operand_bytes(nmax, OB);
    if ((e = cudaMallocAsync((void**)&ddesc, sizeof(LuBatchMesh) * m, s)) != cudaSuccess) return e;
    struct Free {
        void** p[3];
        cudaStream_t s;
        ~Free() {
            for (void** q : p)
                if (*q) cudaFreeAsync(*q, s);
        }
    } fr{{(void**)&ddesc, (void**)&ditems, &tcm}, s};
    if ((e = cudaMallocAsync((void**)&ditems, sizeof(int) * std::max<size_t>(1, items.size()), s)) != cudaSuccess)
        return e;
    if ((e = cudaMallocAsync(&tcm, 2 * opb, s)) != cudaSuccess) return e;
    TcOperand tA, tB;  // one pair for every matrix: the rank updates follow each other on s
    tc_operand_bind(tA, tcm, nmax, OB);
    tc_operand_bind(tB, (char*)tcm + opb, nmax, OB);
    const int sms = tc_num_sms();
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
                case COLS: k_col_solve_batched<<<g, 256, CS_SMEM, s>>>(ddesc, it); break;
                case ROWS: k_row_solve_batched<<<g, 256, RS_SMEM, s>>>(ddesc, it); break;
                case GEMM: k_gemm_sub_batched<<<g, 128, 0, s>>>(ddesc, it); break;
                default: {
                    const int64_t n = ns[st.q], rows = n - st.KE;
                    float* LU = LUs[st.q];
                    e = tc_split(LU + st.KO * n + st.KE, 1, n, rows, OB, tA, bads[st.q], s);
                    if (e == cudaSuccess) e = tc_split(LU + st.KE * n + st.KO, n, 1, rows, OB, tB, bads[st.q], s);
                    if (e == cudaSuccess)
                        e = tc_gemm(tA, rows, tB, rows, -1.f, 1.f, LU + st.KE * n + st.KE, n, sms, bads[st.q], s);
                }
            }
            if (e == cudaSuccess) e = cudaGetLastError();
        }
    }
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
    // The substitution plan reads which systems are active from dact, so one graph of its launches
    // serves every pass; it is destroyed before the plan's buffers are freed.
    struct SubstGraph {
        cudaGraphExec_t exec = nullptr;
        ~SubstGraph() {
            if (exec) cudaGraphExecDestroy(exec);
        }
    } sg;
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
            if (!sg.exec) {  // captured on the first pass, replayed on every later one
                e = capture(s, &sg.exec, [&] {
                    for (const Step& stp : plan) {
                        const int* it = ditems + stp.off * LB_ITEM;
                        if (kmax <= 8)
                            subst_launch<8>(stp.kind, (unsigned)stp.cnt, ddesc, it, dact, stp.dir, s);
                        else if (kmax <= 16)
                            subst_launch<16>(stp.kind, (unsigned)stp.cnt, ddesc, it, dact, stp.dir, s);
                        else
                            subst_launch<32>(stp.kind, (unsigned)stp.cnt, ddesc, it, dact, stp.dir, s);
                    }
                    return cudaGetLastError();
                });
                if (e != cudaSuccess) return e;
            }
            if ((e = cudaGraphLaunch(sg.exec, s)) != cudaSuccess) return e;
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

// X (n x k, ld n) <- U^{-1} L^{-1} X
cudaError_t lu_solve_fp32(LuGraphs* G, const float* LU, int64_t n, float* X, int k, cudaStream_t s) {
    cudaError_t e;
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
        if (!G->split_ws) {
            if ((e = cudaMalloc(&G->split_ws, sizeof(float) * kSkinnyWsFloats)) != cudaSuccess) return e;
            if ((e = cudaMalloc(&G->split_cnt, sizeof(unsigned) * kSkinnyCounters)) != cudaSuccess) return e;
            if ((e = cudaMemset(G->split_cnt, 0, sizeof(unsigned) * kSkinnyCounters)) != cudaSuccess) return e;
        }
        const int64_t nsup = (G->super_n == n && G->dinv4) ? n / SB : 0;
        SkinnySplit sp;
        sp.ws = G->split_ws;
        sp.cnt = G->split_cnt;
        e = capture(s, &G->solve,
                    [&] { return solve_body(LU, G->dinv, G->dinv4, nsup, n, X, G->tmp, k, &sp, s); });
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

cudaError_t lu_invert_fp32(LuGraphs* G, const float* LU, int64_t n, float* Ainv, cudaStream_t s) {
    k_identity<<<nb256(n * n), 256, 0, s>>>(Ainv, n);
    cudaError_t e = lu_solve_fp32(G, LU, n, Ainv, (int)n, s);
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

cudaError_t solve_lu_refined(LuGraphs* G, const float* A32, const float* Alo, const float* LU, int64_t n, int k,
                             const double* rhs, double* x, void* work, double tol, int max_steps, SolveStats* st,
                             cudaStream_t s, const float* Ainv) {
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
            if ((e = skinny(Ainv, n, d32, n, e32, n, n, n, k, 1.f, false, s)) != cudaSuccess) return e;
            k_addf<<<nb256(kn), 256, 0, s>>>(x, e32, kn);
        } else {
            if ((e = lu_solve_fp32(G, LU, n, d32, k, s)) != cudaSuccess) return e;
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
