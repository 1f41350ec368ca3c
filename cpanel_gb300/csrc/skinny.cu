// Skinny products of the block substitutions (see skinny.h).
#include "skinny.h"

#include <algorithm>

namespace {

// ---- skinny products of the block substitutions: C (m x kc) = alpha A (m x K) B (K x kc)
// (+ C when accum), all column-major, kc small.  256 threads per 32 RH rows x KC columns: lane =
// row, warp w takes rows 32 (w % RH) .. and a 32-aligned share of every SK_CH-long chunk of B
// (group w / RH of KG = 8 / RH), which is staged in shared memory column by column (coalesced,
// conflict-free) and read back as float4 broadcasts of four consecutive K indices.  32 loads of
// A in flight per thread, each element of A read once (coalesced along the rows) and used KC
// times; the K groups' partial sums are added in a fixed order.  RH = 2 halves the staging of B
// per row for tall products.  Two blocks per SM: at most 128 registers a thread.
// Split K (gridDim.z > 1): thread block z takes K indices [z kseg, (z + 1) kseg) and writes its
// ROWS x KC partial to ws; the last of a tile's blocks to arrive (counter cnt[tile], which it
// returns to 0) adds the gridDim.z partials in z order and updates C, so the result does not
// depend on the order the blocks ran in.
constexpr int SK_CH = 256;
template <int KC, int RH>
__global__ void __launch_bounds__(256, 2) k_skinny(const float* __restrict__ A, int64_t lda, const float* __restrict__ B,
                                                int64_t ldb, float* __restrict__ C, int64_t ldc, int64_t m,
                                                int64_t K, int kc, float alpha, int accum, int64_t kseg,
                                                float* __restrict__ ws, unsigned* __restrict__ cnt) {
    constexpr int KG = 8 / RH, ROWS = 32 * RH;
    extern __shared__ __align__(16) float dsm[];
    __shared__ int s_last;
    float* Bs = dsm;  // [KC][SK_CH]
    const int t = threadIdx.x, lane = t & 31, w = t >> 5, rh = w % RH, kg = w / RH;
    const int64_t r = (int64_t)blockIdx.x * ROWS + 32 * rh + lane;
    const int c0 = blockIdx.y * KC;
    const int64_t kz0 = (int64_t)blockIdx.z * kseg, kz1 = kz0 + kseg < K ? kz0 + kseg : K;
    float acc[KC];
#pragma unroll
    for (int c = 0; c < KC; c++) acc[c] = 0.f;
    for (int64_t k0 = kz0; k0 < kz1; k0 += SK_CH) {
        const int kch = (int)(kz1 - k0 < SK_CH ? kz1 - k0 : SK_CH);
        const int kst = (kch + 31) & ~31;  // staged length: the compute reads whole groups of 32
        const int kw = ((kch + 32 * KG - 1) / (32 * KG)) * 32, kb = kw * kg;
        float a[32];
        auto load_a = [&](int h) {
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int kk = kb + h + j;
                a[j] = (r < m && kk < kch) ? A[(k0 + kk) * lda + r] : 0.f;
            }
        };
        __syncthreads();
        {  // every load of this thread in flight together, then the stores
            constexpr int PER = SK_CH * KC / 256;
            float v[PER];
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int idx = t + 256 * q, kk = idx % SK_CH, c = idx / SK_CH;
                v[q] = (kk < kch && c0 + c < kc) ? B[(int64_t)(c0 + c) * ldb + k0 + kk] : 0.f;
            }
#pragma unroll
            for (int q = 0; q < PER; q++) {
                const int idx = t + 256 * q;
                if (idx % SK_CH < kst) Bs[idx] = v[q];
            }
        }
        __syncthreads();
        if (r < m) {
            for (int h = 0; h < kw && kb + h < kch; h += 32) {
                load_a(h);
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
#pragma unroll
                    for (int c = 0; c < KC; c++) {
                        const float4 b = *reinterpret_cast<const float4*>(Bs + c * SK_CH + kb + h + j);
                        acc[c] = __fmaf_rn(a[j], b.x, acc[c]);
                        acc[c] = __fmaf_rn(a[j + 1], b.y, acc[c]);
                        acc[c] = __fmaf_rn(a[j + 2], b.z, acc[c]);
                        acc[c] = __fmaf_rn(a[j + 3], b.w, acc[c]);
                    }
                }
            }
        }
    }
    __syncthreads();
    float* red = dsm;  // [KG][ROWS][KC + 1]
#pragma unroll
    for (int c = 0; c < KC; c++) red[(kg * ROWS + 32 * rh + lane) * (KC + 1) + c] = acc[c];
    __syncthreads();
    const int nz = (int)gridDim.z;
    const int64_t tile = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
    if (nz > 1) {
        float* part = ws + (tile * nz + blockIdx.z) * (ROWS * KC);
        for (int idx = t; idx < ROWS * KC; idx += 256) {
            const int rl = idx % ROWS, c = idx / ROWS;
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < KG; q++) s += red[(q * ROWS + rl) * (KC + 1) + c];
            part[idx] = s;
        }
        __threadfence();
        __syncthreads();
        if (t == 0) s_last = atomicAdd(cnt + tile, 1u) == (unsigned)(nz - 1);
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        if (t == 0) cnt[tile] = 0u;
    }
    for (int idx = t; idx < ROWS * KC; idx += 256) {
        const int rl = idx % ROWS, c = idx / ROWS;
        const int64_t rr = (int64_t)blockIdx.x * ROWS + rl;
        if (rr >= m || c0 + c >= kc) continue;
        float s = 0.f;
        if (nz > 1) {
            const float* part = ws + tile * nz * (ROWS * KC) + idx;
            for (int z = 0; z < nz; z++) s += __ldcg(part + z * (ROWS * KC));
        } else {
#pragma unroll
            for (int q = 0; q < KG; q++) s += red[(q * ROWS + rl) * (KC + 1) + c];
        }
        float* p = C + (int64_t)(c0 + c) * ldc + rr;
        *p = accum ? *p + alpha * s : alpha * s;
    }
}
template <int KC>
constexpr int skinny_smem() {  // B staged, then the K groups' partial sums
    return (SK_CH * KC > 256 * (KC + 1) ? SK_CH * KC : 256 * (KC + 1)) * 4;
}
static_assert(skinny_smem<32>() + 16 <= 48 * 1024, "no opt-in shared memory");

// Split rule: K segments of whole rounds of the KG groups (32 KG indices), the count z
// minimising waves x (rounds a block + 1.5 for its staging and epilogue), at most four waves.
template <int KC, int RH>
void skinny_launch(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int64_t m,
                   int64_t K, int kc, float alpha, bool accum, const cpg::SkinnySplit* sp, cudaStream_t s) {
    constexpr int KG = 8 / RH, ROWS = 32 * RH;
    const int64_t gx = (m + ROWS - 1) / ROWS, gy = (kc + KC - 1) / KC, tiles = gx * gy;
    int64_t kseg = K > 0 ? K : 1, z = 1;
    if (sp && sp->ws && K > 0) {
        const int64_t unit = 32 * KG, zmax = std::min<int64_t>((K + unit - 1) / unit, 16);
        double best = -1;
        for (int64_t zz = 1; zz <= zmax; zz++) {
            const int64_t ks = ((K + zz - 1) / zz + unit - 1) / unit * unit;
            if ((K + ks - 1) / ks != zz) continue;  // the segments of a smaller count
            if (zz > 1 && tiles * zz > cpg::kSkinnyMaxBlocks) break;
            const int64_t waves = (tiles * zz + cpg::kSkinnyTarget - 1) / cpg::kSkinnyTarget;
            const double cost = (double)waves * ((double)ks / unit + 1.5);
            if (best < 0 || cost < best - 1e-9) {
                best = cost;
                kseg = ks;
                z = zz;
            }
        }
        if (z > 1 && (size_t)(tiles * z * ROWS * KC) > cpg::kSkinnyWsFloats) z = 1, kseg = K;
    }
    const dim3 g((unsigned)gx, (unsigned)gy, (unsigned)z);
    k_skinny<KC, RH><<<g, 256, skinny_smem<KC>(), s>>>(A, lda, B, ldb, C, ldc, m, K, kc, alpha, accum, kseg,
                                                       z > 1 ? sp->ws : nullptr, z > 1 ? sp->cnt : nullptr);
}
template <int KC>
void skinny_rows(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int64_t m,
                 int64_t K, int kc, float alpha, bool accum, const cpg::SkinnySplit* sp, cudaStream_t s) {
    if (m >= 4096)
        skinny_launch<KC, 2>(A, lda, B, ldb, C, ldc, m, K, kc, alpha, accum, sp, s);
    else
        skinny_launch<KC, 1>(A, lda, B, ldb, C, ldc, m, K, kc, alpha, accum, sp, s);
}

}  // namespace

namespace cpg {

// One kernel per column count: the groups of ceil(kc / 32) are as even as they can be, so no
// multiply-add is spent on a padding column beyond the last group's remainder.
cudaError_t skinny(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int64_t m,
                   int64_t K, int kc, float alpha, bool accum, cudaStream_t s, const SkinnySplit* sp) {
    if (m <= 0 || kc <= 0) return cudaSuccess;
    const int groups = (kc + 31) / 32, kce = (kc + groups - 1) / groups;
    switch (kce) {
#define CPG_SKINNY_CASE(N) \
    case N:                \
        skinny_rows<N>(A, lda, B, ldb, C, ldc, m, K, kc, alpha, accum, sp, s); \
        break;
        CPG_SKINNY_CASE(1) CPG_SKINNY_CASE(2) CPG_SKINNY_CASE(3) CPG_SKINNY_CASE(4) CPG_SKINNY_CASE(5)
        CPG_SKINNY_CASE(6) CPG_SKINNY_CASE(7) CPG_SKINNY_CASE(8) CPG_SKINNY_CASE(9) CPG_SKINNY_CASE(10)
        CPG_SKINNY_CASE(11) CPG_SKINNY_CASE(12) CPG_SKINNY_CASE(13) CPG_SKINNY_CASE(14) CPG_SKINNY_CASE(15)
        CPG_SKINNY_CASE(16) CPG_SKINNY_CASE(17) CPG_SKINNY_CASE(18) CPG_SKINNY_CASE(19) CPG_SKINNY_CASE(20)
        CPG_SKINNY_CASE(21) CPG_SKINNY_CASE(22) CPG_SKINNY_CASE(23) CPG_SKINNY_CASE(24) CPG_SKINNY_CASE(25)
        CPG_SKINNY_CASE(26) CPG_SKINNY_CASE(27) CPG_SKINNY_CASE(28) CPG_SKINNY_CASE(29) CPG_SKINNY_CASE(30)
        CPG_SKINNY_CASE(31) CPG_SKINNY_CASE(32)
#undef CPG_SKINNY_CASE
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace cpg
