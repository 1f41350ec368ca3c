// Tensor-core GEMM of split FP32 operands (tc_gemm.h): TMA loads, tcgen05.mma into tensor
// memory, one persistent CTA per SM.
//
// CTA roles (320 threads):
//   warp 0       TMA producer: draws the CTA's next tile (from a device counter shared by the
//                grid, so that CTAs that start late while other kernels hold SMs take fewer
//                tiles; or round-robin) and hands it to the other warps through a 4-slot ring,
//                then per 64-wide K block one 3-D tensor load of the A tile (hi and lo, 128 rows)
//                and one of the B tile (hi and lo, 256 rows) into a stage;
//   warp 1       allocates 512 tensor-memory columns (two 128 x 256 FP32 accumulators); one
//                thread issues per K block 4 x 3 MMAs (K = 16 each: Ah Bh, Ah Bl, Al Bh) and
//                commits the stage back to the producer, then the accumulator to the epilogue;
//   warps 2-9    epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. (its rows) and one
//                half of the columns, scales and adds into C (column-major, coalesced along
//                the rows of each column).  The accumulator is handed back once its last
//                columns are in registers, so the MMAs of the next tile overlap the C update.
// Shared memory: 2 stages x 96 KB, each tile in the 128-byte swizzled K-major layout that TMA
// writes and the MMA descriptors read (8-row groups 1,024 bytes apart).
// Every wait is bounded (about two seconds of clock cycles); on expiry the kernel records
// the failure, stops issuing work, waits for what it has issued and frees tensor memory.
#include "tc_gemm.h"

#include "assemble.h"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace {

constexpr int BM = 128, BN = 256, BK = cpg::kTcK;
constexpr int STAGES = 2;
constexpr int A_HALF = BM * BK * 2;      // bytes of one A half tile (16 KB)
constexpr int B_HALF = BN * BK * 2;      // 32 KB
constexpr int A_BYTES = 2 * A_HALF;
constexpr int B_BYTES = 2 * B_HALF;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;  // + alignment slack
constexpr int EPI_WARPS = 8;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr uint32_t TMEM_COLS = 2 * BN;
constexpr long long WAIT_CYCLES = 4000000000LL;

// instruction descriptor of tcgen05.mma kind::f16: D F32 (bits 4-5 = 1), A and B F16 (bits
// 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading byte offset 16 (unused by the
// swizzled K-major layout), stride byte offset 1,024 (8 rows of 128 bytes), the fixed 0b001 at
// bits 46-48, base offset 0 (tiles are 1,024-byte aligned), 128-byte swizzle (2 at bits 61-63)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(16 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase of the given parity.  Gives up when the CTA has been told to stop
// (watch_abort) or after WAIT_CYCLES, then records the failure and tells the CTA to stop.
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                                       bool watch_abort) {
    const long long t0 = clock64();
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        if (watch_abort && *abort_flag) return false;
        if (clock64() - t0 > WAIT_CYCLES) {
            *abort_flag = 1;
            if (err) atomicExch(err, 1);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(dst),
        "l"(map), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(cols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
            d),
        "l"(a), "l"(b), "r"(IDESC), "r"(acc)
        : "memory");
}
// arrives on bar once every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

struct GemmArgs {
    int64_t m, n, ldc;
    int kblocks, tiles_m, tiles;
    float alpha, beta;
    float* C;
    const float* isa;
    const float* isb;
    int* err;
    int* counter;  // next tile to hand out (zero at launch), or null: CTA b takes tiles b, b + grid, ...
};

constexpr int RING = 4;  // tiles handed from the producer to the MMA and epilogue warps

__global__ void __launch_bounds__(THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], accf_bar[2], acce_bar[2], fin_bar;
    __shared__ __align__(8) uint64_t tfull_bar[RING], tempty_bar[RING];
    __shared__ int tile_ring[RING];
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_s;
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int* abort_flag = &abort_s;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(su32(&full_bar[s]), 1);
            mbar_init(su32(&empty_bar[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(su32(&accf_bar[b]), 1);
            mbar_init(su32(&acce_bar[b]), EPI_WARPS);
        }
        mbar_init(su32(&fin_bar), 1);
        for (int q = 0; q < RING; q++) {
            mbar_init(su32(&tfull_bar[q]), 1);
            mbar_init(su32(&tempty_bar[q]), 1 + EPI_WARPS);
        }
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        tmem_alloc(su32(&tmem_base_s), TMEM_COLS);
        tmem_relinquish();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base_s;

    if (warp == 0) {
        if (lane == 0) {  // TMA producer; it also draws the tiles and hands them on through the ring
            int issued = 0;
            for (int j = 0; !*abort_flag; j++) {
                const int slot = j % RING;
                if (!mbar_wait(su32(&tempty_bar[slot]), ((uint32_t)(j / RING) & 1u) ^ 1u, abort_flag, g.err, true))
                    break;
                int t = g.counter ? atomicAdd(g.counter, 1) : blockIdx.x + j * (int)gridDim.x;
                if (t >= g.tiles) t = -1;
                *(volatile int*)&tile_ring[slot] = t;
                mbar_arrive(su32(&tfull_bar[slot]));
                if (t < 0) break;
                const int tm = t % g.tiles_m, tn = t / g.tiles_m;
                for (int kb = 0; kb < g.kblocks; kb++) {
                    const int s = issued % STAGES;
                    const uint32_t ph = (uint32_t)(issued / STAGES) & 1u;
                    if (!mbar_wait(su32(&empty_bar[s]), ph ^ 1u, abort_flag, g.err, true)) break;
                    const uint32_t st = su32(smem + s * STAGE_BYTES);
                    mbar_expect_tx(su32(&full_bar[s]), STAGE_BYTES);
                    tma_load_3d(st, &tmA, su32(&full_bar[s]), kb * BK, tm * BM, 0);
                    tma_load_3d(st + A_BYTES, &tmB, su32(&full_bar[s]), kb * BK, tn * BN, 0);
                    issued++;
                }
            }
            // the loads in flight land before the CTA may exit
            for (int j = issued > STAGES ? issued - STAGES : 0; j < issued; j++)
                mbar_wait(su32(&full_bar[j % STAGES]), (uint32_t)(j / STAGES) & 1u, abort_flag, g.err, false);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            int used = 0;
            for (int tl = 0; !*abort_flag; tl++) {
                const int slot = tl % RING;
                if (!mbar_wait(su32(&tfull_bar[slot]), (uint32_t)(tl / RING) & 1u, abort_flag, g.err, true)) break;
                const int t = *(volatile int*)&tile_ring[slot];
                mbar_arrive(su32(&tempty_bar[slot]));
                if (t < 0) break;
                const int b = tl & 1;
                if (!mbar_wait(su32(&acce_bar[b]), ((uint32_t)(tl >> 1) & 1u) ^ 1u, abort_flag, g.err, true)) break;
                fence_after();
                const uint32_t d = tmem + (uint32_t)(b * BN);
                bool ok = true;
                for (int kb = 0; kb < g.kblocks; kb++, used++) {
                    const int s = used % STAGES;
                    if (!mbar_wait(su32(&full_bar[s]), (uint32_t)(used / STAGES) & 1u, abort_flag, g.err, true)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t sa = su32(smem + s * STAGE_BYTES), sb = sa + A_BYTES;
#pragma unroll
                    for (int kk = 0; kk < BK / 16; kk++) {
                        const uint64_t ah = sdesc(sa + kk * 32), al = sdesc(sa + A_HALF + kk * 32);
                        const uint64_t bh = sdesc(sb + kk * 32), bl = sdesc(sb + B_HALF + kk * 32);
                        mma_f16(d, ah, bh, (kb | kk) != 0);
                        mma_f16(d, ah, bl, 1);
                        mma_f16(d, al, bh, 1);
                    }
                    mma_commit(su32(&empty_bar[s]));
                }
                if (!ok) break;
                mma_commit(su32(&accf_bar[b]));
            }
        }
    } else {  // epilogue
        const int e = warp - 2, q = warp & 3, hc = e >> 2;  // lane quarter, column half
        for (int tl = 0;; tl++) {
            const int slot = tl % RING;
            if (!mbar_wait(su32(&tfull_bar[slot]), (uint32_t)(tl / RING) & 1u, abort_flag, g.err, true)) break;
            const int t = *(volatile int*)&tile_ring[slot];
            __syncwarp();
            if (lane == 0) mbar_arrive(su32(&tempty_bar[slot]));
            if (t < 0) break;
            const int b = tl & 1;
            if (!mbar_wait(su32(&accf_bar[b]), (uint32_t)(tl >> 1) & 1u, abort_flag, g.err, true)) break;
            fence_after();
            const int tm = t % g.tiles_m, tn = t / g.tiles_m;
            const int64_t row = (int64_t)tm * BM + q * 32 + lane;
            const bool live = row < g.m;
            const float rs = live ? g.isa[row] * g.alpha : 0.f;
#pragma unroll 1
            for (int c = 0; c < BN / 2; c += 32) {
                const int cc = hc * (BN / 2) + c;
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + cc), v);
                if (c == BN / 2 - 32) {  // this warp's share of the accumulator is in registers
                    fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(su32(&acce_bar[b]));
                }
                const int64_t col0 = (int64_t)tn * BN + cc;
                if (live) {
                    float* p = g.C + col0 * g.ldc + row;
                    if (g.beta != 0.f) {
                        float old[32];
#pragma unroll
                        for (int j = 0; j < 32; j++)
                            if (col0 + j < g.n) old[j] = p[j * g.ldc];
#pragma unroll
                        for (int j = 0; j < 32; j++)
                            if (col0 + j < g.n) p[j * g.ldc] = g.beta * old[j] + v[j] * (rs * g.isb[col0 + j]);
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; j++)
                            if (col0 + j < g.n) p[j * g.ldc] = v[j] * (rs * g.isb[col0 + j]);
                    }
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {  // every issued MMA has completed before tensor memory is freed
        if (lane == 0) {
            mma_commit(su32(&fin_bar));
            mbar_wait(su32(&fin_bar), 0, abort_flag, g.err, false);
        }
        __syncwarp();
        fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ---- split kernels ----

// 2^e with max * 2^e in [2^13, 2^14); 1 for an all-zero row
__device__ __forceinline__ float row_scale(float mx) {
    if (!(mx > 0.f)) return 1.f;
    int ex;
    frexpf(mx, &ex);  // mx in [2^(ex-1), 2^ex)
    return ldexpf(1.f, 14 - ex);
}

__device__ __forceinline__ void split2(float x, __half& hi, __half& lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

// K-major source: one warp per row (max, then split)
__global__ void k_split_kmajor(const float* __restrict__ src, int64_t rs, int64_t rows, int64_t K, int64_t kp,
                               int64_t rows_cap, __half* __restrict__ out, float* __restrict__ inv, int* err) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= rows) return;
    const float* s = src + r * rs;
    float mx = 0.f;
    bool fin = true;
    for (int64_t k = lane; k < K; k += 32) {
        const float a = fabsf(s[k]);
        fin = fin && isfinite(a);
        mx = fmaxf(mx, a);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    fin = __all_sync(0xffffffffu, fin);
    const float sc = row_scale(mx);
    if (lane == 0) {
        inv[r] = 1.f / sc;
        if (!fin && err) atomicExch(err, 2);
    }
    __half* hi = out + r * kp;
    __half* lo = out + rows_cap * kp + r * kp;
    for (int64_t k = 2 * lane; k < kp; k += 64) {
        const float x0 = k < K ? s[k] * sc : 0.f, x1 = k + 1 < K ? s[k + 1] * sc : 0.f;
        __half h0, l0, h1, l1;
        split2(x0, h0, l0);
        split2(x1, h1, l1);
        *(__half2*)(hi + k) = __halves2half2(h0, h1);
        *(__half2*)(lo + k) = __halves2half2(l0, l1);
    }
}

// column-major source, pass 1: row maxima.  Block 32 rows x 16 K groups, eight loads in flight
// per thread.
__global__ void __launch_bounds__(512) k_rowmax_mmajor(const float* __restrict__ src, int64_t ks, int64_t rows,
                                                       int64_t K, float* __restrict__ scale, float* __restrict__ inv,
                                                       int* err) {
    __shared__ float part[16][32];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    const int rl = threadIdx.x & 31, gi = threadIdx.x >> 5;
    const int64_t r = (int64_t)blockIdx.x * 32 + rl;
    float mx = 0.f;
    bool fin = true;
    if (r < rows)
        for (int64_t k = gi; k < K; k += 16 * 8) {
            float a[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int64_t kk = k + 16 * u;
                a[u] = kk < K ? fabsf(src[kk * ks + r]) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                fin = fin && isfinite(a[u]);
                mx = fmaxf(mx, a[u]);
            }
        }
    part[gi][rl] = mx;
    if (!fin) bad = 1;
    __syncthreads();
    if (gi == 0 && r < rows) {
        for (int q = 1; q < 16; q++) mx = fmaxf(mx, part[q][rl]);
        const float sc = row_scale(mx);
        scale[r] = sc;
        inv[r] = 1.f / sc;
    }
    if (threadIdx.x == 0 && bad && err) atomicExch(err, 2);
}

// column-major source, pass 2: 32 rows x 64 K through shared memory, written K-major
__global__ void k_split_mmajor(const float* __restrict__ src, int64_t ks, int64_t rows, int64_t K, int64_t kp,
                               int64_t rows_cap, const float* __restrict__ scale, __half* __restrict__ out) {
    __shared__ float t[64][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 64;
    const int rl = threadIdx.x & 31, kq = threadIdx.x >> 5;  // 8 K rows per pass
    for (int kk = kq; kk < 64; kk += 8) {
        const int64_t r = r0 + rl, k = k0 + kk;
        t[kk][rl] = (r < rows && k < K) ? src[k * ks + r] : 0.f;
    }
    __syncthreads();
    const int rr = threadIdx.x >> 3, k8 = (threadIdx.x & 7) * 8;  // row, first of 8 K values
    const int64_t r = r0 + rr;
    if (r >= rows) return;
    const float sc = scale[r];
    __align__(16) __half h[8], l[8];
#pragma unroll
    for (int j = 0; j < 8; j++) split2(t[k8 + j][rr] * sc, h[j], l[j]);
    *(uint4*)(out + r * kp + k0 + k8) = *(const uint4*)h;
    *(uint4*)(out + rows_cap * kp + r * kp + k0 + k8) = *(const uint4*)l;
}

// ---- host side ----

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// 3-D map over an operand: (k, row, hi/lo), box 64 x box_rows x 2, 128-byte swizzle; rows past
// `rows` read as zero
bool encode_operand(CUtensorMap* map, const cpg::TcOperand& op, int64_t rows, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[3] = {(cuuint64_t)op.kp, (cuuint64_t)rows, 2};
    cuuint64_t strides[2] = {(cuuint64_t)op.kp * 2, (cuuint64_t)(op.rows_cap * op.kp * 2)};
    cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 2};
    cuuint32_t es[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, (void*)op.data, dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

namespace cpg {

size_t tc_operand_bytes(int64_t rows_cap, int64_t kp) {
    const size_t d = ((size_t)2 * rows_cap * kp * sizeof(__half) + 255) & ~(size_t)255;
    return d + (((size_t)2 * rows_cap * sizeof(float) + 255) & ~(size_t)255);
}

void tc_operand_bind(TcOperand& op, void* mem, int64_t rows_cap, int64_t kp) {
    const size_t d = ((size_t)2 * rows_cap * kp * sizeof(__half) + 255) & ~(size_t)255;
    op.data = (__half*)mem;
    op.inv_scale = (float*)((char*)mem + d);
    op.rows_cap = rows_cap;
    op.kp = kp;
}

cudaError_t tc_split(const float* src, int64_t rs, int64_t ks, int64_t rows, int64_t K, TcOperand& op, int* err,
                     cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    if (rows > op.rows_cap || K > op.kp || op.kp % BK != 0 || (rs != 1 && ks != 1)) return cudaErrorInvalidValue;
    if (ks == 1) {
        const int64_t thr = rows * 32;
        k_split_kmajor<<<(unsigned)((thr + 255) / 256), 256, 0, s>>>(src, rs, rows, K, op.kp, op.rows_cap, op.data,
                                                                     op.inv_scale, err);
    } else {
        float* scale = op.inv_scale + op.rows_cap;  // the second half of the scale area
        k_rowmax_mmajor<<<(unsigned)((rows + 31) / 32), 512, 0, s>>>(src, ks, rows, K, scale, op.inv_scale, err);
        dim3 grid((unsigned)((rows + 31) / 32), (unsigned)(op.kp / BK));
        k_split_mmajor<<<grid, 256, 0, s>>>(src, ks, rows, K, op.kp, op.rows_cap, scale, op.data);
    }
    return cudaGetLastError();
}

int tc_num_sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

cudaError_t tc_gemm(const TcOperand& A, int64_t m, const TcOperand& B, int64_t n, float alpha, float beta, float* C,
                    int64_t ldc, int sm_budget, int* err, cudaStream_t s, int* counter) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    if (A.kp != B.kp || A.kp % BK != 0 || m > A.rows_cap || n > B.rows_cap || ldc < m) return cudaErrorInvalidValue;
    static std::once_flag attr[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::call_once(attr[dev & 63],
                   [] { cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES); });
    CUtensorMap ta, tb;
    if (!encode_operand(&ta, A, m, BM) || !encode_operand(&tb, B, n, BN)) return cudaErrorInvalidValue;
    GemmArgs g;
    g.m = m;
    g.n = n;
    g.ldc = ldc;
    g.kblocks = (int)(A.kp / BK);
    g.tiles_m = (int)((m + BM - 1) / BM);
    const int tiles_n = (int)((n + BN - 1) / BN);
    g.tiles = g.tiles_m * tiles_n;
    g.alpha = alpha;
    g.beta = beta;
    g.C = C;
    g.isa = A.inv_scale;
    g.isb = B.inv_scale;
    g.err = err;
    g.counter = counter;
    const int grid = std::max(1, std::min(g.tiles, sm_budget));
    if (counter) {
        cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
        if (e != cudaSuccess) return e;
    }
    ProfScope ps(Prof::TC_GEMM, s);
    k_tc_gemm<<<grid, THREADS, SMEM_BYTES, s>>>(ta, tb, g);
    return cudaGetLastError();
}

}  // namespace cpg

