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

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "assemble.h"

namespace {

constexpr int NB = 128;   // panel width
constexpr int P = NB + 1; // padded smem pitch (no bank conflicts on row access)

// In-place LU (unit lower L, upper U) of the b x b block at A + K*n + K, then the
// inverses of both triangles into Dinv (L11^{-1} then U11^{-1}, column-major,
// ld NB).  Thread t owns row t during the factorization and column t during the
// inversions; one cheap 128-thread barrier per factorization step.
__global__ void __launch_bounds__(NB) k_lu_diag(float* __restrict__ A, int64_t n, int64_t K, int b,
                                                float* __restrict__ Dinv, int* bad) {
    extern __shared__ float sm[];
    float* S = sm;           // S[r*P + c]
    float* Z = sm + NB * P;  // Z[c*P + i]
    const int t = threadIdx.x;
    for (int c = 0; c < b; c++)
        if (t < b) S[t * P + c] = A[(K + c) * n + K + t];
    __syncthreads();
    for (int j = 0; j < b; j++) {
        float piv = S[j * P + j];
        if (piv == 0.f) {
            if (t == 0) atomicExch(bad, 1);
            piv = 1.f;
        }
        if (t > j && t < b) {
            float l = S[t * P + j] / piv;
            S[t * P + j] = l;
            int c = j + 1;
            for (; c + 3 < b; c += 4) {
                float u0 = S[j * P + c], u1 = S[j * P + c + 1], u2 = S[j * P + c + 2], u3 = S[j * P + c + 3];
                S[t * P + c] = __fmaf_rn(-l, u0, S[t * P + c]);
                S[t * P + c + 1] = __fmaf_rn(-l, u1, S[t * P + c + 1]);
                S[t * P + c + 2] = __fmaf_rn(-l, u2, S[t * P + c + 2]);
                S[t * P + c + 3] = __fmaf_rn(-l, u3, S[t * P + c + 3]);
            }
            for (; c < b; c++) S[t * P + c] = __fmaf_rn(-l, S[j * P + c], S[t * P + c]);
        }
        __syncthreads();
    }
    for (int c = 0; c < b; c++)
        if (t < b) A[(K + c) * n + K + t] = S[t * P + c];
    float* Li = Dinv + (K / NB) * 2 * NB * NB;
    float* Ui = Li + NB * NB;
    if (t < b) {
        for (int i = 0; i < b; i++) {  // L z = e_t (unit lower)
            float s0 = i == t ? 1.f : 0.f, s1 = 0.f;
            int j = t;
            for (; j + 1 < i; j += 2) {
                s0 = __fmaf_rn(-S[i * P + j], Z[t * P + j], s0);
                s1 = __fmaf_rn(-S[i * P + j + 1], Z[t * P + j + 1], s1);
            }
            if (j < i) s0 = __fmaf_rn(-S[i * P + j], Z[t * P + j], s0);
            Z[t * P + i] = i < t ? 0.f : s0 + s1;
        }
        for (int i = 0; i < b; i++) Li[t * NB + i] = Z[t * P + i];
        for (int i = b - 1; i >= 0; i--) {  // U z = e_t
            float s0 = i == t ? 1.f : 0.f, s1 = 0.f;
            if (i <= t) {
                int j = i + 1;
                for (; j + 1 <= t; j += 2) {
                    s0 = __fmaf_rn(-S[i * P + j], Z[t * P + j], s0);
                    s1 = __fmaf_rn(-S[i * P + j + 1], Z[t * P + j + 1], s1);
                }
                if (j <= t) s0 = __fmaf_rn(-S[i * P + j], Z[t * P + j], s0);
            }
            Z[t * P + i] = i > t ? 0.f : (s0 + s1) / S[i * P + i];
        }
        for (int i = 0; i < b; i++) Ui[t * NB + i] = Z[t * P + i];
    }
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

bool g_attr_set = false;
void set_attrs() {
    if (g_attr_set) return;
    cudaFuncSetAttribute(k_lu_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * NB * P * 4);
    g_attr_set = true;
}

cublasComputeType_t lu_compute() {
    const char* e = std::getenv("CPG_LU_GEMM");
    if (e && std::string(e) == "sgemm") return CUBLAS_COMPUTE_32F;
    return CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
}

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

cudaError_t factor_body(cublasHandle_t h, float* LU, float* Dinv, float* W, int64_t n, int* bad, cudaStream_t s) {
    const float one = 1.f, mone = -1.f, zero = 0.f;
    cublasComputeType_t ct = lu_compute();
    for (int64_t K = 0; K < n; K += NB) {
        int b = (int)std::min<int64_t>(NB, n - K);
        const float* Li = Dinv + (K / NB) * 2 * NB * NB;
        const float* Ui = Li + NB * NB;
        k_lu_diag<<<1, NB, 2 * NB * P * 4, s>>>(LU, n, K, b, Dinv, bad);
        int64_t rest = n - K - b;
        if (rest <= 0) continue;
        // L21 = A21 U11^{-1} and U12 = L11^{-1} A12 as GEMMs into W, copied back
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)rest, b, b, &one, LU + K * n + K + b, (int)n, Ui, NB, &zero,
                        W, (int)rest) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        cudaError_t e = cudaMemcpy2DAsync(LU + K * n + K + b, n * sizeof(float), W, rest * sizeof(float),
                                          rest * sizeof(float), b, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, b, (int)rest, b, &one, Li, NB, LU + (K + b) * n + K, (int)n,
                        &zero, W, b) != CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        e = cudaMemcpy2DAsync(LU + (K + b) * n + K, n * sizeof(float), W, b * sizeof(float), b * sizeof(float), rest,
                              cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        cublasStatus_t st = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)rest, (int)rest, b, &mone,
                                         LU + K * n + K + b, CUDA_R_32F, (int)n, LU + (K + b) * n + K, CUDA_R_32F,
                                         (int)n, &one, LU + (K + b) * n + K + b, CUDA_R_32F, (int)n, ct,
                                         CUBLAS_GEMM_DEFAULT);
        if (st != CUBLAS_STATUS_SUCCESS) return cudaErrorUnknown;
    }
    return cudaGetLastError();
}

// Blocked forward and backward substitution with the diagonal-block inverses:
// per block, T = inv(D_KK) x_K (small GEMM), x_K <- T, then the rows block K feeds
// are updated by one GEMM.
cudaError_t solve_body(cublasHandle_t h, const float* LU, const float* Dinv, int64_t n, float* X, float* T, int k,
                       cudaStream_t s) {
    const float one = 1.f, mone = -1.f, zero = 0.f;
    const int64_t nblk = (n + NB - 1) / NB;
    for (int64_t q = 0; q < 2 * nblk; q++) {
        bool fwd = q < nblk;
        int64_t blk = fwd ? q : 2 * nblk - 1 - q;
        int64_t K = blk * NB;
        int b = (int)std::min<int64_t>(NB, n - K);
        const float* Di = Dinv + blk * 2 * NB * NB + (fwd ? 0 : NB * NB);
        if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, b, k, b, &one, Di, NB, X + K, (int)n, &zero, T, b) !=
            CUBLAS_STATUS_SUCCESS)
            return cudaErrorUnknown;
        cudaError_t e = cudaMemcpy2DAsync(X + K, n * sizeof(float), T, b * sizeof(float), b * sizeof(float), k,
                                          cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        if (fwd) {
            int64_t rest = n - K - b;
            if (rest > 0 && cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)rest, k, b, &mone, LU + K * n + K + b,
                                        (int)n, T, b, &one, X + K + b, (int)n) != CUBLAS_STATUS_SUCCESS)
                return cudaErrorUnknown;
        } else if (K > 0 && cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)K, k, b, &mone, LU + K * n, (int)n, T, b,
                                        &one, X, (int)n) != CUBLAS_STATUS_SUCCESS) {
            return cudaErrorUnknown;
        }
    }
    return cudaGetLastError();
}

// Capture body() on s into a graph (no profiler events inside the capture).
template <class F>
cudaError_t capture(cudaStream_t s, cudaGraphExec_t* out, F body) {
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
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return e;
}

}  // namespace

void LuGraphs::release() {
    if (factor) cudaGraphExecDestroy(factor);
    if (solve) cudaGraphExecDestroy(solve);
    if (workspace) cudaFree(workspace);
    if (dinv) cudaFree(dinv);
    if (panel) cudaFree(panel);
    if (tmp) cudaFree(tmp);
    factor = solve = nullptr;
    workspace = nullptr;
    dinv = panel = tmp = nullptr;
    tmp_floats = 0;
    solve_X = nullptr;
    solve_k = 0;
    factor_LU = nullptr;
}

cudaError_t lu_factor_fp32(void* blas, LuGraphs* G, float* LU, int64_t n, int* bad, cudaStream_t s) {
    set_attrs();
    cublasHandle_t h = (cublasHandle_t)blas;
    cudaError_t e = prepare_blas(h, G, s);
    if (e != cudaSuccess) return e;
    if (!G->factor || G->factor_LU != LU || G->factor_n != n) {
        if (G->factor) cudaGraphExecDestroy(G->factor);
        G->factor = nullptr;
        if (G->dinv) cudaFree(G->dinv);
        if (G->panel) cudaFree(G->panel);
        G->dinv = G->panel = nullptr;
        size_t nb = (size_t)((n + NB - 1) / NB);
        if ((e = cudaMalloc(&G->dinv, sizeof(float) * nb * 2 * NB * NB)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&G->panel, sizeof(float) * (size_t)n * NB)) != cudaSuccess) return e;
        e = capture(s, &G->factor, [&] { return factor_body(h, LU, G->dinv, G->panel, n, bad, s); });
        if (e != cudaSuccess) return e;
        G->factor_LU = LU;
        G->factor_n = n;
    }
    ProfScope ps(Prof::LU_FACTOR, s);
    return cudaGraphLaunch(G->factor, s);
}

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
        if (G->tmp_floats < (size_t)NB * k) {
            if (G->tmp) cudaFree(G->tmp);
            G->tmp = nullptr;
            if ((e = cudaMalloc(&G->tmp, sizeof(float) * NB * k)) != cudaSuccess) return e;
            G->tmp_floats = (size_t)NB * k;
        }
        e = capture(s, &G->solve, [&] { return solve_body(h, LU, G->dinv, n, X, G->tmp, k, s); });
        if (e != cudaSuccess) return e;
        G->solve_X = X;
        G->solve_k = k;
        G->solve_LU = LU;
    }
    ProfScope ps(Prof::LU_SOLVE, s);
    return cudaGraphLaunch(G->solve, s);
}

size_t solve_lu_work_bytes(int64_t n, int k) {
    size_t kn = (size_t)k * n;
    return sizeof(double) * (2 * kn + 2 * (size_t)k * 64 + 2 * (size_t)k) + sizeof(float) * kn +
           sizeof(double) * (size_t)residual_chunks(n) * 17 * (size_t)n + 64 * 1024;
}

cudaError_t solve_lu_refined(void* blas, LuGraphs* G, const float* A32, const float* Alo, const float* LU, int64_t n,
                             int k, const double* rhs, double* x, void* work, double tol, int max_steps,
                             SolveStats* st, cudaStream_t s) {
    char* p = (char*)work;
    auto take = [&](size_t bytes) {
        char* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    const size_t kn = (size_t)k * n;
    double* r64 = (double*)take(sizeof(double) * kn);
    float* d32 = (float*)take(sizeof(float) * kn);
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
        if ((e = lu_solve_fp32(blas, G, LU, n, d32, k, s)) != cudaSuccess) return e;
        k_addf<<<nb256(kn), 256, 0, s>>>(x, d32, kn);
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
