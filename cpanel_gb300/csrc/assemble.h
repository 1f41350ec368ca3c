// Launchers of the assembly and influence-operator kernels (assemble.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace cpg {

// Optional device-time accounting per kernel class (CUDA events on the launching
// stream).  Enabled per context; the API entry points install it for the calling
// thread for the duration of a call.
struct Prof {
    enum { ASSEMBLE = 0, WAKE_COLUMNS, MATVEC_FP32, MATVEC_FP64, RESIDUAL, BJ_APPLY, BJ_SETUP, CHTLS, POST,
           VECTOR_OPS, NCLS };
    struct Pair {
        cudaEvent_t a, b;
        int cls;
    };
    std::vector<Pair> pending;
    std::vector<cudaEvent_t> pool;
    double ms[NCLS] = {0};
    long long launches[NCLS] = {0};
    cudaEvent_t get();
    void begin(int cls, cudaStream_t s);
    void end(cudaStream_t s);
    void collect();  // call after the stream has synchronized
    void reset();
    ~Prof();
};
extern thread_local Prof* g_prof;
struct ProfScope {
    cudaStream_t s;
    bool on;
    ProfScope(int cls, cudaStream_t st) : s(st), on(g_prof != nullptr) {
        if (on) g_prof->begin(cls, s);
    }
    ~ProfScope() {
        if (on) g_prof->end(s);
    }
};

cudaError_t launch_assemble_fp64(const double* rec, int64_t n, const double* wrec, const int32_t* widx,
                                 const double* wcoef, int64_t nw, double* A, double* B,
                                 unsigned long long* near_count, cudaStream_t s);
cudaError_t launch_assemble_mixed(const double* rec, const float* frec, int64_t n, const double* wrec,
                                  const int32_t* widx, const double* wcoef, int64_t nw, float* A32, float* Alo,
                                  double* rb, unsigned long long* near_count, cudaStream_t s);
cudaError_t launch_phi_batch(const double* verts, const double* poi, int64_t m, double* src, double* dub, int mode,
                             cudaStream_t s);
cudaError_t launch_v_batch(const double* verts, const double* poi, int64_t m, double* vs, double* vd, cudaStream_t s);
cudaError_t launch_wake_potential_op(const double* wrec, int64_t nw, const double* pts, int64_t np, double* G,
                                     cudaStream_t s);

// solve.cu
struct SolveStats {
    int64_t iters_max = 0, iters_total = 0, refinements = 0;
    double residual_max = 0;
};
// Plain FP64 BiCGSTAB with Jacobi preconditioner and zero initial guess on k
// right-hand sides at once (each column follows Eigen::BiCGSTAB exactly: own
// scalars, own restart and stopping rule).  A: n x n column-major FP64.
// rhs, x: k x n (case-major).  work: device scratch of solve_fp64_work_bytes(n,k).
size_t solve_fp64_work_bytes(int64_t n, int k);
cudaError_t solve_fp64(const double* A, int64_t n, int k, const double* rhs, double* x, void* work,
                       double tol, int64_t max_iters, SolveStats* st, cudaStream_t s);
// Mixed: A = A32 + Alo (two FP32 column-major matrices; Alo is zero in the far
// field).  FP32 BiCGSTAB inner solves on A32 with FP64 inner products, wrapped in
// iterative refinement whose residual b - (A32 + Alo) x is accumulated with exact
// FP32 products (double-float).  Stops at relative residual <= tol_outer for
// every column.
// Block-Jacobi preconditioner on index sets perm[off[b] .. off[b+1]).
struct BlockJacobi {
    const int32_t* perm = nullptr;
    const int32_t* off = nullptr;      // device, nb + 1
    const int64_t* doff = nullptr;     // device, offset of block b's inverse in Dinv
    float* Dinv = nullptr;             // column-major block inverses
    int nb = 0;
    int bsmax = 0;
};
cudaError_t bj_setup(const float* A32, int64_t n, const BlockJacobi& bj, float* work, cudaStream_t s);
size_t solve_mixed_work_bytes(int64_t n, int k);
cudaError_t solve_mixed(const float* A32, const float* Alo, const BlockJacobi* bj, int64_t n, int k, const double* rhs, double* x, void* work,
                        double tol_outer, double tol_inner, int max_outer, int64_t max_inner, SolveStats* st,
                        cudaStream_t s);
// y(k x n) = alpha * M x(k x n) for column-major FP64 M (used for -B sigma).
cudaError_t gemm_fp64_nk(const double* M, int64_t n, int k, const double* x, double* y, double alpha, void* work,
                         cudaStream_t s);

// post.cu
struct PostTables;  // device tables built once per mesh
}  // namespace cpg
