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
    enum { ASSEMBLE = 0, WAKE_COLUMNS, MATVEC_FP32, MATVEC_FP64, RESIDUAL, LU_FACTOR, PARTICLES, CHTLS, POST,
           LU_SOLVE, TC_GEMM, NCLS };
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
// order: mixed_block_order's blocks on the device (2 ints per block: row block, source chunk;
// the costliest first);
// erec: per-panel FP64 edge constants of the near field (E_STRIDE doubles per body panel:
// |s_k|, 1/|s_k|, s_k.m with s_k = v_{k+1} - v_k, rounded as the device rounds them)
cudaError_t launch_assemble_mixed(const double* rec, const float* frec, const double* erec, int64_t n,
                                  const double* wrec, const int32_t* widx, const double* wcoef, int64_t nw,
                                  const int* order, float* A32, float* Alo, double* rb, double* rb_part,
                                  unsigned long long* near_count, cudaStream_t s);
// block schedule of the mixed assembly: blocks sorted by the distance between their row
// and source index ranges (near-field-heavy blocks first)
// cent: target/source centroids (3 doubles, stride cstride), longside (stride lstride), matrix order
void mixed_block_order(int64_t n, const double* cent, int64_t cstride, const double* longside, int64_t lstride,
                       std::vector<int>& out);

// Grouped mixed assembly of many meshes in one persistent launch.  One descriptor per
// mesh (device copy); row0 = first row of the mesh in the group's flattened rows, the
// descriptors sorted by row0.  jchunk must be mixed_chunk(n): the partial sums of the
// right-hand-side basis are then split exactly as in the single-mesh launch, so the
// results are bit-identical to launch_assemble_mixed whatever the schedule.
struct MixedMeshDesc {
    const double* rec;
    const float* frec;
    const double* erec;
    int64_t n, jchunk;
    float* A32;
    float* Alo;
    double* rbp;  // mixed_rb_part_doubles(n, nw): chunk partial sums, then the wake table
    double* rb;   // 3n
    unsigned long long* near_count;  // may be null
    const double* wrec;
    const int32_t* widx;
    const double* wcoef;
    int64_t nw;
    int64_t row0;
};
int64_t mixed_chunk(int64_t n);
// Work queue of a grouped launch: 4 ints per item (mesh, row block, first chunk, chunk
// count), costliest first.  Items whose row and source ranges lie within near_band chunk
// lengths hold one chunk; the others up to chunks_per_item.  Returns the item count.
int64_t group_schedule(const int64_t* n, int m, int chunks_per_item, int near_band, std::vector<int>& items);
// The persistent assembly kernel over the queue (blocks = resident blocks in total;
// next: one device int, cleared here), then the partial-sum reduction and the wake
// columns of every mesh (rows = the group's flattened row count).
cudaError_t launch_assemble_mixed_grouped_core(const MixedMeshDesc* meshes, const int* items, int nitems,
                                               int blocks, int* next, cudaStream_t s);
cudaError_t launch_assemble_mixed_grouped_finish(const MixedMeshDesc* meshes, int m, int64_t rows, int64_t max_nw,
                                                 cudaStream_t s);
int assemble_mixed_grouped_max_blocks_per_sm();
// doubles of rb_part that launch_assemble_mixed needs: the per-chunk partial sums, and
// afterwards the wake influence table (nw x n)
int64_t mixed_rb_part_doubles(int64_t n, int64_t nw);
// Panel-induced velocity (bodyPanel::panelV + wakePanel::panelV) at m points from packed
// records: nb body records followed by nw wake records at rec (R_STRIDE doubles each).
cudaError_t launch_panels_velocity_rec(const double* rec, const double* sigma, const double* mu, int64_t nb,
                                       const double* wmu, int64_t nw, const double* pts, int64_t m, double* vel,
                                       cudaStream_t s);
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
// Refinement residual r = b - (A32 + Alo) x for k right-hand sides (x FP64), with
// the leading products formed exactly in FP32 pairs.  P: residual_chunks(n)*17*n doubles.
int64_t residual_chunks(int64_t n);
cudaError_t residual_df(const float* A32, const float* Alo, int64_t n, int k, const double* x, const double* b,
                        double* r, double* P, cudaStream_t s);
// Measured FP64 FMA throughput of this GPU (TFLOP/s), for roofline reporting.
double measure_fp64_tflops(cudaStream_t s);
// Squared column norms of a k x n case-major FP64 block, copied to host[0..k).
cudaError_t column_norms2(const double* v, int64_t n, int k, double* part, double* dd, double* host, cudaStream_t s);
// The same into dd[0..k) on the device (no copy, no synchronization).
cudaError_t column_norms2_device(const double* v, int64_t n, int k, double* part, double* dd, cudaStream_t s);

// lu.cu: FP32 LU without pivoting (blocked; diagonal blocks on the CUDA cores, panel products
// and trailing updates on the tensor cores) and the refined solve x = A^{-1} b against
// A = A32 + Alo.  The substitutions are captured once into a CUDA graph held in LuGraphs and
// replayed.
struct LuGraphs {
    cudaGraphExec_t solve = nullptr;
    int64_t factor_n = 0;
    const float* solve_LU = nullptr;
    const float* solve_X = nullptr;
    int solve_k = 0;
    cudaStream_t panel_stream = nullptr;  // high-priority stream of the diagonal-block factorizations
    cudaStream_t inv_stream = nullptr;    // and of the diagonal blocks' inverses beside them
    cudaStream_t rest_stream = nullptr;   // and of the in-block updates beside the next diagonal step
    cudaEvent_t ev_update = nullptr, ev_panel = nullptr;  // fork / join between the streams
    cudaEvent_t ev_diag = nullptr, ev_inv = nullptr, ev_solve = nullptr, ev_rest = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // the products between two diagonal blocks
    float* dinv = nullptr;      // inverses of the 128-column diagonal blocks (L then U per block)
    float* tmp = nullptr;       // n x k intermediate of the substitutions
    size_t tmp_floats = 0;
    float* dinv4 = nullptr;     // inverses of the full 1,024-column diagonal blocks (L then U)
    float* super_tmp = nullptr; // tile scratch while one of them is built
    int64_t super_n = 0;        // order they were built for (0: none, the substitutions use dinv)
    int64_t super_cap = 0;      // 1,024-column blocks dinv4 holds
    void* tc_mem = nullptr;     // split FP16 operands of the tensor-core products
    size_t tc_bytes = 0;
    float* split_ws = nullptr;      // partials of the split-K substitution products
    unsigned* split_cnt = nullptr;  // and their per-tile arrival counters
    void release();
};
cudaError_t lu_factor_fp32(LuGraphs* G, float* LU, int64_t n, int* bad, cudaStream_t s);
// device bytes lu_factor_fp32 allocates for an n x n factorization (inverses, operands, scratch)
size_t lu_factor_bytes(int64_t n);
// One matrix of a lockstep factorization (device copy).
struct LuBatchMesh {
    float* LU;
    float* dinv;
    int64_t n;
    int* bad;
};
// The factorization of lu_factor_fp32 for m matrices at once (LUs[q]: n_q x n_q, A32 copied
// in; Gs[q] receives the diagonal-block inverses the substitutions use), every block step
// taken for all matrices in one launch.  Issued on s.
cudaError_t lu_factor_batched(LuGraphs* const* Gs, float* const* LUs, const int64_t* ns, int* const* bads, int m,
                              cudaStream_t s);
// One system of a lockstep refined solve: A = A32 + Alo (n x n), its FP32 factors LU with
// the diagonal-block inverses dinv (from lu_factor_fp32 or lu_factor_batched), k right-hand
// sides rhs (k x n) -> x; work: solve_lu_work_bytes(n, k) bytes.
struct RefineMesh {
    const float* A32;
    const float* Alo;
    const float* LU;
    const float* dinv;
    int64_t n;
    int k;
    const double* rhs;
    double* x;
    void* work;
    cudaStream_t stream;  // this system's own work (null: the driver's stream)
};
// solve_lu_refined for m systems at once: every refinement pass does the forward and
// backward block substitutions of all systems still above tol together (one launch per
// block step and direction for all of them), then each system's exact-product residual.
// Each system stops at relative residual tol (or max_steps passes) as solve_lu_refined does;
// st[q] receives its pass count and final residual.  The substitutions run on s, each
// system's conversions, residual and norms on its own stream (joined and forked by events).
cudaError_t solve_lu_refined_batched(const RefineMesh* ms, int m, double tol, int max_steps, SolveStats* st,
                                     cudaStream_t s);
cudaError_t lu_solve_fp32(LuGraphs* G, const float* LU, int64_t n, float* X, int k, cudaStream_t s);
size_t solve_lu_work_bytes(int64_t n, int k);
// Ainv (optional): an FP32 inverse of A; the correction of each pass is then Ainv r
// instead of the two substitutions with LU (LU may be null).
cudaError_t solve_lu_refined(LuGraphs* G, const float* A32, const float* Alo, const float* LU, int64_t n, int k,
                             const double* rhs, double* x, void* work, double tol, int max_steps, SolveStats* st,
                             cudaStream_t s, const float* Ainv = nullptr);
// Ainv (n x n) = U^{-1} L^{-1} from the factors (n substitutions at once); frees the
// n x n scratch afterwards.
cudaError_t lu_invert_fp32(LuGraphs* G, const float* LU, int64_t n, float* Ainv, cudaStream_t s);

// y(k x n) = alpha * M x(k x n) for column-major FP64 M (used for -B sigma).
cudaError_t gemm_fp64_nk(const double* M, int64_t n, int k, const double* x, double* y, double alpha, void* work,
                         cudaStream_t s);

// post.cu
struct PostTables;  // device tables built once per mesh
}  // namespace cpg
