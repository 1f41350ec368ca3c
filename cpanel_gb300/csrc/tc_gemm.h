// Tensor-core GEMM for the FP32 factorizations of the mixed path (sm_103a: tcgen05 + TMA).
//
// An FP32 operand is split per row into two FP16 halves after a power-of-two row scale:
// row r of the operand (its K values contiguous: "K-major") is multiplied by 2^e_r, with e_r
// chosen so that the row's largest magnitude lands in [2^13, 2^14), then hi = fp16(x) and
// lo = fp16(x - hi).  A product sum_k A_ik B_jk is taken as Ah Bh + Ah Bl + Al Bh in one FP32
// accumulator in tensor memory, then scaled back by 2^-(e_i + e_j) (exact).  Each split value
// carries about 22 significant bits, so the products carry a relative error of a few 2^-22:
// a few times that of an FP32 GEMM, and the iterative refinement of the solves absorbs it.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cpg {

// [2][rows_cap][kp] halves (the hi block, then the lo block) and the inverse row scales.
struct TcOperand {
    __half* data = nullptr;
    float* inv_scale = nullptr;
    int64_t rows_cap = 0;
    int64_t kp = 0;  // row length in halves: a multiple of 64
};

constexpr int kTcK = 64;  // K granularity of the operands

// device bytes of an operand of rows_cap rows of kp halves (data, scales, alignment)
size_t tc_operand_bytes(int64_t rows_cap, int64_t kp);
// lays an operand out in mem (tc_operand_bytes(rows_cap, kp) bytes, 256-byte aligned)
void tc_operand_bind(TcOperand& op, void* mem, int64_t rows_cap, int64_t kp);
// the operand's rows from r0 on
inline TcOperand tc_rows(const TcOperand& op, int64_t r0) {
    TcOperand v = op;
    v.data = op.data + r0 * op.kp;
    v.inv_scale = op.inv_scale + r0;
    v.rows_cap = op.rows_cap;  // the hi-to-lo distance stays rows_cap rows
    return v;
}

// Splits rows x K of an FP32 source into op: element (r, k) is src[r * rs + k * ks] (strides in
// elements; one of rs, ks must be 1: K-major or column-major sources); k in [K, kp) is written
// as zero.  err (device, may be null) is set to 2 when a row holds a non-finite value.
cudaError_t tc_split(const float* src, int64_t rs, int64_t ks, int64_t rows, int64_t K, TcOperand& op, int* err,
                     cudaStream_t s);

// C[i + j ldc] = beta C[i + j ldc] + alpha sum_k A_ik B_jk for i < m, j < n, with A (m rows) and B
// (n rows) split over the same kp.  beta = 0 does not read C.  The grid is persistent, one CTA per
// SM, at most sm_budget CTAs (the rest of the SMs stay free for work on other streams).  err
// (device) is set to 1 when one of the kernel's waits ran past its limit (about two seconds);
// the kernel then stops early and C is incomplete.  counter (device int, may be null): the
// CTAs draw tiles from it (it is zeroed on the stream first), so a grid whose CTAs cannot all
// start at once still finishes with the ones that did; it must not be shared by launches
// that may run at the same time.  Each tile is computed by one CTA in a fixed order, so the
// result does not depend on the schedule.
cudaError_t tc_gemm(const TcOperand& A, int64_t m, const TcOperand& B, int64_t n, float alpha, float beta, float* C,
                    int64_t ldc, int sm_budget, int* err, cudaStream_t s, int* counter = nullptr);

// number of SMs of the current device
int tc_num_sms();

}  // namespace cpg
