// Skinny products C (m x kc) = alpha A (m x K) B (K x kc) (+ C) on the CUDA cores: the block
// substitutions of the FP32 LU (lu.cu) and the inverse product of the refinement.  A is read
// once; kc (the right-hand sides) is small.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace cpg {

// Scratch of the split-K products: per-tile partials and per-tile arrival counters, which are
// zero between launches (each launch's last block returns its counter to 0).  One scratch must
// not be shared by launches that may run at the same time.
struct SkinnySplit {
    float* ws = nullptr;      // kSkinnyWsFloats floats
    unsigned* cnt = nullptr;  // kSkinnyCounters counters, zeroed once at allocation
};
constexpr int kSkinnyTarget = 2 * 152;              // thread blocks of one wave (two resident per SM)
constexpr int kSkinnyMaxBlocks = 4 * kSkinnyTarget;  // a split launch has at most four waves
constexpr size_t kSkinnyWsFloats = (size_t)kSkinnyMaxBlocks * 64 * 32;
constexpr int kSkinnyCounters = kSkinnyMaxBlocks;

// All matrices column-major (leading dimensions lda, ldb, ldc).  kc columns of B are taken
// kc at a time for kc <= 32 and in equal groups of at most 32 above; sp (may be null) lets a
// product with too few row tiles to fill the GPU split K.  Issued on s.
cudaError_t skinny(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int64_t m,
                   int64_t K, int kc, float alpha, bool accum, cudaStream_t s, const SkinnySplit* sp = nullptr);

}  // namespace cpg
