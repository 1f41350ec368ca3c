// Shared device helpers for the GB300 panel kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CPG_PI 3.14159265358979323846
#define CPG_FOUR_PI (4.0 * CPG_PI)

struct dv3 {
    double x, y, z;
};
__device__ __forceinline__ dv3 mk3(double x, double y, double z) { return dv3{x, y, z}; }
__device__ __forceinline__ dv3 operator+(dv3 a, dv3 b) { return dv3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ dv3 operator-(dv3 a, dv3 b) { return dv3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ dv3 operator*(double s, dv3 a) { return dv3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ dv3 operator/(dv3 a, double s) { return dv3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double dot3(dv3 a, dv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double norm3(dv3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ dv3 cross3(dv3 a, dv3 b) {
    return dv3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ dv3 ld3(const double* p) { return dv3{p[0], p[1], p[2]}; }

// Packed panel record layout (must match cpg::PanelField in mesh.h).
enum { R_V0 = 0, R_V1 = 3, R_V2 = 6, R_C = 9, R_N = 12, R_L = 15, R_M = 18, R_AREA = 21, R_LONG = 22, R_STRIDE = 24 };

// Per-panel double-float record of the mixed assembly (FP32 pairs):
// [c_hi(3) c_lo(3) n_hi(3) n_lo(3) area_hi area_lo longSide pad] for the far field, then for
// the exact formulas between 3 and 5 longSide, as (hi, lo) pairs: vertices minus centroid
// (3 x 3), n x s_k for the edges s_k = v_{k+1} - v_k (3 x 3), |s_k| (3), 1/|s_k| (3).
enum {
    F_CHI = 0, F_CLO = 3, F_NHI = 6, F_NLO = 9, F_AHI = 12, F_ALO = 13, F_LONG = 14,
    F_VC = 16, F_NS = 34, F_S = 52, F_IS = 58, F_STRIDE = 64
};

// Per-panel FP64 edge constants of the mixed assembly's near field:
// [|s_k| (3), 1/|s_k| (3), s_k.m (3), pad (3)] with s_k = v_{k+1} - v_k.
enum { E_S = 0, E_IS = 3, E_SM = 6, E_STRIDE = 12 };

#define CPG_CUDA_OK(x) ((x) == cudaSuccess)
