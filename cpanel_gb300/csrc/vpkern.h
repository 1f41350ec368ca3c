// Launchers of the vortex-particle case kernels (vpkern.cu).  All arrays on the device.
// rec: body panel records (24 doubles); q1/q2: quad records of the two buffer rows
// (32 doubles); fil: filaments, 8 doubles each (p1, p2, strength, pad).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cpg {

cudaError_t vp_launch_wake_columns(const double* rec, int64_t n, const double* q1, const int32_t* widx,
                                   const double* wcoef, int64_t n1, double* A, cudaStream_t s);
// y += x over n doubles
cudaError_t vp_launch_add(double* y, const double* x, int64_t n, cudaStream_t s);
// A32 = fl(A), Alo = fl(A - A32) elementwise over nn entries
cudaError_t vp_launch_split(const double* A, int64_t nn, float* A32, float* Alo, cudaStream_t s);
cudaError_t vp_launch_cmat(const double* rec, int64_t n, const double* q2, int64_t n2, double* C, cudaStream_t s);
// scratch of the two panel kernels below: vp_scratch_doubles(m, nb) doubles.  far_f32:
// panel pairs beyond five panel lengths in FP32 (same near/far split as FP64).
int64_t vp_scratch_doubles(int64_t m, int64_t nb);
cudaError_t vp_launch_panel_vel(const double* rec, const double* sigma, const double* mu, int64_t nb, const double* q1,
                                const double* mu1, int64_t n1, const double* q2, const double* mu2, int64_t n2,
                                const double* fil, int64_t nf, const double* pts, int64_t m, double skip_r,
                                double* out, double* scratch, cudaStream_t s, bool far_f32 = false);
cudaError_t vp_launch_stretch_panels(const double* rec, const double* sigma, const double* mu, int64_t nb,
                                     const double* q1, const double* mu1, int64_t n1, const double* pos,
                                     const double* str, int64_t m, double skip_x, double* out, double* scratch,
                                     cudaStream_t s, bool far_f32 = false);
cudaError_t vp_launch_convect(double* pos, double* prevVel, const double* part, const double* pan, int64_t m,
                              const double vinf[3], double cref, double dt, cudaStream_t s);
cudaError_t vp_launch_strength(const double* pos, double* str, double* prevStr, const double* dstr,
                               const double* ddif, const double* dpan, int64_t m, double cref, double dt,
                               cudaStream_t s);
cudaError_t vp_launch_sigma(const double* rec, int64_t n, const double* vpart, const double* fil, int64_t nf,
                            const double vinf[3], double* sigma, double* vtot, cudaStream_t s);
cudaError_t vp_launch_rhs_c(const double* C, int64_t n, int64_t n2, const double* mu2, double* rhs, cudaStream_t s);
cudaError_t vp_launch_wake_mu(const double* mu, const int32_t* widx, const double* wcoef, int64_t n1, double* mu1,
                              double* prev1, int keep_prev, cudaStream_t s);
cudaError_t vp_launch_buffer(const double* mu1, const int32_t* parent, int64_t n2, double* mu2, double* prev2,
                             cudaStream_t s);

}  // namespace cpg
