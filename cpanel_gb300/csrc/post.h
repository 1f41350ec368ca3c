// Post-processing tables and launchers (post.cu): CHTLS surface velocity, Cp,
// forces and the Trefftz-plane analysis, all on the device.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cpg {

constexpr int kClMax = 32;  // max cluster size (self included)

struct HostMesh;
// Sorted derivative sequences of chtlsnd (derivSequence + sortBySum, without the zero row) for N = 3
// and N = 2, orders 0..3: ms[N-2][order][k][d], tt[N-2][order] rows, fa[N-2][order][k] =
// 1 / (m_1! ... m_N!) divided out in that order (chtls_host.cpp).
void chtls_tables(int8_t ms[2][4][19][3], int tt[2][4], double fa[2][4][19]);
// The CHTLS weights and modes of every body panel on the host threads, the same bits as
// launch_chtls_weights: F3 (n x 3 x 31), F2 (n x 2 x 31), mode (n); entries past a panel's cluster
// are left as they are.
void chtls_weights_host(const HostMesh& H, double* F3, double* F2, int32_t* mode);

struct PostTables {
    int64_t n = 0, nw = 0;
    const double* rec = nullptr;     // body panel records (n x 24)
    const double* bez = nullptr;     // n x 3
    const int32_t* cl_ptr = nullptr; // n+1
    const int32_t* cl_idx = nullptr;
    const int32_t* tip = nullptr;
    const int32_t* tsorder = nullptr;
    const int32_t* widx = nullptr;   // n_wake x 4
    const double* wcoef = nullptr;
    // built by launch_chtls_weights
    double* F3 = nullptr;            // n x 3 x 31
    double* F2 = nullptr;            // n x 2 x 31
    int32_t* mode = nullptr;         // n: bit0 3-D weights finite, bit1 2-D weights finite, bit2 tip
    // Trefftz
    int n_wakes = 0;
    int n_st = 0;                    // stations per wake (163)
    const double* tz_station = nullptr;  // per station: y, interp, Fy[6], Fz[6], step  (15 doubles)
    const int32_t* tz_lines = nullptr;   // per station: up1 lo1 up2 lo2 pt0 (5 ints)
    const double* G = nullptr;       // n_pts x nw dubPhiInf operator
    int64_t n_pts = 0;
};

struct CaseScalars {  // per flow condition
    double Vinf[3];
    double V, PG, Sref, bref, cref, cg[3];
    double T[9];      // windToBody transform (row-major)
};

cudaError_t launch_chtls_weights(const PostTables& t, cudaStream_t s);
// mu: k x n; outputs k x n (phi, cp), k x n x 3 (vel); forces k x 9 [Fbody Fwind CM];
// trefftz k x 2 [CL CDi]; work: device scratch of post_work_bytes.
size_t post_work_bytes(const PostTables& t, int k);
// Device address, inside the work area of the last launch_post over k cases, of case c's Trefftz
// station loads of wake w: (Cl, Cd) pairs of stations 1..n_st, before the Prandtl-Glauert factors.
const double* post_station_loads(const PostTables& t, int k, int c, int w, const void* work);
cudaError_t launch_post(const PostTables& t, int k, const CaseScalars* cs_dev, const double* mu, double* phi,
                        double* vel, double* cp, double* forces, double* trefftz, double* wake_mu, void* work,
                        cudaStream_t s);

// The surface pass alone for one case whose panel potentials come from an onset velocity
// field (n x 3, device) instead of the free stream: phi, vel, cp as launch_post (any may be
// null), forces 9 [Fbody Fwind CM]; work: post_work_bytes(t, 1).
cudaError_t launch_surface(const PostTables& t, const CaseScalars* cs, const double* mu, const double* onset,
                           double* phi, double* vel, double* cp, double* forces, void* work, cudaStream_t s);

cudaError_t launch_sigma(const double* rec, int64_t n, int k, const CaseScalars* cs, double* sigma, cudaStream_t s);
cudaError_t launch_rhs_basis(const double* rb, int64_t n, int k, const CaseScalars* cs, double* rhs, cudaStream_t s);
// b = a (+ lo when lo is not null), FP32 -> FP64
cudaError_t launch_widen(const float* a, const float* lo, double* b, int64_t m, cudaStream_t s);

}  // namespace cpg
