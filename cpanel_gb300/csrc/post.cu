// Post-processing on the device (compiled with --fmad=false, FP64):
//   * CHTLS surface-velocity weights, once per mesh (bodyPanel::velocity3D/2D,
//     CPanel/bodyPanel.cpp:524-589; chtlsnd::chtlsnd, CPanel/chtlsnd.cpp:20-209);
//   * per flow condition: potential, velocity (with the reference's NaN fallback
//     chain, bodyPanel::pntVelocity :490-521), Cp (:591-594), forces and moments
//     (cpCase::compVelocity, CPanel/cpCase.cpp:342-365) and the Trefftz plane
//     (wake::trefftzPlane / Vradial / wakeStrength, CPanel/wake.cpp:146-188,478-597).
#include <mutex>
#include <vector>

#include "assemble.h"
#include "common.cuh"
#include "post.h"

namespace {

// Sorted derivative sequences (chtlsnd::derivSequence + sortBySum without the
// zero row) for N = 3 and N = 2, orders 0..3.  c_ms[N-2][order][k][d].
__constant__ int8_t c_ms[2][4][19][3];
__constant__ int c_t[2][4];
// 1 / (m_1! ... m_N!) of each row, divided out in the order the fit divides it (1 / m_1!, then
// / m_2!, ...): the same correctly rounded quotients as dividing at each fit, without the FP64
// divisions per panel, term and cluster member
__constant__ double c_fact[2][4][19];

void build_tables() {
    int8_t ms[2][4][19][3] = {};
    int tt[2][4] = {};
    double fa[2][4][19] = {};
    cpg::chtls_tables(ms, tt, fa);
    cudaMemcpyToSymbol(c_ms, ms, sizeof(ms));
    cudaMemcpyToSymbol(c_t, tt, sizeof(tt));
    cudaMemcpyToSymbol(c_fact, fa, sizeof(fa));
}

// once per device, also when several host threads start at the same time
void ensure_tables() {
    static std::once_flag once[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::call_once(once[dev & 63], build_tables);
}

constexpr int WPB = 2;        // warps (panels) per block
constexpr int NF = cpg::kClMax - 1;
constexpr int TM = 19;

// x^e for e in 0..3 as a left-to-right product (matches the CPU restatement bit
// for bit; the CHTLS normal equations are too ill-conditioned on clustered
// trailing edges to tolerate a different rounding of the monomials)
__device__ __forceinline__ double powi(double x, int e) {
    double r = 1;
    for (int k = 0; k < e; k++) r = k == 0 ? x : r * x;
    return r;
}

struct WarpSmem {
    double A[NF][TM];
    double Bm[NF][TM];
    double M[TM][TM];
    double R[TM][NF];
    double W[NF];
    double dX[NF][3];
    double Vb[NF][3];
    double tau[TM];
};

// Solve for the first N rows of F (chtlsnd unconstrained branch) for one panel.
// Returns true if every weight is finite.  Out: F[N][NF].
__device__ bool chtls_warp(WarpSmem& S, int N, int order, int nf, bool withB, double* Fout) {
    const int lane = threadIdx.x & 31;
    // rmax and normalisation
    double r = 0;
    if (lane < nf) {
        double s = 0;
        for (int d = 0; d < N; d++) s += S.dX[lane][d] * S.dX[lane][d];
        r = sqrt(s);
    }
    double rmax = r;
    for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    if (lane < nf) {
        double s = 0;
        for (int d = 0; d < N; d++) {
            S.dX[lane][d] /= rmax;
            s += S.dX[lane][d] * S.dX[lane][d];
        }
        S.W[lane] = 1 / sqrt(s);
    }
    __syncwarp();
    const int t = c_t[N - 2][order];
    if (lane < nf) {
        for (int k = 0; k < t; k++) {
            const double fact = c_fact[N - 2][order][k];
            double prod = 1;
            for (int d = 0; d < N; d++) prod *= powi(S.dX[lane][d], c_ms[N - 2][order][k][d]);
            S.A[lane][k] = fact * prod;
            if (withB) {
                double asum = 0;
                for (int a = 0; a < N; a++) {
                    int ma = c_ms[N - 2][order][k][a];
                    if (ma != 0) {
                        double pr = 1;
                        for (int d = 0; d < N; d++) {
                            int e = c_ms[N - 2][order][k][d] - (d == a ? 1 : 0);
                            pr *= powi(S.dX[lane][d], e);
                        }
                        asum += S.Vb[lane][a] * ma * pr;
                    }
                }
                S.Bm[lane][k] = fact * asum;
            }
        }
    }
    __syncwarp();
    // Normal matrix M = A^T W A (+ Bm^T W Bm), each term (A_i,rr W_i) A_i,cc summed over i in order.
    // The left factor A_i,rr W_i is the same rounded product for every cc: it is formed once, as
    // the right-hand side R = (A W)^T, and for the second sum as Bm W in A's place (A is not read
    // again); M = s1 + s2 as one addition, s2 = +0 without the B rows.
    for (int q = lane; q < t * nf; q += 32) {
        int rr = q / nf, i = q % nf;
        S.R[rr][i] = S.A[i][rr] * S.W[i];
    }
    __syncwarp();
    for (int q = lane; q < t * t; q += 32) {
        int rr = q / t, cc = q % t;
        double s1 = 0;
        for (int i = 0; i < nf; i++) s1 += S.R[rr][i] * S.A[i][cc];
        S.M[rr][cc] = withB ? s1 : s1 + 0.0;
    }
    if (withB) {
        __syncwarp();
        for (int q = lane; q < t * nf; q += 32) {
            int rr = q / nf, i = q % nf;
            S.A[i][rr] = S.Bm[i][rr] * S.W[i];
        }
        __syncwarp();
        for (int q = lane; q < t * t; q += 32) {
            int rr = q / t, cc = q % t;
            double s2 = 0;
            for (int i = 0; i < nf; i++) s2 += S.A[i][rr] * S.Bm[i][cc];
            S.M[rr][cc] = S.M[rr][cc] + s2;
        }
    }
    __syncwarp();
    // Householder QR (Eigen::HouseholderQR, unblocked) and Q^T R
    for (int k = 0; k < t; k++) {
        // sequential tail norm, same order as the CPU restatement (every lane alike)
        double part = 0;
        for (int i = k + 1; i < t; i++) part += S.M[i][k] * S.M[i][k];
        double c0 = S.M[k][k];
        double tau, beta;
        bool zero = part <= 2.2250738585072014e-308;
        if (zero) {
            tau = 0;
            beta = c0;
        } else {
            beta = sqrt(c0 * c0 + part);
            if (c0 >= 0) beta = -beta;
            tau = (beta - c0) / beta;
        }
        __syncwarp();
        for (int i = k + 1 + lane; i < t; i += 32) S.M[i][k] = zero ? 0.0 : S.M[i][k] / (c0 - beta);
        __syncwarp();
        if (lane == 0) {
            S.M[k][k] = beta;
            S.tau[k] = tau;
        }
        __syncwarp();
        if (tau != 0) {
            // the reflector on the columns of M right of k and on every column of R, one column a
            // lane in one pass (u < nm: column k + 1 + u of M, else column u - nm of R), each with
            // the operations in the order of a column at a time
            const int nm = t - k - 1;
            for (int u = lane; u < nm + nf; u += 32) {
                double* X = u < nm ? &S.M[0][k + 1 + u] : &S.R[0][u - nm];
                const int ld = u < nm ? TM : NF;
                double tmp = X[k * ld];
                for (int i = k + 1; i < t; i++) tmp += S.M[i][k] * X[i * ld];
                X[k * ld] -= tau * tmp;
                for (int i = k + 1; i < t; i++) X[i * ld] -= tau * S.M[i][k] * tmp;
            }
        }
        __syncwarp();
    }
    bool fin = true;
    if (lane < nf) {
        for (int i = t - 1; i >= 0; i--) {
            double s = S.R[i][lane];
            for (int j = i + 1; j < t; j++) s -= S.M[i][j] * S.R[j][lane];
            S.R[i][lane] = s / S.M[i][i];
        }
        for (int rr = 0; rr < N; rr++) {
            double f = S.R[rr][lane] / rmax;
            Fout[rr * NF + lane] = f;
            fin = fin && isfinite(f);
        }
    }
    __syncwarp();
    return __all_sync(0xffffffffu, fin);
}

__global__ void __launch_bounds__(32 * WPB) k_chtls(cpg::PostTables T) {
    __shared__ WarpSmem sm[WPB];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t p = (int64_t)blockIdx.x * WPB + w;
    if (p >= T.n) return;
    WarpSmem& S = sm[w];
    const double* rp = T.rec + p * R_STRIDE;
    dv3 c = ld3(rp + R_C), l = ld3(rp + R_L), m = ld3(rp + R_M);
    int c0 = T.cl_ptr[p], nf = T.cl_ptr[p + 1] - c0 - 1;
    int ts = T.tsorder[p];
    bool tip = T.tip[p] != 0;
    int mode = tip ? 4 : 0;
    if (!tip) {
        if (lane < nf) {
            int q = T.cl_idx[c0 + 1 + lane];
            dv3 cq = ld3(T.rec + (int64_t)q * R_STRIDE + R_C);
            S.dX[lane][0] = cq.x - c.x;
            S.dX[lane][1] = cq.y - c.y;
            S.dX[lane][2] = cq.z - c.z;
            S.Vb[lane][0] = T.bez[3 * q];
            S.Vb[lane][1] = T.bez[3 * q + 1];
            S.Vb[lane][2] = T.bez[3 * q + 2];
        }
        __syncwarp();
        if (chtls_warp(S, 3, ts, nf, true, T.F3 + p * 3 * NF)) mode |= 1;
    }
    if (tip || !(mode & 1)) {
        if (lane < nf) {
            int q = T.cl_idx[c0 + 1 + lane];
            dv3 cq = ld3(T.rec + (int64_t)q * R_STRIDE + R_C);
            dv3 d = cq - c;  // global2local(., true): rows l, m
            S.dX[lane][0] = dot3(l, d);
            S.dX[lane][1] = dot3(m, d);
        }
        __syncwarp();
        if (chtls_warp(S, 2, ts, nf, false, T.F2 + p * 2 * NF)) mode |= 2;
    }
    if (lane == 0) T.mode[p] = mode;
}

// Per (panel, case): phi, velocity, Cp and per-block force partials.  The potential of panel
// j is V.c_j - mu_j with V the case's free stream, or, when onset is given (n x 3, one case),
// the onset velocity at that panel (the vortex-particle case's VinfPlusVecPot).
constexpr int PT = 128;
__global__ void __launch_bounds__(PT) k_velocity(cpg::PostTables T, int k, const cpg::CaseScalars* __restrict__ CS,
                                                 const double* __restrict__ mu, const double* __restrict__ onset,
                                                 double* __restrict__ phi_out, double* __restrict__ vel_out,
                                                 double* __restrict__ cp_out, double* __restrict__ fpart) {
    __shared__ double red[9][PT / 32];
    int c = blockIdx.y;
    int64_t i = (int64_t)blockIdx.x * PT + threadIdx.x;
    const cpg::CaseScalars& S = CS[c];
    dv3 Vinf = mk3(S.Vinf[0], S.Vinf[1], S.Vinf[2]);
    double f[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (i < T.n) {
        const double* mc = mu + (int64_t)c * T.n;
        const double* rp = T.rec + i * R_STRIDE;
        dv3 ci = ld3(rp + R_C);
        // panel::setPotential, CPanel/panel.cpp:106-111
        double phii = dot3(onset ? ld3(onset + 3 * i) : Vinf, ci) - mc[i];
        int c0 = T.cl_ptr[i], nf = T.cl_ptr[i + 1] - c0 - 1;
        int mode = T.mode[i];
        bool tip = (mode & 4) != 0;
        dv3 vel;
        bool have = false;
        if (!tip) {
            const double* F = T.F3 + i * 3 * NF;
            double v[3] = {0, 0, 0};
            for (int q = 0; q < nf; q++) {
                int j = T.cl_idx[c0 + 1 + q];
                double df = (dot3(onset ? ld3(onset + 3 * j) : Vinf, ld3(T.rec + (int64_t)j * R_STRIDE + R_C)) -
                             mc[j]) - phii;
                v[0] += F[q] * df;
                v[1] += F[NF + q] * df;
                v[2] += F[2 * NF + q] * df;
            }
            vel = mk3(v[0], v[1], v[2]);
            have = !(isnan(v[0]) || isnan(v[1]) || isnan(v[2]));
        }
        if (!have && (mode & 6)) {  // velocity2D (tip patch, or NaN fallback)
            const double* F = T.F2 + i * 2 * NF;
            double v[2] = {0, 0};
            for (int q = 0; q < nf; q++) {
                int j = T.cl_idx[c0 + 1 + q];
                double df = (dot3(onset ? ld3(onset + 3 * j) : Vinf, ld3(T.rec + (int64_t)j * R_STRIDE + R_C)) -
                             mc[j]) - phii;
                v[0] += F[q] * df;
                v[1] += F[NF + q] * df;
            }
            dv3 l = ld3(rp + R_L), m = ld3(rp + R_M), n = ld3(rp + R_N);
            vel = (v[0] * l + v[1] * m) + 0.0 * n;
            have = !(isnan(vel.x) || isnan(vel.y) || isnan(vel.z));
        }
        dv3 bz = ld3(T.bez + 3 * i);
        if (!have) vel = cross3(cross3(bz, Vinf), bz);  // CBAERO last resort
        vel.x /= S.PG;
        double sp = norm3(vel) / S.V;
        double cp = 1 - sp * sp;
        int64_t o = (int64_t)c * T.n + i;
        if (phi_out) phi_out[o] = phii;
        if (vel_out) {
            vel_out[3 * o] = vel.x;
            vel_out[3 * o + 1] = vel.y;
            vel_out[3 * o + 2] = vel.z;
        }
        if (cp_out) cp_out[o] = cp;
        double area = rp[R_AREA];
        dv3 F = ((-cp * area) * bz) / S.Sref;
        dv3 r = ci - mk3(S.cg[0], S.cg[1], S.cg[2]);
        dv3 Fm = mk3(((-cp) * bz.x) * area, ((-cp) * bz.y) * area, ((-cp) * bz.z) * area);
        dv3 mom = cross3(r, Fm);
        f[0] = F.x;
        f[1] = F.y;
        f[2] = F.z;
        f[3] = mom.x / (S.Sref * S.bref);
        f[4] = mom.y / (S.Sref * S.cref);
        f[5] = mom.z / (S.Sref * S.bref);
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        double v = f[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[q][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0;
        for (int w2 = 0; w2 < PT / 32; w2++) s += red[threadIdx.x][w2];
        fpart[((int64_t)c * gridDim.x + blockIdx.x) * 6 + threadIdx.x] = s;
    }
}

__global__ void k_forces_finish(const double* __restrict__ fpart, int nb, int k, const cpg::CaseScalars* __restrict__ CS,
                                double* __restrict__ out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nb; b++)
        for (int q = 0; q < 6; q++) s[q] += fpart[((int64_t)c * nb + b) * 6 + q];
    const double* T = CS[c].T;
    double* o = out + 9 * c;
    o[0] = s[0];
    o[1] = s[1];
    o[2] = s[2];
    for (int r = 0; r < 3; r++) o[3 + r] = T[0 * 3 + r] * s[0] + T[1 * 3 + r] * s[1] + T[2 * 3 + r] * s[2];
    o[6] = s[3];
    o[7] = s[4];
    o[8] = s[5];
}

// Trefftz plane: one block per case.
__global__ void k_trefftz(cpg::PostTables T, int k, const cpg::CaseScalars* __restrict__ CS,
                          const double* __restrict__ mu, double* __restrict__ wmu_out, double* __restrict__ scratch,
                          double* __restrict__ out) {
    int c = blockIdx.x;
    const double* mc = mu + (int64_t)c * T.n;
    double* wmu = wmu_out + (int64_t)c * T.nw;
    double* phip = scratch + (int64_t)c * (T.n_pts + 2 * T.n_st * T.n_wakes);
    double* clcd = phip + T.n_pts;
    // wakePanel::setMu, CPanel/wakePanel.cpp:94-100
    for (int64_t j = threadIdx.x; j < T.nw; j += blockDim.x) {
        const int32_t* ix = T.widx + 4 * j;
        double cc = T.wcoef[j];
        wmu[j] = (1 - cc) * mc[ix[0]] + (cc - 1) * mc[ix[1]] + cc * mc[ix[2]] - cc * mc[ix[3]];
    }
    __syncthreads();
    // geometry::wakePotential at every sample point
    for (int64_t p = threadIdx.x; p < T.n_pts; p += blockDim.x) {
        const double* g = T.G + p * T.nw;
        double pot = 0;
        for (int64_t j = 0; j < T.nw; j++) pot += -wmu[j] * g[j];
        phip[p] = pot;
    }
    __syncthreads();
    const cpg::CaseScalars& S = CS[c];
    int nst = T.n_st * T.n_wakes;
    for (int q = threadIdx.x; q < nst; q += blockDim.x) {
        const double* st = T.tz_station + (int64_t)q * 15;
        const int32_t* ln = T.tz_lines + (int64_t)q * 5;
        int pt0 = ln[4];
        double phiPOI = phip[pt0];
        double v = 0, w = 0;
        for (int a = 0; a < 6; a++) v += st[2 + a] * (phip[pt0 + 1 + a] - phiPOI);
        for (int a = 0; a < 6; a++) w += st[8 + a] * (phip[pt0 + 7 + a] - phiPOI);
        double Vr = sqrt(v * v + w * w);
        double s1 = mc[ln[0]] - mc[ln[1]], s2 = mc[ln[2]] - mc[ln[3]];
        double dPhi = -(s1 + st[1] * (s2 - s1));
        clcd[2 * q] = 2 * dPhi / (S.V * S.Sref);
        clcd[2 * q + 1] = dPhi * Vr / (S.V * S.V * S.Sref);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double CL = 0, CD = 0;
        for (int wk = 0; wk < T.n_wakes; wk++) {
            const double* base = clcd + 2 * (int64_t)wk * T.n_st;
            double step = T.tz_station[((int64_t)wk * T.n_st) * 15 + 14];
            // Cl(0) = Cl(164) = 0; stations 1..163 stored at 0..162
            auto Cl = [&](int i) { return (i <= 0 || i >= T.n_st + 1) ? 0.0 : base[2 * (i - 1)]; };
            auto Cd = [&](int i) { return (i <= 0 || i >= T.n_st + 1) ? 0.0 : base[2 * (i - 1) + 1]; };
            double cl = 0, cd = 0;
            int i = 0;
            while (i < T.n_st + 2 - 2) {
                cl += 1.0 / 3 * step * (Cl(i) + 4 * Cl(i + 1) + Cl(i + 2));
                cd += 1.0 / 3 * step * (Cd(i) + 4 * Cd(i + 1) + Cd(i + 2));
                i += 2;
            }
            CL += cl / S.PG;
            CD += cd / (S.PG * S.PG);
        }
        out[2 * c] = CL;
        out[2 * c + 1] = CD;
    }
}

// sigma_i = -Vinf . n_i + 0 (bodyPanel::setSigma, CPanel/bodyPanel.cpp:97-100)
__global__ void k_sigma(const double* __restrict__ rec, int64_t n, int k, const cpg::CaseScalars* __restrict__ CS,
                        double* __restrict__ sigma) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)k * n) return;
    int c = (int)(t / n);
    int64_t i = t % n;
    const double* V = CS[c].Vinf;
    const double* nn = rec + i * R_STRIDE + R_N;
    sigma[t] = (-(V[0] * nn[0] + V[1] * nn[1] + V[2] * nn[2]) + 0);
}

// rhs = -B sigma = sum_d Vinf_d * rb_d  (rb_d = B n_d, accumulated by the mixed assembly)
__global__ void k_rhs_basis(const double* __restrict__ rb, int64_t n, int k, const cpg::CaseScalars* __restrict__ CS,
                            double* __restrict__ rhs) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)k * n) return;
    int c = (int)(t / n);
    int64_t i = t % n;
    const double* V = CS[c].Vinf;
    rhs[t] = V[0] * rb[i] + V[1] * rb[n + i] + V[2] * rb[2 * n + i];
}

__global__ void k_widen(const float* __restrict__ a, const float* __restrict__ lo, double* __restrict__ b, int64_t m) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m) b[t] = lo ? (double)a[t] + (double)lo[t] : (double)a[t];
}

}  // namespace

namespace cpg {

cudaError_t launch_sigma(const double* rec, int64_t n, int k, const CaseScalars* cs, double* sigma, cudaStream_t s) {
    int64_t m = (int64_t)k * n;
    k_sigma<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(rec, n, k, cs, sigma);
    return cudaGetLastError();
}

cudaError_t launch_rhs_basis(const double* rb, int64_t n, int k, const CaseScalars* cs, double* rhs, cudaStream_t s) {
    int64_t m = (int64_t)k * n;
    k_rhs_basis<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(rb, n, k, cs, rhs);
    return cudaGetLastError();
}

cudaError_t launch_widen(const float* a, const float* lo, double* b, int64_t m, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    k_widen<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(a, lo, b, m);
    return cudaGetLastError();
}

cudaError_t launch_chtls_weights(const PostTables& t, cudaStream_t s) {
    ensure_tables();
    if (t.n <= 0) return cudaSuccess;
    ProfScope ps(Prof::CHTLS, s);
    k_chtls<<<(unsigned)((t.n + WPB - 1) / WPB), 32 * WPB, 0, s>>>(t);
    return cudaGetLastError();
}

size_t post_work_bytes(const PostTables& t, int k) {
    int64_t nb = (t.n + PT - 1) / PT;
    return sizeof(double) * ((size_t)k * nb * 6 + (size_t)k * (t.n_pts + 2 * t.n_st * t.n_wakes)) + 1024;
}

const double* post_station_loads(const PostTables& t, int k, int c, int w, const void* work) {
    const int64_t nb = (t.n + PT - 1) / PT;
    const double* tz = (const double*)work + (size_t)k * nb * 6;  // k_trefftz's scratch, as launch_post lays it out
    return tz + (int64_t)c * (t.n_pts + 2 * t.n_st * t.n_wakes) + t.n_pts + 2 * (int64_t)w * t.n_st;
}

cudaError_t launch_post(const PostTables& t, int k, const CaseScalars* cs, const double* mu, double* phi, double* vel,
                        double* cp, double* forces, double* trefftz, double* wake_mu, void* work, cudaStream_t s) {
    int64_t nb = (t.n + PT - 1) / PT;
    double* fpart = (double*)work;
    double* tz = fpart + (size_t)k * nb * 6;
    dim3 grid((unsigned)nb, (unsigned)k);
    ProfScope ps(Prof::POST, s);
    k_velocity<<<grid, PT, 0, s>>>(t, k, cs, mu, nullptr, phi, vel, cp, fpart);
    k_forces_finish<<<(k + 31) / 32, 32, 0, s>>>(fpart, (int)nb, k, cs, forces);
    if (t.n_wakes > 0) k_trefftz<<<k, 256, 0, s>>>(t, k, cs, mu, wake_mu, tz, trefftz);
    return cudaGetLastError();
}

cudaError_t launch_surface(const PostTables& t, const CaseScalars* cs, const double* mu, const double* onset,
                           double* phi, double* vel, double* cp, double* forces, void* work, cudaStream_t s) {
    int64_t nb = (t.n + PT - 1) / PT;
    double* fpart = (double*)work;
    ProfScope ps(Prof::POST, s);
    k_velocity<<<dim3((unsigned)nb, 1), PT, 0, s>>>(t, 1, cs, mu, onset, phi, vel, cp, fpart);
    k_forces_finish<<<1, 32, 0, s>>>(fpart, (int)nb, 1, cs, forces);
    return cudaGetLastError();
}

}  // namespace cpg
