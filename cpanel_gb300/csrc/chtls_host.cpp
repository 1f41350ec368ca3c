// CHTLS velocity weights on the host (chtlsnd::chtlsnd, CPanel/chtlsnd.cpp:20-140, 189-196, as
// bodyPanel::setCluster's panels use them): the fit of k_chtls (post.cu) operation for operation,
// so the weights are the same bits, for geometries whose post tables are built on the host threads
// while the device assembles their matrix.  Also the sorted derivative sequences both use.
#include <cmath>
#include <vector>

#include "mesh.h"
#include "post.h"

namespace cpg {

void chtls_tables(int8_t ms[2][4][19][3], int tt[2][4], double fa[2][4][19]) {
    for (int N = 2; N <= 3; N++)
        for (int q = 0; q <= 3; q++) {
            // recursive derivSequence
            std::vector<std::vector<int>> d;
            struct R {
                static std::vector<std::vector<int>> seq(int q, int N) {
                    std::vector<std::vector<int>> out;
                    if (q == 0) {
                        out.push_back(std::vector<int>(N, 0));
                        return out;
                    }
                    for (int i = 0; i <= q; i++) {
                        if (N > 1) {
                            auto sub = seq(q - i, N - 1);
                            for (auto& r : sub) {
                                r.push_back(i);
                                out.push_back(r);
                            }
                        } else {
                            out.push_back(std::vector<int>{i});
                        }
                    }
                    return out;
                }
            };
            d = R::seq(q, N);
            // stable insertion by row sum (sortBySum)
            auto sum = [](const std::vector<int>& r) {
                int s = 0;
                for (int v : r) s += v;
                return s;
            };
            std::vector<std::vector<int>> o{d[0]};
            for (size_t i = 1; i < d.size(); i++) {
                bool ins = false;
                for (size_t j = 0; j < o.size(); j++)
                    if (sum(d[i]) < sum(o[j])) {
                        o.insert(o.begin() + (long)j, d[i]);
                        ins = true;
                        break;
                    }
                if (!ins) o.push_back(d[i]);
            }
            o.erase(o.begin());
            tt[N - 2][q] = (int)o.size();
            for (size_t k = 0; k < o.size() && k < 19; k++) {
                double f = 1;
                for (int a = 0; a < N; a++) {
                    ms[N - 2][q][k][a] = (int8_t)o[k][a];
                    int fi = 1;
                    for (int j = 2; j <= o[k][a]; j++) fi *= j;
                    f /= (double)fi;
                }
                fa[N - 2][q][k] = f;
            }
        }
}

namespace {

constexpr int NF = kClMax - 1;
constexpr int TM = 19;

// x^e for e in 0..3 as a left-to-right product
double powi(double x, int e) {
    double r = 1;
    for (int k = 0; k < e; k++) r = k == 0 ? x : r * x;
    return r;
}

struct Tables {
    int8_t ms[2][4][19][3] = {};
    int tt[2][4] = {};
    double fa[2][4][19] = {};
    Tables() { chtls_tables(ms, tt, fa); }
};
const Tables& tables() {
    static const Tables t;
    return t;
}

struct Fit {
    double A[NF][TM], Bm[NF][TM], M[TM][TM], R[TM][NF], W[NF], dX[NF][3], Vb[NF][3];
};

// chtls_warp of post.cu with its lanes as the loop index: the first N rows of F for one panel;
// false if a weight is not finite.  Out: F[N][NF].
bool fit(Fit& S, int N, int order, int nf, bool withB, double* Fout) {
    const Tables& T = tables();
    double rmax = 0;
    for (int i = 0; i < nf; i++) {
        double s = 0;
        for (int d = 0; d < N; d++) s += S.dX[i][d] * S.dX[i][d];
        rmax = std::fmax(rmax, std::sqrt(s));
    }
    for (int i = 0; i < nf; i++) {
        double s = 0;
        for (int d = 0; d < N; d++) {
            S.dX[i][d] /= rmax;
            s += S.dX[i][d] * S.dX[i][d];
        }
        S.W[i] = 1 / std::sqrt(s);
    }
    const int t = T.tt[N - 2][order];
    const int8_t(*ms)[3] = T.ms[N - 2][order];
    for (int i = 0; i < nf; i++)
        for (int k = 0; k < t; k++) {
            const double fact = T.fa[N - 2][order][k];
            double prod = 1;
            for (int d = 0; d < N; d++) prod *= powi(S.dX[i][d], ms[k][d]);
            S.A[i][k] = fact * prod;
            if (withB) {
                double asum = 0;
                for (int a = 0; a < N; a++) {
                    const int ma = ms[k][a];
                    if (ma != 0) {
                        double pr = 1;
                        for (int d = 0; d < N; d++) pr *= powi(S.dX[i][d], ms[k][d] - (d == a ? 1 : 0));
                        asum += S.Vb[i][a] * ma * pr;
                    }
                }
                S.Bm[i][k] = fact * asum;
            }
        }
    for (int rr = 0; rr < t; rr++)
        for (int i = 0; i < nf; i++) S.R[rr][i] = S.A[i][rr] * S.W[i];
    for (int rr = 0; rr < t; rr++)
        for (int cc = 0; cc < t; cc++) {
            double s1 = 0;
            for (int i = 0; i < nf; i++) s1 += S.R[rr][i] * S.A[i][cc];
            S.M[rr][cc] = withB ? s1 : s1 + 0.0;
        }
    if (withB) {
        for (int rr = 0; rr < t; rr++)
            for (int i = 0; i < nf; i++) S.A[i][rr] = S.Bm[i][rr] * S.W[i];
        for (int rr = 0; rr < t; rr++)
            for (int cc = 0; cc < t; cc++) {
                double s2 = 0;
                for (int i = 0; i < nf; i++) s2 += S.A[i][rr] * S.Bm[i][cc];
                S.M[rr][cc] = S.M[rr][cc] + s2;
            }
    }
    // Householder QR (Eigen::HouseholderQR, unblocked) and Q^T R
    for (int k = 0; k < t; k++) {
        double part = 0;
        for (int i = k + 1; i < t; i++) part += S.M[i][k] * S.M[i][k];
        const double c0 = S.M[k][k];
        double tau, beta;
        const bool zero = part <= 2.2250738585072014e-308;
        if (zero) {
            tau = 0;
            beta = c0;
        } else {
            beta = std::sqrt(c0 * c0 + part);
            if (c0 >= 0) beta = -beta;
            tau = (beta - c0) / beta;
        }
        for (int i = k + 1; i < t; i++) S.M[i][k] = zero ? 0.0 : S.M[i][k] / (c0 - beta);
        S.M[k][k] = beta;
        if (tau != 0) {
            const int nm = t - k - 1;
            for (int u = 0; u < nm + nf; u++) {
                double* X = u < nm ? &S.M[0][k + 1 + u] : &S.R[0][u - nm];
                const int ld = u < nm ? TM : NF;
                double tmp = X[k * ld];
                for (int i = k + 1; i < t; i++) tmp += S.M[i][k] * X[i * ld];
                X[k * ld] -= tau * tmp;
                for (int i = k + 1; i < t; i++) X[i * ld] -= tau * S.M[i][k] * tmp;
            }
        }
    }
    bool fin = true;
    for (int i = 0; i < nf; i++) {
        for (int r = t - 1; r >= 0; r--) {
            double s = S.R[r][i];
            for (int j = r + 1; j < t; j++) s -= S.M[r][j] * S.R[j][i];
            S.R[r][i] = s / S.M[r][r];
        }
        for (int rr = 0; rr < N; rr++) {
            const double f = S.R[rr][i] / rmax;
            Fout[rr * NF + i] = f;
            fin = fin && std::isfinite(f);
        }
    }
    return fin;
}

}  // namespace

void chtls_weights_host(const HostMesh& H, double* F3, double* F2, int32_t* mode) {
    const int64_t n = H.n_body;
    host_parallel((size_t)n, [&](unsigned, size_t lo, size_t hi) {
        Fit S;
        for (int64_t p = (int64_t)lo; p < (int64_t)hi; p++) {
            const double* rp = &H.body[p * PF_STRIDE];
            const double* c = rp + PF_C;
            const double* l = rp + PF_L;
            const double* m = rp + PF_M;
            const int c0 = H.cl_ptr[p], nf = H.cl_ptr[p + 1] - c0 - 1;
            const int ts = H.tsorder[p];
            const bool tip = H.tip[p] != 0;
            int md = tip ? 4 : 0;
            if (!tip) {
                for (int i = 0; i < nf; i++) {
                    const int q = H.cl_idx[c0 + 1 + i];
                    const double* cq = &H.body[(int64_t)q * PF_STRIDE + PF_C];
                    S.dX[i][0] = cq[0] - c[0];
                    S.dX[i][1] = cq[1] - c[1];
                    S.dX[i][2] = cq[2] - c[2];
                    S.Vb[i][0] = H.bez[3 * q];
                    S.Vb[i][1] = H.bez[3 * q + 1];
                    S.Vb[i][2] = H.bez[3 * q + 2];
                }
                if (fit(S, 3, ts, nf, true, F3 + p * 3 * NF)) md |= 1;
            }
            if (tip || !(md & 1)) {
                for (int i = 0; i < nf; i++) {
                    const int q = H.cl_idx[c0 + 1 + i];
                    const double* cq = &H.body[(int64_t)q * PF_STRIDE + PF_C];
                    const double d0 = cq[0] - c[0], d1 = cq[1] - c[1], d2 = cq[2] - c[2];
                    S.dX[i][0] = l[0] * d0 + l[1] * d1 + l[2] * d2;
                    S.dX[i][1] = m[0] * d0 + m[1] * d1 + m[2] * d2;
                }
                if (fit(S, 2, ts, nf, false, F2 + p * 2 * NF)) md |= 2;
            }
            mode[p] = md;
        }
    });
}

}  // namespace cpg
