// FP64 constant-strength triangle influence functions (device).
//
// Include only from translation units compiled with --fmad=false: products and
// sums are then rounded exactly as the reference's Eigen expressions are, which
// keeps every branch decision (self, near/far, on-edge, log guard) identical to
// the CPU restatement.  sqrt and division are IEEE-rounded in CUDA; atan2 and log
// are CUDA's own (<= 2 ulp).
#pragma once
#include "common.cuh"

// panel::vortexPhi, CPanel/panel.cpp:713-735
__device__ __forceinline__ double vortex_phi(double PN, double Al, dv3 a, dv3 b, dv3 s, dv3 l, dv3 m) {
    const double eps = 1e-15;  // pow(10,-15)
    double PA = dot3(a, cross3(l, cross3(a, s)));
    double sm = dot3(s, m);
    double PB = PA - Al * sm;
    double na = norm3(a), nb = norm3(b);
    double num = sm * PN * (nb * PA - na * PB);
    double denom = PA * PB + (PN * PN) * na * nb * (sm * sm);
    if (denom == 0.0 && fabs(PN) < eps) return PN >= 0 ? 0.5 * CPG_PI : -0.5 * CPG_PI;
    return atan2(num, denom);
}

// bodyPanel::srcSidePhi, CPanel/bodyPanel.cpp:361-373 (the log edge factor GL)
__device__ __forceinline__ double src_gl(dv3 a, dv3 b, dv3 s) {
    double A = norm3(a), B = norm3(b), S = norm3(s);
    double GL = 0;
    if (fabs(A + B - S) > 0 && S > 0) GL = 1 / S * log(fabs((A + B + S) / (A + B - S)));
    return GL;
}

// bodyPanel::panelPhiInf, CPanel/bodyPanel.cpp:132-190, for a packed panel record.
// Returns 1 if the pair is in the near field (edge integrals), 0 if far.
__device__ __forceinline__ int panel_phi_inf(const double* r, dv3 poi, double& phiSrc, double& phiDub) {
    dv3 c = ld3(r + R_C);
    dv3 pjk = poi - c;
    double d = norm3(pjk);
    bool itself = d < 1e-10;
    dv3 n = ld3(r + R_N);
    double PN = dot3(pjk, n);
    double area = r[R_AREA];
    if (d / r[R_LONG] > 5) {
        phiSrc = area / (CPG_FOUR_PI * d);
        phiDub = PN * area / (CPG_FOUR_PI * (d * d * d));
        return 0;
    }
    dv3 l = ld3(r + R_L), m = ld3(r + R_M);
    dv3 p[3] = {ld3(r + R_V0), ld3(r + R_V1), ld3(r + R_V2)};
    double src = 0, dub = 0, phiV = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        dv3 p1 = p[i], p2 = p[i == 2 ? 0 : i + 1];
        dv3 a = poi - p1, b = poi - p2, s = p2 - p1;
        double Al = dot3(n, cross3(s, a));
        if (!itself) {
            phiV = vortex_phi(PN, Al, a, b, s, l, m);
            dub += phiV;
        }
        src += Al * src_gl(a, b, s) - PN * phiV;
    }
    phiSrc = src / CPG_FOUR_PI;
    phiDub = itself ? -0.5 : dub / CPG_FOUR_PI;
    return 1;
}

// panel_phi_inf for a near pair of the mixed path, with the panel's per-edge constants
// precomputed (ec: |s_k|, 1/|s_k|, s_k.m for k = 0..2, rounded as the device would form
// them) and the three vertex distances formed once per pair (edge k's |b| is edge k+1's
// |a|).  The three vortexPhi edge angles sum to the triangle's solid angle with the
// opposite sign; from one longSide out, unless the target lies within 1e-12 of its
// distance from the panel plane (where the reference's coplanar branch applies), that sum
// is taken as 2 atan2(a0.(a1 x a2), D) (Van Oosterom and Strackee), one atan2 instead
// of three.  On the test wings the two differ by at most 1.3e-13 there; closer in (up to
// 7e-12 for the nearest neighbours, amplified by the CHTLS weights) the edge sum is kept.
__device__ __forceinline__ void panel_phi_inf_pre(const double* r, const double* ec, dv3 poi, double& phiSrc,
                                                  double& phiDub) {
    dv3 c = ld3(r + R_C);
    dv3 pjk = poi - c;
    double d = norm3(pjk);
    bool itself = d < 1e-10;
    dv3 n = ld3(r + R_N);
    double PN = dot3(pjk, n);
    dv3 p[3] = {ld3(r + R_V0), ld3(r + R_V1), ld3(r + R_V2)};
    dv3 av[3] = {poi - p[0], poi - p[1], poi - p[2]};
    double dn[3] = {norm3(av[0]), norm3(av[1]), norm3(av[2])};
    const bool edge_sum = !itself && (!(fabs(PN) >= 1e-12 * d) || d < r[R_LONG]);
    double ss = 0, dub = 0, phiV = 0, src = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const int i2 = i == 2 ? 0 : i + 1;
        dv3 a = av[i], s = p[i2] - p[i];
        double Al = dot3(n, cross3(s, a));
        const double na = dn[i], nb = dn[i2];
        if (edge_sum) {  // vortex_phi with sm and the norms supplied
            const double eps = 1e-15;
            const dv3 l = ld3(r + R_L);
            double PA = dot3(a, cross3(l, cross3(a, s)));
            double sm = ec[6 + i];
            double PB = PA - Al * sm;
            double num = sm * PN * (nb * PA - na * PB);
            double denom = PA * PB + (PN * PN) * na * nb * (sm * sm);
            if (denom == 0.0 && fabs(PN) < eps)
                phiV = PN >= 0 ? 0.5 * CPG_PI : -0.5 * CPG_PI;
            else
                phiV = atan2(num, denom);
            dub += phiV;
        }
        // src_gl with S and 1/S supplied
        const double S = ec[i];
        double GL = 0;
        if (fabs(na + nb - S) > 0 && S > 0) GL = ec[3 + i] * log(fabs((na + nb + S) / (na + nb - S)));
        if (edge_sum)
            src += Al * GL - PN * phiV;
        else
            ss += Al * GL;
    }
    if (!edge_sum && !itself) {
        const double N3 = dot3(av[0], cross3(av[1], av[2]));
        const double D = dn[0] * dn[1] * dn[2] + dot3(av[0], av[1]) * dn[2] + dot3(av[0], av[2]) * dn[1] +
                         dot3(av[1], av[2]) * dn[0];
        dub = 2 * atan2(N3, D);
        src = ss - PN * dub;
    } else if (itself) {
        src = ss;  // phiV stays 0 for the panel's own centroid
    }
    phiSrc = src / CPG_FOUR_PI;
    phiDub = itself ? -0.5 : dub / CPG_FOUR_PI;
}

// panel::dubPhiInf, CPanel/panel.cpp:208-252
__device__ __forceinline__ double dub_phi_inf(const double* r, dv3 poi) {
    dv3 c = ld3(r + R_C);
    dv3 pjk = poi - c;
    dv3 n = ld3(r + R_N);
    double PN = dot3(pjk, n);
    double d = norm3(pjk);
    if (d < 0.0000001) return -0.5;
    if (d / r[R_LONG] > 5) return PN * r[R_AREA] / (CPG_FOUR_PI * (d * d * d));
    dv3 l = ld3(r + R_L), m = ld3(r + R_M);
    dv3 p[3] = {ld3(r + R_V0), ld3(r + R_V1), ld3(r + R_V2)};
    double phi = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        dv3 p1 = p[i], p2 = p[i == 2 ? 0 : i + 1];
        dv3 a = poi - p1, b = poi - p2, s = p2 - p1;
        double Al = dot3(n, cross3(s, a));
        phi += vortex_phi(PN, Al, a, b, s, l, m);
    }
    return phi / CPG_FOUR_PI;
}

// panel::vortexV, CPanel/panel.cpp:707-711 (core 0.05, panel.h:67)
__device__ __forceinline__ dv3 vortex_v(dv3 a, dv3 b, dv3 s) {
    double na = norm3(a), nb = norm3(b), cs = 0.05 * norm3(s);
    return (double(na + nb) * cross3(a, b)) / (na * nb * (na * nb + dot3(a, b)) + cs * cs);
}

// bodyPanel::panelVInf, CPanel/bodyPanel.cpp:305-348
__device__ __forceinline__ void panel_v_inf(const double* r, dv3 poi, dv3& vSrc, dv3& vDub) {
    dv3 c = ld3(r + R_C);
    dv3 pjk = poi - c;
    dv3 n = ld3(r + R_N);
    double PN = dot3(pjk, n);
    double d = norm3(pjk);
    double area = r[R_AREA];
    if (d / r[R_LONG] > 5) {
        double d3c = d * d * d;
        vSrc = (-1.0) * ((area * pjk) / (CPG_FOUR_PI * d3c));
        vDub = (area * ((3 * dot3(pjk, n)) * pjk - (d * d) * n)) / (CPG_FOUR_PI * (d3c * d * d));
        return;
    }
    dv3 l = ld3(r + R_L), m = ld3(r + R_M);
    dv3 p[3] = {ld3(r + R_V0), ld3(r + R_V1), ld3(r + R_V2)};
    dv3 vs = mk3(0, 0, 0), vd = mk3(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        dv3 p1 = p[i], p2 = p[i == 2 ? 0 : i + 1];
        dv3 a = poi - p1, b = poi - p2, s = a - b;
        double Al = dot3(n, cross3(s, a));
        vd = vd + vortex_v(a, b, s);
        double GL = src_gl(a, b, s);
        double CJK = vortex_phi(PN, Al, a, b, s, l, m);
        vs = vs + (GL * (dot3(s, m) * l - dot3(s, l) * m) + CJK * n);
    }
    vDub = vd / CPG_FOUR_PI;
    vSrc = vs / CPG_FOUR_PI;
}

// panel::dubVInf, CPanel/panel.cpp:666-704 (wake triangles; the edge vector is p2 - p1)
__device__ __forceinline__ dv3 dub_v_inf(const double* r, dv3 poi) {
    dv3 c = ld3(r + R_C);
    dv3 pjk = poi - c;
    dv3 n = ld3(r + R_N);
    double d = norm3(pjk);
    if (d / r[R_LONG] > 5) {
        double d3c = d * d * d;
        return (r[R_AREA] * ((3 * dot3(pjk, n)) * pjk - (d * d) * n)) / (CPG_FOUR_PI * (d3c * d * d));
    }
    dv3 p[3] = {ld3(r + R_V0), ld3(r + R_V1), ld3(r + R_V2)};
    dv3 vd = mk3(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        dv3 p1 = p[i], p2 = p[i == 2 ? 0 : i + 1];
        vd = vd + vortex_v(poi - p1, poi - p2, p2 - p1);
    }
    return vd / CPG_FOUR_PI;
}
