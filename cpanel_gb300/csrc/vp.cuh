// Device functions of the vortex-particle case: quadrilateral wake panels and the
// panel-to-particle velocity gradients.  Include only from translation units compiled
// with --fmad=false (branch decisions round as the host's do).
#pragma once
#include "common.cuh"
#include "panel64.cuh"

// Packed quad record, must match cpg::QuadField in vpgeom.h.
enum { Q_V0 = 0, Q_C = 12, Q_N = 15, Q_L = 18, Q_M = 21, Q_AREA = 24, Q_LONG = 25, Q_STRIDE = 32 };

struct dm3 {
    double a[3][3];
};
__device__ __forceinline__ dm3 zero_m3() {
    dm3 g;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) g.a[r][c] = 0;
    return g;
}
__device__ __forceinline__ dv3 mul_m3(const dm3& M, dv3 v) {
    return mk3(M.a[0][0] * v.x + M.a[0][1] * v.y + M.a[0][2] * v.z, M.a[1][0] * v.x + M.a[1][1] * v.y + M.a[1][2] * v.z,
               M.a[2][0] * v.x + M.a[2][1] * v.y + M.a[2][2] * v.z);
}

// panel::dubPhiInf for a quad record, CPanel/panel.cpp:208-252
__device__ __forceinline__ double dub_phi_inf_q(const double* q, dv3 poi) {
    dv3 c = ld3(q + Q_C), n = ld3(q + Q_N);
    dv3 pjk = poi - c;
    double PN = dot3(pjk, n);
    double d = norm3(pjk);
    if (d < 0.0000001) return -0.5;
    if (d / q[Q_LONG] > 5) return PN * q[Q_AREA] / (CPG_FOUR_PI * (d * d * d));
    dv3 l = ld3(q + Q_L), m = ld3(q + Q_M);
    double phi = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        dv3 p1 = ld3(q + 3 * i), p2 = ld3(q + 3 * (i == 3 ? 0 : i + 1));
        dv3 a = poi - p1, b = poi - p2, s = p2 - p1;
        double Al = dot3(n, cross3(s, a));
        phi += vortex_phi(PN, Al, a, b, s, l, m);
    }
    return phi / CPG_FOUR_PI;
}

// panel::dubVInf for a quad record, CPanel/panel.cpp:666-704
__device__ __forceinline__ dv3 dub_v_inf_q(const double* q, dv3 poi) {
    dv3 c = ld3(q + Q_C), n = ld3(q + Q_N);
    dv3 pjk = poi - c;
    double d = norm3(pjk);
    if (d / q[Q_LONG] > 5) {
        double d3c = d * d * d;
        return (q[Q_AREA] * ((3 * dot3(pjk, n)) * pjk - (d * d) * n)) / (CPG_FOUR_PI * (d3c * d * d));
    }
    dv3 vd = mk3(0, 0, 0);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        dv3 p1 = ld3(q + 3 * i), p2 = ld3(q + 3 * (i == 3 ? 0 : i + 1));
        vd = vd + vortex_v(poi - p1, poi - p2, p2 - p1);
    }
    return vd / CPG_FOUR_PI;
}

// panel::global2local with translation, CPanel/panel.cpp:183-191
__device__ __forceinline__ dv3 to_local(dv3 c, dv3 l, dv3 m, dv3 n, dv3 g) {
    dv3 t = g - c;
    return mk3(dot3(l, t), dot3(m, t), dot3(n, t));
}

// convexHull(points, true).compareNodes(nodes), CPanel/convexHull.cpp:23-164, for the np
// panel vertices plus the point (pts[np]), all in panel-local coordinates.  The reference
// sorts the reversed range [minBegin, 0) at convexHull.cpp:61 (minEnd is never set):
// undefined behaviour, taken here as an empty sort.
__device__ bool hull_is_nodes(const dv3* pts, int np) {
    const int M = np + 1;
    double mx[5], my[5], mz[5], th[5], dd[5];
    dv3 base = pts[0];
    for (int i = 1; i < M; i++)
        if ((pts[i].y == base.y && pts[i].x < base.x) || (pts[i].y < base.y)) base = pts[i];
    double minT = CPG_PI, maxT = 0;
    int cnt = 0;
    int front = 0;  // members equal to the base go to the front, latest first
    double fx[5], fy[5], fz[5], ft[5], fd[5];
    for (int i = 0; i < M; i++) {
        double t = atan2(pts[i].y - base.y, pts[i].x - base.x);
        double dy = pts[i].y - base.y, dx = pts[i].x - base.x;
        double d = sqrt(dy * dy + dx * dx);
        bool isBase = pts[i].x == base.x && pts[i].y == base.y && pts[i].z == base.z;
        if (!isBase) {
            if (t < minT) minT = t;
            if (t > maxT) maxT = t;
            mx[cnt] = pts[i].x;
            my[cnt] = pts[i].y;
            mz[cnt] = pts[i].z;
            th[cnt] = t;
            dd[cnt] = d;
            cnt++;
        } else {
            fx[front] = pts[i].x;
            fy[front] = pts[i].y;
            fz[front] = pts[i].z;
            ft[front] = t;
            fd[front] = d;
            front++;
        }
    }
    // members = [base copies in reverse insertion order] + [others in order]
    double X[5], Y[5], Z[5], T[5], D[5];
    int k = 0;
    for (int i = front - 1; i >= 0; i--) {
        X[k] = fx[i]; Y[k] = fy[i]; Z[k] = fz[i]; T[k] = ft[i]; D[k] = fd[i];
        k++;
    }
    for (int i = 0; i < cnt; i++) {
        X[k] = mx[i]; Y[k] = my[i]; Z[k] = mz[i]; T[k] = th[i]; D[k] = dd[i];
        k++;
    }
    // stable insertion sort of members[1..] by theta
    for (int i = 2; i < M; i++) {
        double x = X[i], y = Y[i], z = Z[i], t = T[i], d = D[i];
        int j = i;
        while (j > 1 && t < T[j - 1]) {
            X[j] = X[j - 1]; Y[j] = Y[j - 1]; Z[j] = Z[j - 1]; T[j] = T[j - 1]; D[j] = D[j - 1];
            j--;
        }
        X[j] = x; Y[j] = y; Z[j] = z; T[j] = t; D[j] = d;
    }
    int maxBegin = M;
    for (int i = 1; i + 1 < M; i++) {
        if (T[i] == minT) {
        } else if (T[i] == maxT && maxBegin == M) {
            maxBegin = i;
        }
    }
    // stable insertion sort of members[maxBegin..] by distance, descending
    for (int i = maxBegin + 1; i < M; i++) {
        double x = X[i], y = Y[i], z = Z[i], t = T[i], d = D[i];
        int j = i;
        while (j > maxBegin && d > D[j - 1]) {
            X[j] = X[j - 1]; Y[j] = Y[j - 1]; Z[j] = Z[j - 1]; T[j] = T[j - 1]; D[j] = D[j - 1];
            j--;
        }
        X[j] = x; Y[j] = y; Z[j] = z; T[j] = t; D[j] = d;
    }
    // computeHull, then compareNodes
    int hsize = 1;
    bool ok = false;
    // hull[0] = members[0]
    {
        bool found = false;
        for (int q = 0; q < np; q++)
            if (X[0] == pts[q].x && Y[0] == pts[q].y && Z[0] == pts[q].z) found = true;
        ok = found;
    }
    for (int i = 0; i + 1 < M; i++) {
        int i2 = (i == M - 2) ? 0 : i + 2;
        double v1x = X[i + 1] - X[i], v1y = Y[i + 1] - Y[i], v2x = X[i2] - X[i], v2y = Y[i2] - Y[i];
        double crossZ = v1x * v2y - v1y * v2x;
        if (crossZ > 0) {
            hsize++;
            bool found = false;
            for (int q = 0; q < np; q++)
                if (X[i + 1] == pts[q].x && Y[i + 1] == pts[q].y && Z[i + 1] == pts[q].z) found = true;
            ok = ok && found;
        }
    }
    if (hsize > np) return false;
    return ok;
}

// panel::onPanelCheck / inPanelProjection, CPanel/panel.cpp:113-153 (np vertices at v)
// The height test is taken first: the hull is only built when it can matter.
__device__ __forceinline__ bool on_panel_check(const double* v, int np, dv3 c, dv3 n, dv3 l, dv3 m, double longSide,
                                               dv3 poi) {
    dv3 pts[5];
    pts[np] = to_local(c, l, m, n, poi);
    if (!(pts[np].z < 0.05 * longSide)) return false;
    for (int i = 0; i < np; i++) pts[i] = to_local(c, l, m, n, ld3(v + 3 * i));
    return hull_is_nodes(pts, np);
}

// panel::nearFilamentCheck, CPanel/panel.cpp:939-966
__device__ __forceinline__ bool near_filament(dv3 p1, dv3 p2, dv3 poi) {
    const double core = 0.05;
    double el = norm3(p2 - p1);
    double p1d = norm3(p1 - poi), p2d = norm3(p2 - poi);
    if (p1d < core * el || p2d < core * el) return true;
    bool outside = (p1d > el || p2d > el);
    double dist = norm3(cross3(p1 - poi, p2 - poi)) / el;
    return dist < core * el && !outside;
}

// panel::gradDoub, CPanel/panel.cpp:893-937 (rows d/dx, d/dy, d/dz)
__device__ __forceinline__ dm3 grad_doub(dv3 a, dv3 b, dv3 s) {
    const double core = 0.05;
    dm3 G;
    double an = norm3(a), bn = norm3(b);
    dv3 top = (an + bn) * cross3(a, b);
    double cs = core * norm3(s);
    double ab = dot3(a, b);
    double bot = an * bn * (an * bn + ab) + cs * cs;
    const dv3 e[3] = {mk3(1, 0, 0), mk3(0, 1, 0), mk3(0, 0, 1)};
    const double dan[3] = {a.x / an, a.y / an, a.z / an};
    const double dbn[3] = {b.x / bn, b.y / bn, b.z / bn};
#pragma unroll
    for (int r = 0; r < 3; r++) {
        dv3 dtop = (an + bn) * (cross3(e[r], b) + cross3(a, e[r])) + (dan[r] + dbn[r]) * cross3(a, b);
        double dbot = dan[r] * bn * (an * bn + ab) + an * dbn[r] * (an * bn + ab) +
                      an * bn * (dan[r] * bn + an * dbn[r] + dot3(e[r], b) + dot3(a, e[r]));
        dv3 row = (bot * dtop - dbot * top) / (bot * bot);
        G.a[r][0] = row.x;
        G.a[r][1] = row.y;
        G.a[r][2] = row.z;
    }
    return G;
}

// panel::velocityGradientDoublet, CPanel/panel.cpp:852-891 (np vertices at v)
__device__ dm3 vel_grad_doublet(const double* v, int np, dv3 c, dv3 n, dv3 l, dv3 m, double longSide, double mu,
                                dv3 poi) {
    dm3 G = zero_m3();
    bool onPanel = on_panel_check(v, np, c, n, l, m, longSide, poi);
    for (int i = 0; i < np; i++) {
        dv3 p1 = ld3(v + 3 * i), p2 = ld3(v + 3 * (i + 1 < np ? i + 1 : 0));
        dv3 a = poi - p1, b = poi - p2, s = p2 - p1;
        bool nearFil = near_filament(p1, p2, poi);
        if (!nearFil && !onPanel) {
            dm3 g = grad_doub(a, b, s);
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int q = 0; q < 3; q++) G.a[r][q] += g.a[r][q];
        } else if (!nearFil && onPanel) {
            dm3 g = grad_doub(a, b, s);
#pragma unroll
            for (int r = 0; r < 3; r++) G.a[r][2] += g.a[r][2];
        }
    }
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) G.a[r][q] = G.a[r][q] * mu / CPG_FOUR_PI;
    return G;
}

// panel::velocityGradientPointDoublet, CPanel/panel.cpp:818-850
__device__ __forceinline__ dm3 vel_grad_point_doublet(dv3 c, double area, double mu, dv3 poi) {
    dm3 G;
    double x = c.x, y = c.y, z = c.z, x0 = poi.x, y0 = poi.y;
    double dx = x - x0, dy = y - y0;
    double b = dx * dx + dy * dy + z * z;
    double ddd = b * b * b * sqrt(b);
    double uv = 3 * mu * area / CPG_FOUR_PI;
    double w = -mu * area / CPG_FOUR_PI;
    G.a[0][0] = uv * z * (-4 * (dx * dx) + dy * dy + z * z) / ddd;
    G.a[1][0] = uv * (-5) * z * dy * dx / ddd;
    G.a[2][0] = uv * dx * (dx * dx + dy * dy - 4 * z * z) / ddd;
    G.a[0][1] = uv * (-5) * dx * dy * z / ddd;
    G.a[1][1] = uv * z * (dx * dx - 4 * (dy * dy) + z * z) / ddd;
    G.a[2][1] = uv * dy * (dx * dx + dy * dy - 4 * z * z) / ddd;
    G.a[0][2] = w * (-3) * dx * (dx * dx + dy * dy - 4 * z * z) / ddd;
    G.a[1][2] = w * (-3) * dy * (dx * dx + dy * dy - 4 * z * z) / ddd;
    G.a[2][2] = w * (-3) * z * (3 * (dx * dx) + 3 * (dy * dy) - 2 * z * z) / ddd;
    return G;
}

// bodyPanel::velocityGradientPointSource, CPanel/bodyPanel.cpp:732-762
__device__ __forceinline__ dm3 vel_grad_point_source(dv3 c, double area, double sigma, dv3 poi) {
    dm3 G;
    double x = c.x, y = c.y, z = c.z, x0 = poi.x, y0 = poi.y, z0 = poi.z;
    double dx = x - x0, dy = y - y0;
    double b = dx * dx + dy * dy + z * z;
    double sdd = b * b * sqrt(b);
    double k = sigma * area / CPG_FOUR_PI;
    G.a[0][0] = (-2 * dx * dx + dy * dy + z * z) / sdd;
    G.a[1][0] = -3 * dx * dy / sdd;
    G.a[2][0] = -3 * dx * z / sdd;
    G.a[0][1] = -3 * dx * dy / sdd;
    G.a[1][1] = (dx * dx - dy * dy + z * z) / sdd;
    G.a[2][1] = -3 * z * dy / sdd;
    G.a[0][2] = -3 * dx * (z - z0) / sdd;
    G.a[1][2] = -3 * dy * (z - z0) / sdd;
    G.a[2][2] = (-3 * z * (z - z0) + (dx * dx + dy * dy + z * z)) / sdd;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) G.a[r][q] *= k;
    return G;
}

// bodyPanel::velocityGradientTriSource, CPanel/bodyPanel.cpp:929-1063 (r: body record)
__device__ dm3 vel_grad_tri_source(const double* r, double sigma, dv3 poi) {
    dv3 c = ld3(r + R_C), n = ld3(r + R_N), l = ld3(r + R_L), m = ld3(r + R_M);
    dv3 n1 = to_local(c, l, m, n, ld3(r + R_V0)), n2 = to_local(c, l, m, n, ld3(r + R_V1)),
        n3 = to_local(c, l, m, n, ld3(r + R_V2));
    dv3 pl = to_local(c, l, m, n, poi);
    const double x1 = n1.x, x2 = n2.x, x3 = n3.x, y1 = n1.y, y2 = n2.y, y3 = n3.y;
    const double x = pl.x, y = pl.y, z = pl.z;
    const double k = sigma / CPG_FOUR_PI;
    double d12 = sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
    double d23 = sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2));
    double d31 = sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3));
    double r1 = sqrt((x - x1) * (x - x1) + (y - y1) * (y - y1) + z * z);
    double r2 = sqrt((x - x2) * (x - x2) + (y - y2) * (y - y2) + z * z);
    double r3 = sqrt((x - x3) * (x - x3) + (y - y3) * (y - y3) + z * z);
    double dr1[3] = {(x - x1) / r1, (y - y1) / r1, z / r1};
    double dr2[3] = {(x - x2) / r2, (y - y2) / r2, z / r2};
    double dr3[3] = {(x - x3) / r3, (y - y3) / r3, z / r3};
    double m12 = (y2 - y1) / (x2 - x1), m23 = (y3 - y2) / (x3 - x2), m31 = (y1 - y3) / (x1 - x3);
    double e1 = (x - x1) * (x - x1) + z * z, e2 = (x - x2) * (x - x2) + z * z, e3 = (x - x3) * (x - x3) + z * z;
    double h1 = (x - x1) * (y - y1), h2 = (x - x2) * (y - y2), h3 = (x - x3) * (y - y3);
    // d/dk of (e, h) per vertex: e = (x-xi)^2 + z^2, h = (x-xi)(y-yi)
    double de1[3] = {2 * (x - x1), 0, 2 * z}, de2[3] = {2 * (x - x2), 0, 2 * z}, de3[3] = {2 * (x - x3), 0, 2 * z};
    double dh1[3] = {(y - y1), (x - x1), 0}, dh2[3] = {(y - y2), (x - x2), 0}, dh3[3] = {(y - y3), (x - x3), 0};
    auto lt = [](double dyv, double ra, double rb, double d, double da, double db) {
        double s = ra + rb + d;
        return dyv * s * (da + db) * (2 * d) / (d) / (ra + rb - d) / (s * s);
    };
    auto at = [&](double mm, double e, double h, double rr, double dnum, double dden) {
        double f = (mm * e - h) / (z * rr);
        double zr = z * rr;
        return (1 / (1 + f * f)) * ((zr * dnum - (mm * e - h) * dden) / (zr * zr));
    };
    dm3 G;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        G.a[q][0] = lt(y2 - y1, r1, r2, d12, dr1[q], dr2[q]) + lt(y3 - y2, r2, r3, d23, dr2[q], dr3[q]) +
                    lt(y1 - y3, r3, r1, d31, dr3[q], dr1[q]);
        G.a[q][1] = lt(x1 - x2, r1, r2, d12, dr1[q], dr2[q]) + lt(x2 - x3, r2, r3, d23, dr2[q], dr3[q]) +
                    lt(x3 - x1, r3, r1, d31, dr3[q], dr1[q]);
    }
    // column 2 (dw/dk): d/dk (z r) is z dr/dk, plus r for k = z
    double dzr1[3] = {z * dr1[0], z * dr1[1], r1 + z * dr1[2]};
    double dzr2[3] = {z * dr2[0], z * dr2[1], r2 + z * dr2[2]};
    double dzr3[3] = {z * dr3[0], z * dr3[1], r3 + z * dr3[2]};
#pragma unroll
    for (int q = 0; q < 3; q++) {
        G.a[q][2] = at(m12, e1, h1, r1, m12 * de1[q] - dh1[q], dzr1[q]) - at(m12, e2, h2, r2, m12 * de2[q] - dh2[q], dzr2[q]) +
                    at(m23, e2, h2, r2, m23 * de2[q] - dh2[q], dzr2[q]) - at(m23, e3, h3, r3, m23 * de3[q] - dh3[q], dzr3[q]) +
                    at(m31, e3, h3, r3, m31 * de3[q] - dh3[q], dzr3[q]) - at(m31, e1, h1, r1, m31 * de1[q] - dh1[q], dzr1[q]);
    }
#pragma unroll
    for (int r_ = 0; r_ < 3; r_++)
#pragma unroll
        for (int q = 0; q < 3; q++) G.a[r_][q] *= k;
    return G;
}
