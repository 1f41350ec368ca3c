// Off-body streamlines: streamline::streamline and streamline::rkf (CPanel/streamline.cpp:20-78).
//
// The reference integrates one line at a time with an adaptive Runge-Kutta-Fehlberg 4(5) step and
// evaluates geometry::pntVelocity (a sum over every panel) once per stage.  Here every line advances
// together: each of the six stages gathers the stage points of all live lines and asks the velocity
// field for all of them at once, so that one batched panel-velocity launch serves every line.  Each
// line's own arithmetic (stage points, step weights, error estimate, step-size update, stop test)
// follows the reference's per-line sequence.
#include <cmath>
#include <cstdint>
#include <vector>

#include "streamline.h"

namespace cpg {

int streamlines_rkf45(cpg_velocity_fn fn, void* user, double speed, const double* starts, int n_lines, double x_max,
                      double tol, int max_points, double* pts, double* vel, int32_t* counts, int32_t* ended) {
    // weights of the fifth- and fourth-order solutions (streamline.cpp:24-25)
    static const double c5[6] = {16.0 / 135, 0, 6656.0 / 12825, 28561.0 / 56430, -9.0 / 50, 2.0 / 55};
    static const double c4[6] = {25.0 / 216, 0, 1408.0 / 2565, 2197.0 / 4104, -0.2, 0};
    struct Line {
        double x[3];
        double dt, err;
        double k[6][3];
        bool live;
    };
    std::vector<Line> L((size_t)n_lines);
    for (int i = 0; i < n_lines; i++) {
        for (int c = 0; c < 3; c++) L[i].x[c] = starts[3 * i + c];
        L[i].dt = 0.1 / speed;
        L[i].err = 0;
        for (int j = 0; j < 6; j++)
            for (int c = 0; c < 3; c++) L[i].k[j][c] = 0;
        L[i].live = true;
        counts[i] = 0;
        ended[i] = 0;
    }
    std::vector<int> act;
    std::vector<double> P, V;
    for (bool first = true;; first = false) {
        act.clear();
        for (int i = 0; i < n_lines; i++) {
            Line& l = L[i];
            if (!l.live) continue;
            if (!first) {  // the reference's loop: while (next.x < xMax) { adapt dt; step }
                if (!(l.x[0] < x_max)) {
                    l.live = false;
                    ended[i] = 1;
                    continue;
                }
                if (l.err > 0) l.dt = l.dt * std::pow(tol * l.dt / (2 * l.err), 0.25);
            }
            if (counts[i] >= max_points) {  // out of room: the line stops short of x_max
                l.live = false;
                continue;
            }
            act.push_back(i);
        }
        if (act.empty()) return 0;
        const int64_t m = (int64_t)act.size();
        P.resize(3 * m);
        V.resize(3 * m);
        for (int s = 0; s < 6; s++) {
            for (int64_t a = 0; a < m; a++) {
                const Line& l = L[act[a]];
                for (int c = 0; c < 3; c++) {
                    const double x = l.x[c];
                    const double k0 = l.k[0][c], k1 = l.k[1][c], k2 = l.k[2][c], k3 = l.k[3][c], k4 = l.k[4][c];
                    double y;  // stage points of streamline::rkf, same operations in the same order
                    switch (s) {
                        case 0: y = x; break;
                        case 1: y = x + 1.0 / 4 * k0; break;
                        case 2: y = x + 1.0 / 32 * (3 * k0 + 9.0 * k1); break;
                        case 3: y = x + 1.0 / 2197 * (1932 * k0 - 7200 * k1 + 7296 * k2); break;
                        case 4: y = x + 439.0 / 216 * k0 - 8 * k1 + 3680.0 / 513 * k2 - 845.0 / 4104 * k3; break;
                        default:
                            y = x - 8.0 / 27 * k0 + 2 * k1 - 3544.0 / 2565 * k2 + 1859.0 / 4104 * k3 - 11.0 / 40 * k4;
                    }
                    P[3 * a + c] = y;
                }
            }
            int rc = fn(user, P.data(), m, V.data());
            if (rc != 0) return rc;
            for (int64_t a = 0; a < m; a++) {
                const int i = act[a];
                Line& l = L[i];
                if (s == 0) {  // every step start is recorded with its velocity
                    double* po = pts + 3 * ((int64_t)i * max_points + counts[i]);
                    double* vo = vel + 3 * ((int64_t)i * max_points + counts[i]);
                    for (int c = 0; c < 3; c++) {
                        po[c] = l.x[c];
                        vo[c] = V[3 * a + c];
                    }
                    counts[i]++;
                }
                for (int c = 0; c < 3; c++) l.k[s][c] = l.dt * V[3 * a + c];
            }
        }
        for (int64_t a = 0; a < m; a++) {
            Line& l = L[act[a]];
            double e2 = 0, s5[3];
            for (int c = 0; c < 3; c++) {
                double a5 = 0, a4 = 0;
                for (int j = 0; j < 6; j++) {
                    a5 += c5[j] * l.k[j][c];
                    a4 += c4[j] * l.k[j][c];
                }
                s5[c] = a5;
                e2 += (a5 - a4) * (a5 - a4);
            }
            l.err = std::sqrt(e2);
            for (int c = 0; c < 3; c++) l.x[c] = l.x[c] + s5[c];
        }
    }
}

}  // namespace cpg

extern "C" int cpg_streamlines_field(cpg_velocity_fn fn, void* user, double speed, const double* starts, int n_lines,
                                     double x_max, double tol, int max_points, double* pts, double* vel,
                                     int32_t* counts, int32_t* ended) {
    if (!fn || n_lines < 0 || max_points < 0 || !(speed > 0) || !(tol > 0)) return CPG_E_INVALID;
    if (n_lines > 0 && (!starts || !counts || !ended || (max_points > 0 && (!pts || !vel)))) return CPG_E_INVALID;
    return cpg::streamlines_rkf45(fn, user, speed, starts, n_lines, x_max, tol, max_points, pts, vel, counts, ended);
}
