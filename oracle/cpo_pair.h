/*
 * cpo_pair.h -- particle pair kernels of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 * particle::velInflAlgSmooth / velInfl / vortexStretching / viscousDiffusion,
 * CPanel/particle.cpp:31-140, in FP64 and the reference's evaluation order.
 */
#pragma once
#include <cmath>
#include <cstdint>

namespace cpo_pair {
constexpr double kPi = 3.14159265358979323846;
constexpr double kCore = 1.5;  // particle::coreOverlap, CPanel/particle.h:32
constexpr int kMaxLevel = 32;  // deepest node level that may be split is kMaxLevel - 1

struct P3 {
    double x = 0, y = 0, z = 0;
};
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 add(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 scl(double s, P3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double nrm(P3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline P3 crs(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline P3 ld(const double* p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

struct Part {
    P3 pos, str;
    double rad;
};

/* particle::velInflAlgSmooth, CPanel/particle.cpp:31-38 */
inline P3 velAlg(const Part& s, P3 poi) {
    double sigma = kCore * s.rad;
    P3 dist = sub(poi, s.pos);
    double r = nrm(dist);
    double f = -1 / (4 * kPi) * (std::pow(r, 2) + 2.5 * std::pow(sigma, 2)) /
               (std::pow(std::pow(r, 2) + std::pow(sigma, 2), 2.5));
    return scl(f, crs(dist, s.str));
}

inline double gaussK(double rho) {
    return (1 / (4 * kPi * rho) * std::erf(rho / std::pow(2, 0.5)) -
            1 / (std::pow(2 * kPi, 1.5)) * std::exp(-0.5 * rho * rho)) /
           (rho * rho);
}

/* particle::velInfl(particle*), CPanel/particle.cpp:42-58: velocity at t due to s */
inline P3 velGaussPart(const Part& s, const Part& t) {
    double sigma = std::sqrt(std::pow(kCore * s.rad, 2) + std::pow(kCore * t.rad, 2)) / std::sqrt(2);
    P3 dist = sub(t.pos, s.pos);
    double rho = nrm(dist) / sigma;
    double K = gaussK(rho);
    return scl(-1 / std::pow(sigma, 3) * K, crs(dist, s.str));
}

/* particle::velInfl(POI), CPanel/particle.cpp:60-77 */
inline P3 velGaussPoint(const Part& s, P3 poi) {
    if (nrm(sub(s.pos, poi)) == 0) return {0, 0, 0};
    double sigma = kCore * s.rad;
    P3 dist = sub(poi, s.pos);
    double rho = nrm(dist) / sigma;
    double K = gaussK(rho);
    return scl(-1 / std::pow(sigma, 3) * K, crs(dist, s.str));
}

/* particle::vortexStretching, CPanel/particle.cpp:80-118 (this = s, part = t) */
inline P3 stretch(const Part& s, const Part& t) {
    P3 Xi = s.pos, Xj = t.pos;
    P3 d = sub(Xi, Xj);
    if (nrm(d) > 5 * s.rad) return {0, 0, 0};
    double sig = std::sqrt(std::pow(kCore * s.rad, 2) + std::pow(kCore * t.rad, 2)) / std::sqrt(2);
    double rho = nrm(d) / sig;
    double xi = 1 / (std::pow(2 * kPi, 1.5)) * std::exp(-rho * rho / 2);
    double G = 1 / (4 * kPi * rho) * std::erf(rho / std::sqrt(2));
    double K = (G - xi) / (rho * rho);
    double F = (3 * K - xi) / (rho * rho);
    double dv[3] = {d.x, d.y, d.z};
    double M[3][3];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++)
            M[k][l] = (k == l) ? K - 1 / (sig * sig) * F * dv[k] * dv[l] : -1 / (sig * sig) * F * dv[k] * dv[l];
    P3 a = t.str;
    double At[3][3] = {{0, -a.z, a.y}, {a.z, 0, -a.x}, {-a.y, a.x, 0}};
    double c = 1 / std::pow(sig, 3);
    double G3[3][3];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
            double acc = 0;
            for (int q = 0; q < 3; q++) acc += (c * At[k][q]) * M[q][l];
            G3[k][l] = acc;
        }
    double sv[3] = {s.str.x, s.str.y, s.str.z}, o[3];
    for (int k = 0; k < 3; k++) o[k] = G3[k][0] * sv[0] + G3[k][1] * sv[1] + G3[k][2] * sv[2];
    return {o[0], o[1], o[2]};
}

/* particle::viscousDiffusion, CPanel/particle.cpp:122-140 (this = s, part = t) */
inline P3 diffusion(const Part& s, const Part& t) {
    const double nu = 1.983e-5;
    double sig = std::sqrt(std::pow(kCore * s.rad, 2) + std::pow(kCore * t.rad, 2)) / std::sqrt(2);
    double rho = nrm(sub(s.pos, t.pos)) / sig;
    double Vi = 4 * kPi / 3 * std::pow(s.rad, 3);
    double Vj = 4 * kPi / 3 * std::pow(t.rad, 3);
    double xi = 1 / (std::pow(2 * kPi, 1.5) * std::pow(rho, 3)) * std::exp(-rho * rho / 2);
    double f = 2 * nu / (sig * sig) * xi;
    return scl(f, sub(scl(Vi, t.str), scl(Vj, s.str)));
}

}  // namespace cpo_pair
