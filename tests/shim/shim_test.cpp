// C++ caller of the drop-in shim (include/cpanel_shim.hpp), linked against libcpanel_gb300.so.
// It drives the library the way CPanel's own classes drive the hot path:
//   1. bodyPanel::panelPhiInf / dubPhiInf on the unit triangle of the reference's influence test
//      (CPanelTests/influenceTests.cpp:579-664: near and far point, collocation self term);
//   2. geometry::readTri + setInfCoeff + getA/getB and cpCase::solveMatrixEq on the reference's
//      4412 case, as cpCase::run uses them (CPanel/cpCase.cpp:185-214): the doublet strengths and
//      Cp of every panel against the reference's surfaceData-0.vtu (6 significant digits), CL and
//      CDi against its .CPout (5 decimals), and the solved system's residual |A mu + B sigma|
//      computed here from the matrices getA/getB return;
//   3. particle::velInfl / vortexStretching / viscousDiffusion and particleFMM::build /
//      barnesHutVel / barnesHutStretch / barnesHutDiff against the CPU oracle's values.
// argv[1]: a directory holding mesh4412.tri, case4412.bin and particles.bin (written by
// tests/test_shim.py).  Prints one line per check; exit status 0 when every check passes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "cpanel_shim.hpp"

using cpg::shim::Vector3d;

static int failures = 0;

static void expect(bool ok, const char* what, double got, double want) {
    std::printf("%s %s: %.9g (expected %.9g)\n", ok ? "ok  " : "FAIL", what, got, want);
    if (!ok) failures++;
}

static std::vector<double> read_doubles(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    std::vector<double> v;
    double x;
    while (f.read(reinterpret_cast<char*>(&x), sizeof x)) v.push_back(x);
    return v;
}

// |ours - ref| within half a unit of the 6th significant digit of ref (+ float32 storage)
static bool printed(double ours, double ref) { return std::fabs(ours - ref) <= 5.1e-6 * std::fabs(ref) + 1e-12; }

static void unit_triangle() {
    cpg::shim::bodyPanel p(Vector3d(1, 0, 0), Vector3d(-1, 1, 0), Vector3d(-1, -1, 0));
    double src = 0, dub = 0;
    p.panelPhiInf(Vector3d(2, 2, 2), src, dub);
    expect(std::fabs(src - 0.043411) < 1e-5, "near point phi source", src, 0.043411);
    expect(std::fabs(dub - 0.006645) < 1e-5, "near point phi doublet", dub, 0.006645);
    expect(std::fabs(p.dubPhiInf(Vector3d(2, 2, 2)) - dub) < 1e-15, "dubPhiInf = panelPhiInf doublet",
           p.dubPhiInf(Vector3d(2, 2, 2)), dub);
    src = dub = 0;
    p.panelPhiInf(Vector3d(7, 7, 7), src, dub);
    expect(std::fabs(src - 0.012919) < 1e-5, "far point phi source", src, 0.012919);
    expect(std::fabs(dub - 0.0005958) < 1e-5, "far point phi doublet", dub, 0.0005958);
    src = dub = 0;
    p.panelPhiInf(Vector3d(-1.0 / 3, 0, 0), src, dub);
    expect(dub == -0.5, "collocation self term", dub, -0.5);
}

static void case4412(const std::string& dir) {
    const std::vector<double> c = read_doubles(dir + "/case4412.bin");
    const int64_t n = (int64_t)c[0];
    const double V = c[1], alpha = c[2], beta = c[3], mach = c[4], Sref = c[5], bref = c[6], cref = c[7];
    const double cg[3] = {c[8], c[9], c[10]};
    const double CL = c[11], CDi = c[12];
    const double* mu_ref = c.data() + 13;
    const double* cp_ref = mu_ref + n;
    std::unique_ptr<cpg::shim::geometry> geom = cpg::shim::geometry::readTri(dir + "/mesh4412.tri");
    expect(geom->nBodyPanels() == n, "body panels", (double)geom->nBodyPanels(), (double)n);
    geom->setInfCoeff();
    cpg::shim::Matrix* A = geom->getA();
    cpg::shim::Matrix* B = geom->getB();
    cpg::shim::cpCase cs(geom.get(), V, alpha, beta, mach, Sref, bref, cref, cg);
    expect(cs.solveMatrixEq(), "solveMatrixEq converged", 1, 1);
    const std::vector<double>& mu = cs.getMu();
    const std::vector<double>& sigma = cs.getSigma();
    const std::vector<double>& cp = cs.getCp();
    int64_t bad_mu = 0, bad_cp = 0;
    for (int64_t i = 0; i < n; i++) {
        bad_mu += !printed(mu[i], mu_ref[i]);
        bad_cp += !printed(cp[i], cp_ref[i]);
    }
    expect(bad_mu == 0, "panels whose doublet strength misses the reference's digits", (double)bad_mu, 0);
    expect(bad_cp == 0, "panels whose Cp misses the reference's digits", (double)bad_cp, 0);
    expect(std::fabs(cs.getCL() - CL) <= 0.5e-5 + 1e-12, "CL (Trefftz plane)", cs.getCL(), CL);
    expect(std::fabs(cs.getCD() - CDi) <= 0.5e-5 + 1e-12, "CDi (Trefftz plane)", cs.getCD(), CDi);
    // the solved system, from the matrices getA/getB return: A mu = -B sigma (cpCase.cpp:192-199)
    double r2 = 0, b2 = 0;
    for (int64_t i = 0; i < n; i++) {
        double am = 0, bs = 0;
        for (int64_t j = 0; j < n; j++) {
            am += (*A)(i, j) * mu[j];
            bs += (*B)(i, j) * sigma[j];
        }
        r2 += (am + bs) * (am + bs);
        b2 += bs * bs;
    }
    const double rel = std::sqrt(r2 / b2);
    expect(rel < 1e-9, "relative residual |A mu + B sigma| / |B sigma|", rel, 0);
}

static void particles(const std::string& dir) {
    const std::vector<double> d = read_doubles(dir + "/particles.bin");
    const int64_t n = (int64_t)d[0], m = (int64_t)d[1];
    const double* pos = d.data() + 2;
    const double* str = pos + 3 * n;
    const double* rad = str + 3 * n;
    const double* pts = rad + n;
    const double* e_pts = pts + 3 * m;      // barnesHutVel at the points
    const double* e_vel = e_pts + 3 * m;    // barnesHutVel / Stretch / Diff per particle
    const double* e_str = e_vel + 3 * n;
    const double* e_dif = e_str + 3 * n;
    const double* e_pair = e_dif + 3 * n;   // velInfl(part), vortexStretching(part), viscousDiffusion(part),
                                            // velInfl(POI), velInflAlgSmooth(POI) of particles 0 and 1
    std::vector<cpg::shim::particle> parts;
    parts.reserve((size_t)n);
    for (int64_t i = 0; i < n; i++)
        parts.emplace_back(Vector3d(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                           Vector3d(str[3 * i], str[3 * i + 1], str[3 * i + 2]), rad[i]);
    std::vector<cpg::shim::particle*> ptrs;
    for (auto& p : parts) ptrs.push_back(&p);
    cpg::shim::particleOctree tree;
    tree.setMaxMembers(10);
    tree.addData(ptrs);
    cpg::shim::particleFMM fmm;
    fmm.build(&tree);
    auto worst = [](const double* got, const double* want, int64_t k) {
        double e = 0, s = 0;
        for (int64_t i = 0; i < k; i++) {
            e = std::max(e, std::fabs(got[i] - want[i]));
            s = std::max(s, std::fabs(want[i]));
        }
        return e / (s > 0 ? s : 1);
    };
    std::vector<double> got((size_t)(3 * std::max(n, m)));
    for (int64_t j = 0; j < m; j++) {
        const Vector3d v = fmm.barnesHutVel(Vector3d(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]));
        for (int q = 0; q < 3; q++) got[3 * j + q] = v(q);
    }
    double e = worst(got.data(), e_pts, 3 * m);
    expect(e < 1e-12, "particleFMM::barnesHutVel(POI) vs oracle (relative)", e, 0);
    const double* exp3[3] = {e_vel, e_str, e_dif};
    const char* names[3] = {"particleFMM::barnesHutVel(part)", "particleFMM::barnesHutStretch",
                            "particleFMM::barnesHutDiff"};
    for (int w = 0; w < 3; w++) {
        for (int64_t i = 0; i < n; i++) {
            const Vector3d v = w == 0 ? fmm.barnesHutVel(ptrs[i]) : w == 1 ? fmm.barnesHutStretch(ptrs[i])
                                                                            : fmm.barnesHutDiff(ptrs[i]);
            for (int q = 0; q < 3; q++) got[3 * i + q] = v(q);
        }
        e = worst(got.data(), exp3[w], 3 * n);
        expect(e < 1e-12, names[w], e, 0);
    }
    const Vector3d poi(pts[0], pts[1], pts[2]);
    const Vector3d pair[5] = {parts[0].velInfl(ptrs[1]), parts[0].vortexStretching(ptrs[1]),
                              parts[0].viscousDiffusion(ptrs[1]), parts[0].velInfl(poi),
                              parts[0].velInflAlgSmooth(poi)};
    const char* pnames[5] = {"particle::velInfl(part)", "particle::vortexStretching", "particle::viscousDiffusion",
                             "particle::velInfl(POI)", "particle::velInflAlgSmooth"};
    for (int w = 0; w < 5; w++) {
        for (int q = 0; q < 3; q++) got[q] = pair[w](q);
        e = worst(got.data(), e_pair + 3 * w, 3);
        expect(e < 1e-12, pnames[w], e, 0);
    }
    const Vector3d self = parts[0].velInfl(ptrs[0]);
    expect(self.norm() == 0, "a particle does not influence itself", self.norm(), 0);
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <data dir>\n", argv[0]);
        return 2;
    }
    try {
        unit_triangle();
        case4412(argv[1]);
        particles(argv[1]);
    } catch (const cpg::shim::error& e) {
        std::printf("FAIL shim error %d: %s\n", e.status, e.what());
        return 1;
    }
    std::printf("%s: %d failed checks\n", failures ? "FAILED" : "shim ok", failures);
    return failures ? 1 : 0;
}
