/*
 * cpanel_shim.hpp -- C++ drop-in shim of CPanel's hot-path interfaces over the C ABI
 * (cpanel_gpu.h, cpanel_vp.h).
 *
 * Code written against CPanel's classes keeps its call sites: the classes below carry the
 * reference's names and member signatures for the hot path, and run it on the GB300 library.
 *
 *   shim class / member                      replaces (paths relative to the CPanel project)
 *   bodyPanel::panelPhiInf(POI, src, dub)    CPanel/bodyPanel.h:98, bodyPanel.cpp:132-190
 *   bodyPanel::panelV(POI)                   CPanel/bodyPanel.h:96, bodyPanel.cpp:122-130
 *   bodyPanel::dubPhiInf(POI)                CPanel/panel.h:98, panel.cpp:208-252
 *   geometry::readTri / setInfCoeff /        CPanel/geometry.h:253,310-311, geometry.cpp:132-891
 *     getA / getB
 *   cpCase::solveMatrixEq / run / getCL ...  CPanel/cpCase.h:84,140-147, cpCase.cpp:185-214
 *   particle::velInfl(POI), velInfl(part),   CPanel/particle.h:56-62, particle.cpp:31-140
 *     velInflAlgSmooth, vortexStretching,
 *     viscousDiffusion
 *   particleOctree::addData / removeData /   octree/include/octree.h:151-195
 *     setMaxMembers
 *   particleFMM::build / barnesHutVel /      CPanel/particleFMM.h:52-56, particleFMM.cpp:22-116
 *     barnesHutStretch / barnesHutDiff
 *
 * Vectors: the members are templates over the caller's 3-vector type V (anything with
 * V(x, y, z) and v(i) -- Eigen::Vector3d included) and default to shim::Vector3d; the library
 * underneath takes plain doubles, so no Eigen is needed to build or link it.
 *
 * Costs: a single-point call (panelPhiInf, velInfl(POI), ...) is one small device round trip,
 * as correct as the batched calls but far slower per point; the batched members take many
 * points per call.  particleFMM evaluates every particle's velocity, stretching and diffusion
 * in one traversal on the first per-particle query after build() and answers the others from
 * that table.  Errors throw shim::error with the library's status and message (the reference
 * exits instead).
 */
#ifndef CPANEL_SHIM_HPP
#define CPANEL_SHIM_HPP

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "cpanel_gpu.h"
#include "cpanel_vp.h"

namespace cpg {
namespace shim {

constexpr double kShimPi = 3.14159265358979323846;

struct error : std::runtime_error {
    int status;
    error(int st, const std::string& what) : std::runtime_error(what), status(st) {}
};

struct Vector3d {
    double d[3] = {0, 0, 0};
    Vector3d() = default;
    Vector3d(double x, double y, double z) : d{x, y, z} {}
    double x() const { return d[0]; }
    double y() const { return d[1]; }
    double z() const { return d[2]; }
    double operator()(int i) const { return d[i]; }
    double& operator()(int i) { return d[i]; }
    double norm() const { return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]); }
    template <class V>
    V as() const {  // to the caller's vector type, e.g. as<Eigen::Vector3d>()
        return V(d[0], d[1], d[2]);
    }
};

// point arguments: any vector type, pointers excluded (those are particles)
template <class V>
using point_t = typename std::enable_if<!std::is_pointer<V>::value, V>::type;

template <class V>
inline void to3(const V& v, double* out) {
    out[0] = v(0);
    out[1] = v(1);
    out[2] = v(2);
}
template <class V>
inline V from3(const double* p) {
    return V(p[0], p[1], p[2]);
}

// The device context the shim objects use: one per device, created on first use.
cpg_ctx* context(int device = 0);
// throws shim::error unless status is CPG_OK
void check(int status, cpg_ctx* ctx, const char* what);

// ---- influence functions of one triangle ----------------------------------------------------
// core (plain doubles): verts 9 doubles (3 vertices), m points
void tri_phi_inf(const double* verts, const double* poi, int64_t m, double* phi_src, double* phi_dub);
void tri_dub_phi_inf(const double* verts, const double* poi, int64_t m, double* phi_dub);
void tri_v_inf(const double* verts, const double* poi, int64_t m, double* v_src, double* v_dub);

class bodyPanel {
  public:
    template <class V>
    bodyPanel(const V& p0, const V& p1, const V& p2) {
        to3(p0, v_);
        to3(p1, v_ + 3);
        to3(p2, v_ + 6);
        geom();
    }
    void setSigma(double s) { sigma_ = s; }
    void setMu(double m) { mu_ = m; }
    double getSigma() const { return sigma_; }
    double getMu() const { return mu_; }
    double getLongSide() const { return longSide_; }

    // The reference's semantics: beyond five panel lengths the point source and doublet are
    // assigned to phiSrc and phiDub; closer in, the edge sums are added to what the caller
    // passes and the totals divided by 4 pi, and the panel's own centroid gets phiDub = -0.5.
    template <class V>
    void panelPhiInf(const V& POI, double& phiSrc, double& phiDub) const {
        static_assert(!std::is_pointer<V>::value, "POI is a point");
        double p[3], s, d;
        to3(POI, p);
        tri_phi_inf(v_, p, 1, &s, &d);
        const double r = dist(p);
        if (r / longSide_ > 5) {
            phiSrc = s;
            phiDub = d;
        } else {
            phiSrc = phiSrc / (4 * kShimPi) + s;
            phiDub = r < 1e-10 ? -0.5 : phiDub / (4 * kShimPi) + d;
        }
    }
    // sigma vSrc + mu vDub at POI (the panel's own strengths, setSigma / setMu)
    template <class V>
    V panelV(const V& POI) const {
        double p[3], vs[3], vd[3];
        to3(POI, p);
        tri_v_inf(v_, p, 1, vs, vd);
        return V(sigma_ * vs[0] + mu_ * vd[0], sigma_ * vs[1] + mu_ * vd[1], sigma_ * vs[2] + mu_ * vd[2]);
    }
    template <class V>
    double dubPhiInf(const V& POI) const {
        double p[3], d;
        to3(POI, p);
        tri_dub_phi_inf(v_, p, 1, &d);
        return d;
    }
    // batched: m points (m x 3), outputs m (assigned, as for a caller that zeroes first)
    void panelPhiInf(const double* poi, int64_t m, double* phiSrc, double* phiDub) const {
        tri_phi_inf(v_, poi, m, phiSrc, phiDub);
    }
    const double* verts() const { return v_; }

  private:
    void geom();
    double dist(const double* p) const {
        const double a = p[0] - c_[0], b = p[1] - c_[1], c = p[2] - c_[2];
        return std::sqrt(a * a + b * b + c * c);
    }
    double v_[9];
    double c_[3];
    double longSide_ = 0;
    double sigma_ = 0, mu_ = 0;
};

// ---- geometry and the steady case -------------------------------------------------------------
// Column-major matrix as Eigen stores it: A(i, j) = data()[j * rows() + i].
class Matrix {
  public:
    Matrix() = default;
    Matrix(int64_t r, int64_t c) : r_(r), c_(c), d_((size_t)(r * c)) {}
    int64_t rows() const { return r_; }
    int64_t cols() const { return c_; }
    double operator()(int64_t i, int64_t j) const { return d_[(size_t)(j * r_ + i)]; }
    double* data() { return d_.data(); }
    const double* data() const { return d_.data(); }

  private:
    int64_t r_ = 0, c_ = 0;
    std::vector<double> d_;
};

class geometry {
  public:
    // geometry::readTri on arrays: nodes n x 3, tris m x 3 (1-based), surface ids (>1000: wake)
    geometry(const double* nodes, int64_t n_nodes, const int64_t* tris, const int32_t* ids, int64_t n_tris,
             int device = 0);
    // geometry::readTri of a Cart3D .tri file
    static std::unique_ptr<geometry> readTri(const std::string& path, int device = 0);
    ~geometry();
    geometry(const geometry&) = delete;
    geometry& operator=(const geometry&) = delete;

    void setInfCoeff();      // FP64 A and B on the device (the reference method)
    Matrix* getA();          // host copies, fetched on first use after setInfCoeff
    Matrix* getB();
    int64_t nBodyPanels() const { return n_; }
    // per body panel in matrix order: centroid, unit normal (bezier normal of the panel)
    const std::vector<double>& centers() const { return cen_; }
    const std::vector<double>& normals() const { return nrm_; }
    cpg_geometry* handle() { return g_; }
    cpg_ctx* ctx() { return ctx_; }

  private:
    cpg_ctx* ctx_ = nullptr;
    cpg_geometry* g_ = nullptr;
    int64_t n_ = 0;
    bool assembled_ = false;
    std::unique_ptr<Matrix> A_, B_;
    std::vector<double> cen_, nrm_;
};

class cpCase {
  public:
    // one flow condition (V, degrees, Mach) and the reference quantities of the coefficients
    cpCase(geometry* geom, double V, double alpha, double beta, double mach, double Sref, double bref, double cref,
           const double cg[3], bool mixed = false);
    // setSourceStrengths + solveMatrixEq (RHS = -B sigma, BiCGSTAB) and the post-processing;
    // true when the solve reached the reference's tolerance
    bool solveMatrixEq();
    void run() { solveMatrixEq(); }
    double getCL() const { return CL_; }
    double getCD() const { return CDi_; }
    const std::vector<double>& getMu() const { return mu_; }
    const std::vector<double>& getSigma() const { return sigma_; }
    const std::vector<double>& getCp() const { return cp_; }
    const double* getBodyForces() const { return Fb_; }
    const double* getWindForces() const { return Fw_; }
    const double* getMoment() const { return CM_; }

  private:
    geometry* geom_;
    cpg_flow flow_;
    cpg_refs refs_;
    bool mixed_;
    std::vector<double> mu_, sigma_, cp_;
    double CL_ = 0, CDi_ = 0, Fb_[3] = {0, 0, 0}, Fw_[3] = {0, 0, 0}, CM_[3] = {0, 0, 0};
};

// ---- vortex particles -------------------------------------------------------------------------
// core: the Gaussian (CPG_VEL_GAUSS) or algebraic (CPG_VEL_ALG) velocity of particles at points
void particles_velocity_at(const double* pos, const double* strength, const double* radius, int64_t n,
                           const double* pts, int64_t m, int kernel, double* vel);
// the symmetrised-core velocity (particle::velInfl(particle*)), stretching and diffusion on each
// of n particles from all the others (any output may be null)
void particles_mutual(const double* pos, const double* strength, const double* radius, int64_t n, double* vel,
                      double* stretch, double* diff);

class particle {
  public:
    template <class V>
    particle(const V& p, const V& s, double r, int shed = 0) : radius(r), shedTime(shed) {
        to3(p, pos_);
        to3(s, str_);
    }
    template <class V = Vector3d>
    V getPos() const {
        return from3<V>(pos_);
    }
    template <class V = Vector3d>
    V getStrength() const {
        return from3<V>(str_);
    }
    template <class V>
    void setPos(const V& p) {
        to3(p, pos_);
    }
    template <class V>
    void setStrength(const V& s) {
        to3(s, str_);
    }
    // velocity this particle induces at POI (Gaussian core 1.5 r) / at part (symmetrised core)
    template <class V>
    point_t<V> velInfl(const V& POI) const {
        double p[3], v[3];
        to3(POI, p);
        particles_velocity_at(pos_, str_, &radius, 1, p, 1, CPG_VEL_GAUSS, v);
        return from3<V>(v);
    }
    Vector3d velInfl(const particle* part) const {
        Vector3d v;
        pair(part, 0, v.d);
        return v;
    }
    template <class V>
    point_t<V> velInflAlgSmooth(const V& POI) const {
        double p[3], v[3];
        to3(POI, p);
        particles_velocity_at(pos_, str_, &radius, 1, p, 1, CPG_VEL_ALG, v);
        return from3<V>(v);
    }
    Vector3d vortexStretching(const particle* part) const {
        Vector3d v;
        pair(part, 1, v.d);
        return v;
    }
    Vector3d viscousDiffusion(const particle* part) const {
        Vector3d v;
        pair(part, 2, v.d);
        return v;
    }
    const double* pos() const { return pos_; }
    const double* strength() const { return str_; }

    double radius;
    int shedTime;

  private:
    void pair(const particle* part, int what, double* out) const;
    double pos_[3], str_[3];
};

// particleOctree: the particle set the FMM is built on (the reference's octree stores the
// pointers; the tree itself is built by particleFMM::build with the reference's rules)
class particleOctree {
  public:
    void setMaxMembers(int m) { maxMembers_ = m; }
    void addData(const std::vector<particle*>& parts) { parts_.insert(parts_.end(), parts.begin(), parts.end()); }
    void removeData() { parts_.clear(); }
    const std::vector<particle*>& data() const { return parts_; }
    int maxMembers() const { return maxMembers_; }

  private:
    std::vector<particle*> parts_;
    int maxMembers_ = 10;
};

class particleFMM {
  public:
    explicit particleFMM(int device = 0, double theta = 0.5) : device_(device), theta_(theta) {}
    ~particleFMM();
    particleFMM(const particleFMM&) = delete;
    particleFMM& operator=(const particleFMM&) = delete;

    // the octree and its expansions for the tree's particles as they are now
    void build(particleOctree* tree);
    template <class V>
    point_t<V> barnesHutVel(const V& POI) {
        double p[3], v[3];
        to3(POI, p);
        velocity_points(p, 1, v);
        return from3<V>(v);
    }
    Vector3d barnesHutVel(const particle* part) { return from3<Vector3d>(row(part, 0)); }
    Vector3d barnesHutStretch(const particle* part) { return from3<Vector3d>(row(part, 1)); }
    Vector3d barnesHutDiff(const particle* part) { return from3<Vector3d>(row(part, 2)); }
    // batched: velocity at m points
    void velocity_points(const double* pts, int64_t m, double* vel);

  private:
    const double* row(const particle* part, int what);
    void release();
    int device_;
    double theta_;
    cpg_ptree* tree_ = nullptr;
    void* dev_ = nullptr;  // device copies of the particles (pos, strength, radius)
    int64_t n_ = 0;
    std::unordered_map<const particle*, int64_t> index_;
    std::vector<double> table_;  // n x 9: velocity, stretching, diffusion
    bool have_table_ = false;
};

}  // namespace shim
}  // namespace cpg

#endif /* CPANEL_SHIM_HPP */
