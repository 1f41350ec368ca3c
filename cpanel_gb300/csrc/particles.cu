// Vortex-particle operators on the GPU: direct sums and Barnes-Hut traversals.
//
// Pair kernels (FP64) restate CPanel/particle.cpp:
//   gauss_sym  particle::velInfl(particle*)   :42-58  (core sqrt((1.5 r_s)^2 + (1.5 r_t)^2)/sqrt 2)
//   gauss_poi  particle::velInfl(POI)         :60-77  (core 1.5 r_s; zero at distance 0)
//   alg        particle::velInflAlgSmooth     :31-38
//   stretch    particle::vortexStretching     :80-118 (`this` = first argument)
//   diffusion  particle::viscousDiffusion     :122-140 (`this` = first argument)
// The Barnes-Hut traversal is node::calcVel/calcStretch/calcDiff (octree/include/
// node.h:236-364) from the root's children (CPanel/particleFMM.cpp:65-116), made
// stackless: nodes are stored in pre-order with a skip index past each subtree, so
// "descend" is i+1 and "use the expansion" is skip[i], which visits nodes in the
// reference's recursion order.  One traversal serves velocity, stretching and
// diffusion together: all three take the same far-field decisions.
//
// Branch decisions (far field 2 half.x / |x_exp - x| < theta, stretching cut-off
// |x_s - x_t| > 5 r_s, zero distance) are computed with explicitly rounded
// intrinsics, so they match the host exactly although this file keeps FMA
// contraction for the pair arithmetic.
//
// The *_f32 traversals are the mixed-precision form: far nodes and leaf pairs in FP32
// (leaf pairs closer than a hundredth of their core width in FP64), the same decisions as
// the FP64 traversal.
#include <cuda_runtime.h>

#include <cmath>

#include "common.cuh"
#include "octree.h"
#include "particles.h"

namespace cpg {
namespace {

struct Tgt {
    dv3 x;
    double r;
    dv3 a;
    double idx;
};

__device__ __forceinline__ double exact_norm(double dx, double dy, double dz) {
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

__device__ __forceinline__ Tgt load_part(const BHPart& p) {
    return Tgt{mk3(p.x, p.y, p.z), p.r, mk3(p.ax, p.ay, p.az), p.idx};
}

// (erf(rho/sqrt2)/(4 pi rho) - exp(-rho^2/2)/(2 pi)^1.5) / rho^2
__device__ __forceinline__ double gauss_K(double rho, const VPConst& c) {
    return (1.0 / (c.four_pi * rho) * erf(rho / c.sqrt2) - c.c15 * exp(-0.5 * rho * rho)) / (rho * rho);
}

__device__ __forceinline__ double sym_sigma(double rs, double rt, const VPConst& c) {
    double a = 1.5 * rs, b = 1.5 * rt;
    return sqrt(a * a + b * b) / c.sqrt2;
}

// velocity at target t induced by source s, symmetrised Gaussian core
__device__ __forceinline__ dv3 vel_gauss_sym(const Tgt& s, const Tgt& t, const VPConst& c) {
    double sig = sym_sigma(s.r, t.r, c);
    dv3 d = t.x - s.x;
    double rho = norm3(d) / sig;
    double K = gauss_K(rho, c);
    return (-1.0 / (sig * sig * sig) * K) * cross3(d, s.a);
}

// velocity at a point, Gaussian core 1.5 r_s, zero when the point is on the particle
__device__ __forceinline__ dv3 vel_gauss_poi(const Tgt& s, dv3 poi, const VPConst& c) {
    double ddx = s.x.x - poi.x, ddy = s.x.y - poi.y, ddz = s.x.z - poi.z;
    if (exact_norm(ddx, ddy, ddz) == 0.0) return mk3(0, 0, 0);
    double sig = 1.5 * s.r;
    dv3 d = poi - s.x;
    double rho = norm3(d) / sig;
    double K = gauss_K(rho, c);
    return (-1.0 / (sig * sig * sig) * K) * cross3(d, s.a);
}

// high-order algebraic core
__device__ __forceinline__ dv3 vel_alg(const Tgt& s, dv3 poi, const VPConst& c) {
    double sig = 1.5 * s.r;
    dv3 d = poi - s.x;
    double r2 = dot3(d, d);
    double q = r2 + sig * sig;
    double f = -c.inv_four_pi * (r2 + 2.5 * sig * sig) / (q * q * sqrt(q));
    return f * cross3(d, s.a);
}

// particle::vortexStretching with this = P, part = Q
__device__ __forceinline__ dv3 stretch(const Tgt& P, const Tgt& Q, const VPConst& c) {
    double dx = P.x.x - Q.x.x, dy = P.x.y - Q.x.y, dz = P.x.z - Q.x.z;
    double dn = exact_norm(dx, dy, dz);
    if (dn > __dmul_rn(5.0, P.r)) return mk3(0, 0, 0);
    double sig = sym_sigma(P.r, Q.r, c);
    double rho = dn / sig;
    double xi = c.c15 * exp(-rho * rho / 2);
    double G = 1.0 / (c.four_pi * rho) * erf(rho / c.sqrt2);
    double K = (G - xi) / (rho * rho);
    double F = (3 * K - xi) / (rho * rho);
    dv3 d = mk3(dx, dy, dz);
    // M a_P = K a_P - F/sig^2 d (d . a_P);  result = (1/sig^3) a_Q x (M a_P)
    dv3 Ma = K * P.a - (F / (sig * sig) * dot3(d, P.a)) * d;
    return (1.0 / (sig * sig * sig)) * cross3(Q.a, Ma);
}

// particle::viscousDiffusion with this = P, part = Q
__device__ __forceinline__ dv3 diffusion(const Tgt& P, const Tgt& Q, const VPConst& c) {
    double sig = sym_sigma(P.r, Q.r, c);
    double rho = norm3(P.x - Q.x) / sig;
    double Vi = c.four_pi_3 * (P.r * P.r * P.r);
    double Vj = c.four_pi_3 * (Q.r * Q.r * Q.r);
    double xi = 1.0 / (c.two_pi_15 * (rho * rho * rho)) * exp(-rho * rho / 2);
    return (2 * c.nu / (sig * sig) * xi) * (Vi * Q.a - Vj * P.a);
}

__device__ __forceinline__ bool far_field(const BHNode& nd, dv3 x, double theta) {
    double d = exact_norm(nd.ex - x.x, nd.ey - x.y, nd.ez - x.z);
    return __ddiv_rn(nd.width, d) < theta;
}

__device__ __forceinline__ BHNode load_node(const BHNode* __restrict__ nodes, int i) {
    const double2* p = reinterpret_cast<const double2*>(nodes + i);
    double2 a0 = __ldg(p), a1 = __ldg(p + 1), b0 = __ldg(p + 2), b1 = __ldg(p + 3);
    const int4 q = __ldg(reinterpret_cast<const int4*>(nodes + i) + 4);
    BHNode nd;
    nd.ex = a0.x; nd.ey = a0.y; nd.ez = a1.x; nd.ax = a1.y;
    nd.ay = b0.x; nd.az = b0.y; nd.erad = b1.x; nd.width = b1.y;
    nd.first = q.x; nd.count = q.y; nd.skip = q.z; nd.leaf = q.w;
    return nd;
}

__device__ __forceinline__ Tgt load_part_g(const BHPart* __restrict__ parts, int64_t q) {
    const double2* p = reinterpret_cast<const double2*>(parts + q);
    double2 a0 = __ldg(p), a1 = __ldg(p + 1), b0 = __ldg(p + 2), b1 = __ldg(p + 3);
    return Tgt{mk3(a0.x, a0.y, a1.x), a1.y, mk3(b0.x, b0.y, b1.x), b1.y};
}

// ---- FP32 far field and leaves ----
// A far node's interaction is evaluated in FP32 from the node's float view (BHNodeF)
// and a target split into high and low floats; a leaf member's from the FP64 separation
// rounded once (leaf_pair_f below).  Far/near and stretching cut-off decisions compare
// float squared distances with a relative margin of 1e-5 (far beyond any float rounding
// of the distance) and take the exact FP64 test inside it, so the traversal visits the
// same nodes and pairs in the same order as the FP64 one.  Float contributions are
// summed with compensation (Kahan) and added to the FP64 accumulators once per target.

constexpr float kBandLo = 1.0f - 1e-5f, kBandHi = 1.0f + 1e-5f;

struct TgtF {
    float hx, hy, hz, lx, ly, lz;
    float r, ax, ay, az;
};

__device__ __forceinline__ TgtF split_tgt(const Tgt& t) {
    TgtF f;
    f.hx = __double2float_rn(t.x.x);
    f.hy = __double2float_rn(t.x.y);
    f.hz = __double2float_rn(t.x.z);
    f.lx = __double2float_rn(t.x.x - (double)f.hx);
    f.ly = __double2float_rn(t.x.y - (double)f.hy);
    f.lz = __double2float_rn(t.x.z - (double)f.hz);
    f.r = __double2float_rn(t.r);
    f.ax = __double2float_rn(t.a.x);
    f.ay = __double2float_rn(t.a.y);
    f.az = __double2float_rn(t.a.z);
    return f;
}

__device__ __forceinline__ BHNodeF load_fnode(const BHNodeF* __restrict__ f, int i) {
    const float4* p = reinterpret_cast<const float4*>(f + i);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    return BHNodeF{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
}

__device__ __forceinline__ int4 load_links(const BHNode* __restrict__ nodes, int i) {
    return __ldg(reinterpret_cast<const int4*>(nodes + i) + 4);  // first, count, skip, leaf
}

struct KSum {  // compensated float sum of a 3-vector
    float x = 0, y = 0, z = 0, cx = 0, cy = 0, cz = 0;
    __device__ __forceinline__ void add1(float& s, float& c, float v) {
        float y_ = v - c;
        float t = s + y_;
        c = (t - s) - y_;
        s = t;
    }
    __device__ __forceinline__ void add(float vx, float vy, float vz) {
        add1(x, cx, vx);
        add1(y, cy, vy);
        add1(z, cz, vz);
    }
    __device__ __forceinline__ dv3 value() const {
        return mk3((double)x - (double)cx, (double)y - (double)cy, (double)z - (double)cz);
    }
};

struct VPConstF {
    float inv_four_pi, inv_sqrt2, c15, four_pi_3, two_nu;
};

__device__ __forceinline__ VPConstF fconst(const VPConst& c) {
    return VPConstF{(float)c.inv_four_pi, (float)(1.0 / c.sqrt2), (float)c.c15, (float)c.four_pi_3, (float)(2 * c.nu)};
}

// far node f acting on target t; (dx, dy, dz) = target - expansion centre, d2 = |.|^2.
// V: symmetrised Gaussian velocity; S: stretching with `this` = the node (acts only when
// stretch_on); D: diffusion with `this` = the node.
template <bool V, bool S, bool D>
__device__ __forceinline__ void far_pair_f(const BHNodeF& f, const TgtF& t, float dx, float dy, float dz, float d2,
                                           bool stretch_on, const VPConstF& c, KSum& v, KSum& s, KSum& dd) {
    const float a = 1.5f * f.erad, b = 1.5f * t.r;
    const float sig = sqrtf(a * a + b * b) * c.inv_sqrt2;
    const float isig = 1.0f / sig;
    const float rho = sqrtf(d2) * isig;
    const float rho2 = rho * rho;
    const float ex = expf(-0.5f * rho2);
    const float xi = c.c15 * ex;
    const float isig3 = isig * isig * isig;
    float K = 0;
    if (V || S) {
        const float G = erff(rho * c.inv_sqrt2) * c.inv_four_pi / rho;
        K = (G - xi) / rho2;
    }
    if (V) {
        const float k = -K * isig3;  // -(K / sig^3) (d x a_node)
        v.add(k * (dy * f.az - dz * f.ay), k * (dz * f.ax - dx * f.az), k * (dx * f.ay - dy * f.ax));
    }
    if (S && stretch_on) {
        const float F = (3 * K - xi) / rho2;
        const float da = dx * f.ax + dy * f.ay + dz * f.az;
        const float g = F * isig * isig * da;
        const float mx = K * f.ax - g * dx, my = K * f.ay - g * dy, mz = K * f.az - g * dz;
        s.add(isig3 * (t.ay * mz - t.az * my), isig3 * (t.az * mx - t.ax * mz), isig3 * (t.ax * my - t.ay * mx));
    }
    if (D) {
        const float vi = c.four_pi_3 * (f.erad * f.erad * f.erad), vj = c.four_pi_3 * (t.r * t.r * t.r);
        const float k = c.two_nu * isig * isig * (xi / (rho2 * rho));
        dd.add(k * (vi * t.ax - vj * f.ax), k * (vi * t.ay - vj * f.ay), k * (vi * t.az - vj * f.az));
    }
}

// ---- FP32 leaf pairs ----
// K(rho) and F(rho) = (3 K - xi) / rho^2 of the Gaussian core as Taylor series in rho^2,
// from the series of erf and exp:
//   K / c15 = sum_j (-1)^j rho^2j / ((2j + 3) 2^j j!),  F / c15 = sum_j (-1)^j rho^2j / ((2j + 5) 2^j j!)
// (c15 = (2 pi)^-1.5).  Eleven terms hold both to 1e-8 relative for rho^2 < 2, where the
// closed forms lose digits to cancellation; beyond it the closed forms are used.
constexpr int kSeriesTerms = 11;
constexpr float kSeriesRho2 = 2.0f;
// pairs closer than rho^2 = kTinyRho2 (and coincident ones) stay in FP64
constexpr float kTinyRho2 = 1e-4f;

__host__ __device__ constexpr double series_coef(int j, int off) {
    double f = 1;
    for (int i = 1; i <= j; i++) f *= -2.0 * i;  // (-1)^j 2^j j!
    return 1.0 / ((2 * j + off) * f);
}

template <int OFF, int J = 0>
__device__ __forceinline__ float series_rho2(float r2) {
    constexpr float c = (float)series_coef(J, OFF);
    if constexpr (J == kSeriesTerms - 1)
        return c;
    else
        return fmaf(series_rho2<OFF, J + 1>(r2), r2, c);
}

// Leaf member mb acting on target t in FP32 (symmetrised Gaussian velocity, stretching and
// diffusion with `this` = the member, as the FP64 leaf sums).  The separation is taken in
// FP64 and rounded once; the stretching cut-off |x_m - x_t| > 5 r_m is decided on the float
// distance outside a 1e-5 relative margin and by the exact FP64 test inside it.  Returns
// false, adding nothing, for pairs closer than rho^2 = kTinyRho2: the caller takes those
// in FP64.
template <bool V, bool S, bool D>
__device__ __forceinline__ bool leaf_pair_f(const Tgt& mb, const Tgt& t, const TgtF& tf, const VPConstF& c,
                                            KSum& v, KSum& s, KSum& dd) {
    const float dx = __double2float_rn(t.x.x - mb.x.x), dy = __double2float_rn(t.x.y - mb.x.y),
                dz = __double2float_rn(t.x.z - mb.x.z);
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float rm = __double2float_rn(mb.r);
    const float a = 1.5f * rm, b = 1.5f * tf.r;
    const float sig2 = 0.5f * (a * a + b * b);
    const float rho2 = d2 / sig2;
    if (!(rho2 >= kTinyRho2)) return false;
    const float ax = __double2float_rn(mb.a.x), ay = __double2float_rn(mb.a.y), az = __double2float_rn(mb.a.z);
    const float isig = 1.0f / sqrtf(sig2);
    const float isig3 = isig * isig * isig;
    const float xi = c.c15 * expf(-0.5f * rho2);
    const bool series = rho2 < kSeriesRho2;
    const float rho = sqrtf(rho2);
    bool on = false;
    if (S) {
        const float cut = 5.0f * rm, cut2 = cut * cut;
        if (d2 < cut2 * kBandLo)
            on = true;
        else if (d2 > cut2 * kBandHi)
            on = false;
        else
            on = !(exact_norm(mb.x.x - t.x.x, mb.x.y - t.x.y, mb.x.z - t.x.z) > __dmul_rn(5.0, mb.r));
    }
    float K = 0;
    if (V || (S && on)) {
        K = series ? c.c15 * series_rho2<3>(rho2)
                   : (erff(rho * c.inv_sqrt2) * c.inv_four_pi / rho - xi) / rho2;
    }
    if (V) {
        const float k = -K * isig3;
        v.add(k * (dy * az - dz * ay), k * (dz * ax - dx * az), k * (dx * ay - dy * ax));
    }
    if (S && on) {
        const float F = series ? c.c15 * series_rho2<5>(rho2) : (3 * K - xi) / rho2;
        const float da = dx * ax + dy * ay + dz * az;
        const float g = F * isig * isig * da;
        const float mx = K * ax - g * dx, my = K * ay - g * dy, mz = K * az - g * dz;
        s.add(isig3 * (tf.ay * mz - tf.az * my), isig3 * (tf.az * mx - tf.ax * mz), isig3 * (tf.ax * my - tf.ay * mx));
    }
    if (D) {
        const float vi = c.four_pi_3 * (rm * rm * rm), vj = c.four_pi_3 * (tf.r * tf.r * tf.r);
        const float k = c.two_nu * isig * isig * (xi / (rho2 * rho));
        dd.add(k * (vi * tf.ax - vj * ax), k * (vi * tf.ay - vj * ay), k * (vi * tf.az - vj * az));
    }
    return true;
}

// leaf member mb at point x, algebraic core in FP32 (finite everywhere, zero at distance 0)
__device__ __forceinline__ void leaf_alg_f(const Tgt& mb, dv3 x, float i4p, KSum& v) {
    const float dx = __double2float_rn(x.x - mb.x.x), dy = __double2float_rn(x.y - mb.x.y),
                dz = __double2float_rn(x.z - mb.x.z);
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float sg = 1.5f * __double2float_rn(mb.r), sg2 = sg * sg;
    const float qq = d2 + sg2;
    const float k = -i4p * (d2 + 2.5f * sg2) / (qq * qq * sqrtf(qq));
    const float ax = __double2float_rn(mb.a.x), ay = __double2float_rn(mb.a.y), az = __double2float_rn(mb.a.z);
    v.add(k * (dy * az - dz * ay), k * (dz * ax - dx * az), k * (dx * ay - dy * ax));
}

// float difference target - node centre
__device__ __forceinline__ float3 diff_f(const TgtF& t, const BHNodeF& f) {
    return make_float3((t.hx - f.hx) + (t.lx - f.lx), (t.hy - f.hy) + (t.ly - f.ly), (t.hz - f.hz) + (t.lz - f.lz));
}

// exact FP64 tests of node i (used inside the margin only)
__device__ __forceinline__ bool far_exact(const BHNode* __restrict__ nodes, int i, dv3 x, double theta) {
    return far_field(load_node(nodes, i), x, theta);
}
// stretching of node i acts on x: not (|x_exp - x| > 5 erad), as in stretch()
__device__ __forceinline__ bool cut_exact(const BHNode* __restrict__ nodes, int i, dv3 x) {
    const BHNode nd = load_node(nodes, i);
    return !(exact_norm(nd.ex - x.x, nd.ey - x.y, nd.ez - x.z) > __dmul_rn(5.0, nd.erad));
}

// one traversal with FP32 far nodes for target t; `self` skips the member with the
// target's index.  Accumulates into v, s, d (FP64).
template <bool V, bool S, bool D>
__device__ __forceinline__ void traverse_f32(const BHNode* __restrict__ nodes, const BHNodeF* __restrict__ fn, int nn,
                                             const BHPart* __restrict__ parts, double theta, const Tgt& t,
                                             const VPConst& c, dv3& v, dv3& s, dv3& d) {
    const TgtF tf = split_tgt(t);
    const VPConstF cf = fconst(c);
    KSum fv, fs, fd;
    int i = 1;
    while (i < nn) {
        const int4 L = load_links(nodes, i);
        if (L.w) {
            for (int32_t k = L.x; k < L.x + L.y; k++) {
                const Tgt m = load_part_g(parts, k);
                if (m.idx == t.idx || leaf_pair_f<V, S, D>(m, t, tf, cf, fv, fs, fd)) continue;
                if (V) v = v + vel_gauss_sym(m, t, c);
                if (S) s = s + stretch(m, t, c);
                if (D) d = d + diffusion(m, t, c);
            }
            i++;
            continue;
        }
        const BHNodeF f = load_fnode(fn, i);
        const float3 dl = diff_f(tf, f);
        const float d2 = dl.x * dl.x + dl.y * dl.y + dl.z * dl.z;
        bool far;
        if (d2 > f.far2 * kBandHi)
            far = true;
        else if (d2 < f.far2 * kBandLo)
            far = false;
        else
            far = far_exact(nodes, i, t.x, theta);
        if (!far) {
            i++;
            continue;
        }
        bool on = false;
        if (S) {
            if (d2 < f.cut2 * kBandLo)
                on = true;
            else if (d2 > f.cut2 * kBandHi)
                on = false;
            else
                on = cut_exact(nodes, i, t.x);
        }
        far_pair_f<V, S, D>(f, tf, dl.x, dl.y, dl.z, d2, on, cf, fv, fs, fd);
        i = L.z;
    }
    if (V) v = v + fv.value();
    if (S) s = s + fs.value();
    if (D) d = d + fd.value();
}

// particleFMM::barnesHutVel(part) / barnesHutStretch / barnesHutDiff for every particle.
// Thread q handles the particle in slot q (leaf order: neighbouring threads traverse
// neighbouring paths).  Leaves: `this` = member (node.h:274-276, 307-309, 341-343).
template <bool V, bool S, bool D>
__global__ void __launch_bounds__(128) k_bh_particles(const BHNode* __restrict__ nodes, int nn,
                                                      const BHPart* __restrict__ parts, int64_t n, double theta,
                                                      VPConst c, double* __restrict__ vel, double* __restrict__ str,
                                                      double* __restrict__ dif) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const Tgt t = load_part_g(parts, q);
    dv3 v = mk3(0, 0, 0), s = mk3(0, 0, 0), d = mk3(0, 0, 0);
    int i = 1;
    while (i < nn) {
        const BHNode nd = load_node(nodes, i);
        if (nd.leaf) {
            for (int32_t k = nd.first; k < nd.first + nd.count; k++) {
                const Tgt m = load_part_g(parts, k);
                if (m.idx == t.idx) continue;
                if (V) v = v + vel_gauss_sym(m, t, c);
                if (S) s = s + stretch(m, t, c);
                if (D) d = d + diffusion(m, t, c);
            }
            i++;
        } else if (far_field(nd, t.x, theta)) {
            const Tgt e{mk3(nd.ex, nd.ey, nd.ez), nd.erad, mk3(nd.ax, nd.ay, nd.az), -1.0};
            if (V) v = v + vel_gauss_sym(e, t, c);
            if (S) s = s + stretch(e, t, c);
            if (D) d = d + diffusion(e, t, c);
            i = nd.skip;
        } else {
            i++;
        }
    }
    int64_t o = 3 * (int64_t)t.idx;
    if (V) { vel[o] = v.x; vel[o + 1] = v.y; vel[o + 2] = v.z; }
    if (S) { str[o] = s.x; str[o + 1] = s.y; str[o + 2] = s.z; }
    if (D) { dif[o] = d.x; dif[o + 1] = d.y; dif[o + 2] = d.z; }
}

// The same traversal for an explicit list of target particles (original order), which
// may include particles that are in no leaf (shed after the tree was built).
template <bool V, bool S, bool D>
__global__ void __launch_bounds__(128) k_bh_targets(const BHNode* __restrict__ nodes, int nn,
                                                    const BHPart* __restrict__ slots, double theta,
                                                    const BHPart* __restrict__ tgt, int64_t m, VPConst c,
                                                    double* __restrict__ vel, double* __restrict__ str,
                                                    double* __restrict__ dif) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= m) return;
    const Tgt t = load_part_g(tgt, q);
    dv3 v = mk3(0, 0, 0), s = mk3(0, 0, 0), d = mk3(0, 0, 0);
    int i = 1;
    while (i < nn) {
        const BHNode nd = load_node(nodes, i);
        if (nd.leaf) {
            for (int32_t k = nd.first; k < nd.first + nd.count; k++) {
                const Tgt mm = load_part_g(slots, k);
                if (mm.idx == t.idx) continue;
                if (V) v = v + vel_gauss_sym(mm, t, c);
                if (S) s = s + stretch(mm, t, c);
                if (D) d = d + diffusion(mm, t, c);
            }
            i++;
        } else if (far_field(nd, t.x, theta)) {
            const Tgt e{mk3(nd.ex, nd.ey, nd.ez), nd.erad, mk3(nd.ax, nd.ay, nd.az), -1.0};
            if (V) v = v + vel_gauss_sym(e, t, c);
            if (S) s = s + stretch(e, t, c);
            if (D) d = d + diffusion(e, t, c);
            i = nd.skip;
        } else {
            i++;
        }
    }
    if (V) { vel[3 * q] = v.x; vel[3 * q + 1] = v.y; vel[3 * q + 2] = v.z; }
    if (S) { str[3 * q] = s.x; str[3 * q + 1] = s.y; str[3 * q + 2] = s.z; }
    if (D) { dif[3 * q] = d.x; dif[3 * q + 1] = d.y; dif[3 * q + 2] = d.z; }
}

// k_bh_particles / k_bh_targets with far nodes and leaf pairs in FP32
template <bool V, bool S, bool D>
__global__ void __launch_bounds__(128) k_bh_particles_f32(const BHNode* __restrict__ nodes,
                                                          const BHNodeF* __restrict__ fn, int nn,
                                                          const BHPart* __restrict__ parts, int64_t n, double theta,
                                                          VPConst c, double* __restrict__ vel,
                                                          double* __restrict__ str, double* __restrict__ dif) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const Tgt t = load_part_g(parts, q);
    dv3 v = mk3(0, 0, 0), s = mk3(0, 0, 0), d = mk3(0, 0, 0);
    traverse_f32<V, S, D>(nodes, fn, nn, parts, theta, t, c, v, s, d);
    int64_t o = 3 * (int64_t)t.idx;
    if (V) { vel[o] = v.x; vel[o + 1] = v.y; vel[o + 2] = v.z; }
    if (S) { str[o] = s.x; str[o + 1] = s.y; str[o + 2] = s.z; }
    if (D) { dif[o] = d.x; dif[o + 1] = d.y; dif[o + 2] = d.z; }
}

template <bool V, bool S, bool D>
__global__ void __launch_bounds__(128) k_bh_targets_f32(const BHNode* __restrict__ nodes,
                                                        const BHNodeF* __restrict__ fn, int nn,
                                                        const BHPart* __restrict__ slots, double theta,
                                                        const BHPart* __restrict__ tgt, int64_t m, VPConst c,
                                                        double* __restrict__ vel, double* __restrict__ str,
                                                        double* __restrict__ dif) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= m) return;
    const Tgt t = load_part_g(tgt, q);
    dv3 v = mk3(0, 0, 0), s = mk3(0, 0, 0), d = mk3(0, 0, 0);
    traverse_f32<V, S, D>(nodes, fn, nn, slots, theta, t, c, v, s, d);
    if (V) { vel[3 * q] = v.x; vel[3 * q + 1] = v.y; vel[3 * q + 2] = v.z; }
    if (S) { str[3 * q] = s.x; str[3 * q + 1] = s.y; str[3 * q + 2] = s.z; }
    if (D) { dif[3 * q] = d.x; dif[3 * q + 1] = d.y; dif[3 * q + 2] = d.z; }
}

// ---- one warp per target (small target counts) ----
// With few targets, one thread per target leaves most SMs idle while each thread runs
// a long FP64 traversal.  Here the 32 lanes of a warp share one target: all lanes take
// the same far/near decisions, split each leaf's members between them and take the far
// nodes in turn; the lanes' sums are added by a fixed butterfly at the end.
__device__ __forceinline__ dv3 warp_sum3(dv3 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
    }
    return v;
}

// far decision of internal node i for target x (FP32 band test with the FP64 test inside
// the margin when fn is given, else the FP64 test); d: float target - centre, d2 = |d|^2
template <bool F32>
__device__ __forceinline__ bool far_decide(const BHNode* __restrict__ nodes, const BHNodeF* __restrict__ fn, int i,
                                           dv3 x, const TgtF& tf, double theta, BHNodeF& f, float3& dl, float& d2) {
    if (F32) {
        f = load_fnode(fn, i);
        dl = diff_f(tf, f);
        d2 = dl.x * dl.x + dl.y * dl.y + dl.z * dl.z;
        if (d2 > f.far2 * kBandHi) return true;
        if (d2 < f.far2 * kBandLo) return false;
        return far_exact(nodes, i, x, theta);
    }
    return far_exact(nodes, i, x, theta);
}

template <bool V, bool S, bool D, bool F32>
__global__ void __launch_bounds__(128) k_bh_targets_w(const BHNode* __restrict__ nodes,
                                                      const BHNodeF* __restrict__ fn, int nn,
                                                      const BHPart* __restrict__ slots, double theta,
                                                      const BHPart* __restrict__ tgt, int64_t m, VPConst c,
                                                      double* __restrict__ vel, double* __restrict__ str,
                                                      double* __restrict__ dif) {
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= m) return;  // uniform across the warp
    const Tgt t = load_part_g(tgt, q);
    TgtF tf{};
    if (F32) tf = split_tgt(t);
    const VPConstF cf = fconst(c);
    dv3 v = mk3(0, 0, 0), s = mk3(0, 0, 0), d = mk3(0, 0, 0);
    KSum fv, fs, fd;
    int i = 1, nfar = 0;
    while (i < nn) {
        const int4 L = load_links(nodes, i);
        if (L.w) {
            for (int32_t k = L.x + lane; k < L.x + L.y; k += 32) {
                const Tgt mb = load_part_g(slots, k);
                if (mb.idx == t.idx) continue;
                if (F32 && leaf_pair_f<V, S, D>(mb, t, tf, cf, fv, fs, fd)) continue;
                if (V) v = v + vel_gauss_sym(mb, t, c);
                if (S) s = s + stretch(mb, t, c);
                if (D) d = d + diffusion(mb, t, c);
            }
            i++;
            continue;
        }
        BHNodeF f{};
        float3 dl = make_float3(0.f, 0.f, 0.f);
        float d2 = 0.f;
        if (!far_decide<F32>(nodes, fn, i, t.x, tf, theta, f, dl, d2)) {
            i++;
            continue;
        }
        if ((nfar & 31) == lane) {
            if (F32) {
                bool on = false;
                if (S) {
                    if (d2 < f.cut2 * kBandLo)
                        on = true;
                    else if (d2 > f.cut2 * kBandHi)
                        on = false;
                    else
                        on = cut_exact(nodes, i, t.x);
                }
                far_pair_f<V, S, D>(f, tf, dl.x, dl.y, dl.z, d2, on, cf, fv, fs, fd);
            } else {
                const BHNode nd = load_node(nodes, i);
                const Tgt e{mk3(nd.ex, nd.ey, nd.ez), nd.erad, mk3(nd.ax, nd.ay, nd.az), -1.0};
                if (V) v = v + vel_gauss_sym(e, t, c);
                if (S) s = s + stretch(e, t, c);
                if (D) d = d + diffusion(e, t, c);
            }
        }
        nfar++;
        i = L.z;
    }
    if (F32) {
        if (V) v = v + fv.value();
        if (S) s = s + fs.value();
        if (D) d = d + fd.value();
    }
    if (V) v = warp_sum3(v);
    if (S) s = warp_sum3(s);
    if (D) d = warp_sum3(d);
    if (lane != 0) return;
    if (V) { vel[3 * q] = v.x; vel[3 * q + 1] = v.y; vel[3 * q + 2] = v.z; }
    if (S) { str[3 * q] = s.x; str[3 * q + 1] = s.y; str[3 * q + 2] = s.z; }
    if (D) { dif[3 * q] = d.x; dif[3 * q + 1] = d.y; dif[3 * q + 2] = d.z; }
}

// barnesHutVel(POI) with one warp per point (algebraic core)
template <bool F32>
__global__ void __launch_bounds__(128) k_bh_points_w(const BHNode* __restrict__ nodes, const BHNodeF* __restrict__ fn,
                                                     int nn, const BHPart* __restrict__ parts, double theta,
                                                     const double* __restrict__ pts, int64_t m, VPConst c,
                                                     double* __restrict__ vel) {
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= m) return;
    const dv3 x = ld3(pts + 3 * q);
    const Tgt t{x, 0.0, mk3(0, 0, 0), -1.0};
    TgtF tf{};
    if (F32) tf = split_tgt(t);
    const float i4p = (float)c.inv_four_pi;
    dv3 v = mk3(0, 0, 0);
    KSum fv;
    int i = 1, nfar = 0;
    while (i < nn) {
        const int4 L = load_links(nodes, i);
        if (L.w) {
            for (int32_t k = L.x + lane; k < L.x + L.y; k += 32) {
                if (F32)
                    leaf_alg_f(load_part_g(parts, k), x, i4p, fv);
                else
                    v = v + vel_alg(load_part_g(parts, k), x, c);
            }
            i++;
            continue;
        }
        BHNodeF f{};
        float3 dl = make_float3(0.f, 0.f, 0.f);
        float d2 = 0.f;
        if (!far_decide<F32>(nodes, fn, i, x, tf, theta, f, dl, d2)) {
            i++;
            continue;
        }
        if ((nfar & 31) == lane) {
            if (F32) {
                const float sg = 1.5f * f.erad, sg2 = sg * sg;
                const float qq = d2 + sg2;
                const float k = -i4p * (d2 + 2.5f * sg2) / (qq * qq * sqrtf(qq));
                fv.add(k * (dl.y * f.az - dl.z * f.ay), k * (dl.z * f.ax - dl.x * f.az), k * (dl.x * f.ay - dl.y * f.ax));
            } else {
                const BHNode nd = load_node(nodes, i);
                const Tgt e{mk3(nd.ex, nd.ey, nd.ez), nd.erad, mk3(nd.ax, nd.ay, nd.az), -1.0};
                v = v + vel_alg(e, x, c);
            }
        }
        nfar++;
        i = L.z;
    }
    if (F32) v = v + fv.value();
    v = warp_sum3(v);
    if (lane != 0) return;
    vel[3 * q] = v.x;
    vel[3 * q + 1] = v.y;
    vel[3 * q + 2] = v.z;
}

// slots[q] <- the current state of particle perm[q]
__global__ void k_refresh_slots(const int64_t* __restrict__ perm, int64_t ns, const double* __restrict__ pos,
                                const double* __restrict__ str, const double* __restrict__ rad,
                                BHPart* __restrict__ slots) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= ns) return;
    int64_t i = perm[q];
    slots[q] = BHPart{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], rad[i], str[3 * i], str[3 * i + 1], str[3 * i + 2],
                      (double)i};
}

// particleFMM::barnesHutVel(POI): algebraic kernel in leaves and far nodes (node.h:236-264)
__global__ void __launch_bounds__(128) k_bh_points(const BHNode* __restrict__ nodes, int nn,
                                                   const BHPart* __restrict__ parts, double theta,
                                                   const double* __restrict__ pts, int64_t m, VPConst c,
                                                   double* __restrict__ vel) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= m) return;
    const dv3 x = ld3(pts + 3 * q);
    dv3 v = mk3(0, 0, 0);
    int i = 1;
    while (i < nn) {
        const BHNode nd = load_node(nodes, i);
        if (nd.leaf) {
            for (int32_t k = nd.first; k < nd.first + nd.count; k++) v = v + vel_alg(load_part_g(parts, k), x, c);
            i++;
        } else if (far_field(nd, x, theta)) {
            const Tgt e{mk3(nd.ex, nd.ey, nd.ez), nd.erad, mk3(nd.ax, nd.ay, nd.az), -1.0};
            v = v + vel_alg(e, x, c);
            i = nd.skip;
        } else {
            i++;
        }
    }
    vel[3 * q] = v.x;
    vel[3 * q + 1] = v.y;
    vel[3 * q + 2] = v.z;
}

// k_bh_points with far nodes and leaf members in FP32 (algebraic core)
__global__ void __launch_bounds__(128) k_bh_points_f32(const BHNode* __restrict__ nodes,
                                                       const BHNodeF* __restrict__ fn, int nn,
                                                       const BHPart* __restrict__ parts, double theta,
                                                       const double* __restrict__ pts, int64_t m, VPConst c,
                                                       double* __restrict__ vel) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= m) return;
    const dv3 x = ld3(pts + 3 * q);
    const Tgt t{x, 0.0, mk3(0, 0, 0), -1.0};
    const TgtF tf = split_tgt(t);
    const float i4p = (float)c.inv_four_pi;
    dv3 v = mk3(0, 0, 0);
    KSum fv;
    int i = 1;
    while (i < nn) {
        const int4 L = load_links(nodes, i);
        if (L.w) {
            for (int32_t k = L.x; k < L.x + L.y; k++) leaf_alg_f(load_part_g(parts, k), x, i4p, fv);
            i++;
            continue;
        }
        const BHNodeF f = load_fnode(fn, i);
        const float3 dl = diff_f(tf, f);
        const float d2 = dl.x * dl.x + dl.y * dl.y + dl.z * dl.z;
        bool far;
        if (d2 > f.far2 * kBandHi)
            far = true;
        else if (d2 < f.far2 * kBandLo)
            far = false;
        else
            far = far_exact(nodes, i, x, theta);
        if (!far) {
            i++;
            continue;
        }
        const float sg = 1.5f * f.erad, sg2 = sg * sg;
        const float qq = d2 + sg2;
        const float k = -i4p * (d2 + 2.5f * sg2) / (qq * qq * sqrtf(qq));
        fv.add(k * (dl.y * f.az - dl.z * f.ay), k * (dl.z * f.ax - dl.x * f.az), k * (dl.x * f.ay - dl.y * f.ax));
        i = L.z;
    }
    v = v + fv.value();
    vel[3 * q] = v.x;
    vel[3 * q + 1] = v.y;
    vel[3 * q + 2] = v.z;
}

constexpr int kTile = 128;

// Direct sums, sources staged through shared memory in tiles of kTile particles.
// VK: 0 none, 1 gauss_sym (self skipped), 2 gauss_poi, 3 alg.  S/D: the direct
// stretching/diffusion of cpCaseVP::particleStrengthUpdate (`this` = target, j != i).
// Targets are particles (tgt != null) or points (pts).
// Block (x, y) sums the sources [y * chunk, min(n, (y + 1) * chunk)) and writes its part of
// each output at offset y * ystride: with one source range (chunk >= n) straight into the
// outputs, else into per-range slices that k_direct_reduce adds up in range order.
template <int VK, bool S, bool D>
__global__ void __launch_bounds__(kTile) k_direct(const BHPart* __restrict__ src, int64_t n,
                                                  const BHPart* __restrict__ tgt, const double* __restrict__ pts,
                                                  int64_t m, VPConst c, double* __restrict__ vel,
                                                  double* __restrict__ str, double* __restrict__ dif, int64_t chunk,
                                                  int64_t ystride) {
    __shared__ BHPart tile[kTile];
    const int64_t b0 = blockIdx.y * chunk;
    const int64_t b1 = b0 + chunk < n ? b0 + chunk : n;
    vel += blockIdx.y * ystride;
    str += blockIdx.y * ystride;
    dif += blockIdx.y * ystride;
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool live = q < m;
    Tgt t{mk3(0, 0, 0), 0, mk3(0, 0, 0), -1.0};
    if (live) {
        if (tgt)
            t = load_part_g(tgt, q);
        else
            t.x = ld3(pts + 3 * q);
    }
    dv3 v = mk3(0, 0, 0), s = mk3(0, 0, 0), d = mk3(0, 0, 0);
    for (int64_t b = b0; b < b1; b += kTile) {
        __syncthreads();
        if (b + threadIdx.x < b1) tile[threadIdx.x] = src[b + threadIdx.x];
        __syncthreads();
        int lim = (int)((b1 - b) < kTile ? (b1 - b) : kTile);
        if (!live) continue;
        for (int k = 0; k < lim; k++) {
            const Tgt p = load_part(tile[k]);
            bool self = p.idx == t.idx;
            if (VK == 1 && !self) v = v + vel_gauss_sym(p, t, c);
            if (VK == 2) v = v + vel_gauss_poi(p, t.x, c);
            if (VK == 3) v = v + vel_alg(p, t.x, c);
            if (S && !self) s = s + stretch(t, p, c);
            if (D && !self) d = d + diffusion(t, p, c);
        }
    }
    if (!live) return;
    if (VK) { vel[3 * q] = v.x; vel[3 * q + 1] = v.y; vel[3 * q + 2] = v.z; }
    if (S) { str[3 * q] = s.x; str[3 * q + 1] = s.y; str[3 * q + 2] = s.z; }
    if (D) { dif[3 * q] = d.x; dif[3 * q + 1] = d.y; dif[3 * q + 2] = d.z; }
}

// out_o[i] = sum over ranges y of part[o * ns * len + y * len + i], ranges in order
__global__ void k_direct_reduce(const double* __restrict__ part, int ns, int64_t len, double* __restrict__ o0,
                                double* __restrict__ o1, double* __restrict__ o2) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= len) return;
    double* outs[3] = {o0, o1, o2};
    for (int o = 0; o < 3; o++) {
        if (!outs[o]) continue;
        const double* p = part + (int64_t)o * ns * len + i;
        double a = 0;
        for (int y = 0; y < ns; y++) a += p[(int64_t)y * len];
        outs[o][i] = a;
    }
}

__global__ void k_pack_parts(const double* __restrict__ pos, const double* __restrict__ str,
                             const double* __restrict__ rad, int64_t n, BHPart* __restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = BHPart{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], rad[i], str[3 * i], str[3 * i + 1], str[3 * i + 2],
                    (double)i};
}

unsigned blocks(int64_t m, int t) { return (unsigned)((m + t - 1) / t); }

// up to this many targets a traversal runs one warp per target (k_bh_targets_w,
// k_bh_points_w); above, one thread per target fills the GPU on its own
constexpr int64_t kWarpPerTargetMax = 16384;

}  // namespace

cudaError_t launch_bh_particles(const BHNode* nodes, const BHNodeF* fnodes, int nn, const BHPart* parts, int64_t n,
                                double theta, const VPConst& c, double* vel, double* str, double* dif,
                                cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int mask = (vel ? 1 : 0) | (str ? 2 : 0) | (dif ? 4 : 0);
    dim3 g(blocks(n, 128)), b(128);
    if (fnodes) {
#define CPG_BHF(V_, S_, D_) \
    k_bh_particles_f32<V_, S_, D_><<<g, b, 0, s>>>(nodes, fnodes, nn, parts, n, theta, c, vel, str, dif)
        switch (mask) {
            case 1: CPG_BHF(true, false, false); break;
            case 2: CPG_BHF(false, true, false); break;
            case 3: CPG_BHF(true, true, false); break;
            case 4: CPG_BHF(false, false, true); break;
            case 5: CPG_BHF(true, false, true); break;
            case 6: CPG_BHF(false, true, true); break;
            case 7: CPG_BHF(true, true, true); break;
            default: return cudaSuccess;
        }
#undef CPG_BHF
        return cudaGetLastError();
    }
    switch (mask) {
        case 1: k_bh_particles<true, false, false><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        case 2: k_bh_particles<false, true, false><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        case 3: k_bh_particles<true, true, false><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        case 4: k_bh_particles<false, false, true><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        case 5: k_bh_particles<true, false, true><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        case 6: k_bh_particles<false, true, true><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        case 7: k_bh_particles<true, true, true><<<g, b, 0, s>>>(nodes, nn, parts, n, theta, c, vel, str, dif); break;
        default: return cudaSuccess;
    }
    return cudaGetLastError();
}

cudaError_t launch_bh_targets(const BHNode* nodes, const BHNodeF* fnodes, int nn, const BHPart* slots, double theta,
                              const BHPart* tgt, int64_t m, const VPConst& c, double* vel, double* str, double* dif,
                              cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    int mask = (vel ? 1 : 0) | (str ? 2 : 0) | (dif ? 4 : 0);
    if (m <= kWarpPerTargetMax) {
        dim3 gw(blocks(32 * m, 128)), bw(128);
#define CPG_BHW(V_, S_, D_, F_) \
    k_bh_targets_w<V_, S_, D_, F_><<<gw, bw, 0, s>>>(nodes, fnodes, nn, slots, theta, tgt, m, c, vel, str, dif)
        if (fnodes) {
            switch (mask) {
                case 1: CPG_BHW(true, false, false, true); break;
                case 6: CPG_BHW(false, true, true, true); break;
                case 7: CPG_BHW(true, true, true, true); break;
                default: return cudaErrorInvalidValue;
            }
        } else {
            switch (mask) {
                case 1: CPG_BHW(true, false, false, false); break;
                case 6: CPG_BHW(false, true, true, false); break;
                case 7: CPG_BHW(true, true, true, false); break;
                default: return cudaErrorInvalidValue;
            }
        }
#undef CPG_BHW
        return cudaGetLastError();
    }
    dim3 g(blocks(m, 128)), b(128);
    if (fnodes) {
        switch (mask) {
            case 1: k_bh_targets_f32<true, false, false><<<g, b, 0, s>>>(nodes, fnodes, nn, slots, theta, tgt, m, c, vel, str, dif); break;
            case 6: k_bh_targets_f32<false, true, true><<<g, b, 0, s>>>(nodes, fnodes, nn, slots, theta, tgt, m, c, vel, str, dif); break;
            case 7: k_bh_targets_f32<true, true, true><<<g, b, 0, s>>>(nodes, fnodes, nn, slots, theta, tgt, m, c, vel, str, dif); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    switch (mask) {
        case 1: k_bh_targets<true, false, false><<<g, b, 0, s>>>(nodes, nn, slots, theta, tgt, m, c, vel, str, dif); break;
        case 6: k_bh_targets<false, true, true><<<g, b, 0, s>>>(nodes, nn, slots, theta, tgt, m, c, vel, str, dif); break;
        case 7: k_bh_targets<true, true, true><<<g, b, 0, s>>>(nodes, nn, slots, theta, tgt, m, c, vel, str, dif); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_refresh_slots(const int64_t* perm, int64_t ns, const double* pos, const double* str,
                                 const double* rad, BHPart* slots, cudaStream_t s) {
    if (ns <= 0) return cudaSuccess;
    k_refresh_slots<<<blocks(ns, 256), 256, 0, s>>>(perm, ns, pos, str, rad, slots);
    return cudaGetLastError();
}

cudaError_t launch_bh_points(const BHNode* nodes, const BHNodeF* fnodes, int nn, const BHPart* parts, double theta,
                             const double* pts, int64_t m, const VPConst& c, double* vel, cudaStream_t s) {
    if (m <= 0) return cudaSuccess;
    if (m <= kWarpPerTargetMax) {
        if (fnodes)
            k_bh_points_w<true><<<blocks(32 * m, 128), 128, 0, s>>>(nodes, fnodes, nn, parts, theta, pts, m, c, vel);
        else
            k_bh_points_w<false><<<blocks(32 * m, 128), 128, 0, s>>>(nodes, fnodes, nn, parts, theta, pts, m, c, vel);
        return cudaGetLastError();
    }
    if (fnodes)
        k_bh_points_f32<<<blocks(m, 128), 128, 0, s>>>(nodes, fnodes, nn, parts, theta, pts, m, c, vel);
    else
        k_bh_points<<<blocks(m, 128), 128, 0, s>>>(nodes, nn, parts, theta, pts, m, c, vel);
    return cudaGetLastError();
}

cudaError_t launch_pack_parts(const double* pos, const double* str, const double* rad, int64_t n, BHPart* out,
                              cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_pack_parts<<<blocks(n, 256), 256, 0, s>>>(pos, str, rad, n, out);
    return cudaGetLastError();
}

namespace {
int device_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        n = v > 0 ? v : 1;
    }
    return n;
}

// source ranges for m targets over n sources: enough blocks for about eight per SM,
// ranges of whole tiles
int64_t direct_ranges(int64_t n, int64_t m) {
    const int64_t tb = blocks(m, kTile), tiles = blocks(n, kTile);
    const int64_t want = (8 * (int64_t)device_sms() + tb - 1) / tb;
    int64_t r = want < tiles ? want : tiles;
    return r > 1 ? r : 1;
}
}  // namespace

int64_t direct_scratch_doubles(int64_t n, int64_t m) {
    const int64_t r = direct_ranges(n, m);
    return r > 1 ? 9 * m * r : 0;
}

cudaError_t launch_direct(int vk, bool S, bool D, const BHPart* src, int64_t n, const BHPart* tgt, const double* pts,
                          int64_t m, const VPConst& c, double* vel, double* str, double* dif, cudaStream_t s,
                          double* scratch, int64_t scratch_doubles) {
    if (m <= 0) return cudaSuccess;
    int64_t ranges = direct_ranges(n, m);
    if (!scratch || scratch_doubles < 9 * m * ranges) ranges = 1;
    const int64_t chunk = ranges > 1 ? kTile * ((blocks(n, kTile) + ranges - 1) / ranges) : (n > 0 ? n : 1);
    if (ranges > 1) ranges = (n + chunk - 1) / chunk;
    dim3 g(blocks(m, kTile), (unsigned)ranges), b(kTile);
    const int64_t len = 3 * m;
    double* kv = ranges > 1 ? scratch : vel;
    double* ks = ranges > 1 ? scratch + ranges * len : str;
    double* kd = ranges > 1 ? scratch + 2 * ranges * len : dif;
    const int64_t ystride = ranges > 1 ? len : 0;
#define CPG_DIRECT(VK_, S_, D_) \
    k_direct<VK_, S_, D_><<<g, b, 0, s>>>(src, n, tgt, pts, m, c, kv, ks, kd, chunk, ystride)
    int key = vk * 4 + (S ? 2 : 0) + (D ? 1 : 0);
    switch (key) {
        case 4: CPG_DIRECT(1, false, false); break;
        case 8: CPG_DIRECT(2, false, false); break;
        case 11: CPG_DIRECT(2, true, true); break;
        case 10: CPG_DIRECT(2, true, false); break;
        case 9: CPG_DIRECT(2, false, true); break;
        case 12: CPG_DIRECT(3, false, false); break;
        case 3: CPG_DIRECT(0, true, true); break;
        case 2: CPG_DIRECT(0, true, false); break;
        case 1: CPG_DIRECT(0, false, true); break;
        default: return cudaErrorInvalidValue;
    }
#undef CPG_DIRECT
    if (ranges > 1)
        k_direct_reduce<<<blocks(len, 256), 256, 0, s>>>(scratch, (int)ranges, len, vk ? vel : nullptr,
                                                          S ? str : nullptr, D ? dif : nullptr);
    return cudaGetLastError();
}

VPConst vp_constants() {
    VPConst c;
    const double pi = 3.14159265358979323846;
    c.four_pi = 4 * pi;
    c.inv_four_pi = 1 / (4 * pi);
    c.sqrt2 = std::pow(2.0, 0.5);
    c.two_pi_15 = std::pow(2 * pi, 1.5);
    c.c15 = 1 / c.two_pi_15;
    c.four_pi_3 = 4 * pi / 3;
    c.nu = 1.983e-5;  // CPanel/particle.cpp:126
    return c;
}

}  // namespace cpg
