"""ctypes front end of the CPU oracle (test infrastructure only)."""
import ctypes as C
import math
import os

import numpy as np

from . import build as _build

_lib = None

D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)
I64 = C.POINTER(C.c_int64)


class CaseParams(C.Structure):
    _fields_ = [("V", C.c_double), ("alpha", C.c_double), ("beta", C.c_double), ("mach", C.c_double),
                ("Sref", C.c_double), ("bref", C.c_double), ("cref", C.c_double), ("cg", C.c_double * 3)]


class CaseResult(C.Structure):
    _fields_ = [("CL", C.c_double), ("CDi", C.c_double), ("Fbody", C.c_double * 3), ("Fwind", C.c_double * 3),
                ("CM", C.c_double * 3), ("iters", C.c_int64), ("error", C.c_double), ("converged", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.cpo_mesh_new.restype = C.c_void_p
        L.cpo_mesh_new.argtypes = [D, C.c_int64, I64, I32, C.c_int64]
        L.cpo_mesh_free.argtypes = [C.c_void_p]
        for f in ("cpo_n_body", "cpo_n_wake", "cpo_n_wakes"):
            getattr(L, f).restype = C.c_int64
            getattr(L, f).argtypes = [C.c_void_p]
        L.cpo_n_wakelines.restype = C.c_int64
        L.cpo_n_wakelines.argtypes = [C.c_void_p, C.c_int64]
        L.cpo_body_table.argtypes = [C.c_void_p, D]
        L.cpo_wake_table.argtypes = [C.c_void_p, D, I32, D]
        L.cpo_clusters.argtypes = [C.c_void_p, I32]
        L.cpo_body_verts.argtypes = [C.c_void_p, D]
        L.cpo_wake_verts.argtypes = [C.c_void_p, D]
        L.cpo_tri_phi_inf.argtypes = [D, D, D, D]
        L.cpo_tri_dub_phi_inf.restype = C.c_double
        L.cpo_tri_dub_phi_inf.argtypes = [D, D]
        L.cpo_tri_v_inf.argtypes = [D, D, D, D]
        L.cpo_set_inf_coeff.argtypes = [C.c_void_p, D, D, C.c_int64, C.c_int64, C.c_int]
        L.cpo_case_run.restype = C.c_int
        L.cpo_case_run.argtypes = [C.c_void_p, D, D, C.POINTER(CaseParams), D, D, D, D, D, D,
                                   C.POINTER(CaseResult), C.c_int]
        L.cpo_case_post.restype = C.c_int
        L.cpo_case_post.argtypes = [C.c_void_p, C.POINTER(CaseParams), D, D, D, D, C.POINTER(CaseResult)]
        L.cpo_spanwise.restype = C.c_int
        L.cpo_spanwise.argtypes = [C.c_void_p, C.c_int, D, D, D]
        L.cpo_bicgstab.restype = C.c_int
        L.cpo_bicgstab.argtypes = [D, C.c_int64, D, D, C.c_double, C.c_int64, I64, D, C.c_int]
        L.cpo_tri_dub_v_inf.argtypes = [D, D, D]
        L.cpo_panels_velocity.argtypes = [D, D, D, C.c_int64, D, D, C.c_int64, D, C.c_int64, D, C.c_int]
        L.cpo_vpcase_new.restype = C.c_void_p
        L.cpo_vpcase_new.argtypes = [D, C.c_int64, I64, I32, C.c_int64, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_int, C.c_int]
        L.cpo_vpcase_free.argtypes = [C.c_void_p]
        L.cpo_vpcase_info.argtypes = [C.c_void_p, I64]
        L.cpo_vpcase_dt.restype = C.c_double
        L.cpo_vpcase_dt.argtypes = [C.c_void_p]
        L.cpo_vpcase_wake.argtypes = [C.c_void_p, D, D, I32, D]
        L.cpo_vpcase_matrices.argtypes = [C.c_void_p, D, D, D]
        L.cpo_vpcase_set_refs.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.cpo_vpcase_trefftz.argtypes = [C.c_void_p, D]
        L.cpo_vpcase_trefftz_row.argtypes = [C.c_void_p, C.c_int, D]
        L.cpo_vpcase_step.restype = C.c_int
        L.cpo_vpcase_step.argtypes = [C.c_void_p]
        L.cpo_vpcase_particles.argtypes = [C.c_void_p, D, D, D, I32, I32]
        L.cpo_vpcase_strengths.argtypes = [C.c_void_p, D, D, D, D]
        L.cpo_vpcase_surface.argtypes = [C.c_void_p, D, C.c_double, C.c_double, D, D, D, D]
        L.cpo_panels_stretching.argtypes = [D, D, D, C.c_int64, D, D, C.c_int64, D, D, C.c_int64, D]
        L.cpo_vp_direct_velocity.argtypes = [D, D, D, C.c_int64, D, C.c_int64, C.c_int, D]
        L.cpo_vp_direct_stretch.argtypes = [D, D, D, C.c_int64, D]
        L.cpo_vp_direct_diffusion.argtypes = [D, D, D, C.c_int64, D]
        L.cpo_bh_build.restype = C.c_void_p
        L.cpo_bh_build.argtypes = [D, D, D, C.c_int64, C.c_int64, C.c_double]
        L.cpo_bh_free.argtypes = [C.c_void_p]
        for f in ("cpo_bh_num_nodes", "cpo_bh_num_levels"):
            getattr(L, f).restype = C.c_int64
            getattr(L, f).argtypes = [C.c_void_p]
        L.cpo_bh_nodes.argtypes = [C.c_void_p, D]
        L.cpo_bh_leaf_members.argtypes = [C.c_void_p, I64]
        L.cpo_bh_velocity.argtypes = [C.c_void_p, D, C.c_int64, C.c_int, D]
        L.cpo_bh_stretch.argtypes = [C.c_void_p, D]
        L.cpo_bh_diffusion.argtypes = [C.c_void_p, D]
        _lib = L
    return _lib


def _p(a, t=D):
    return a.ctypes.data_as(t) if a is not None else None


def nthreads_default():
    return max(1, os.cpu_count() or 1)


class Mesh:
    """Oracle mesh: geometry::readTri topology on a .tri-style array triple."""

    def __init__(self, nodes, tris, ids):
        self.L = lib()
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.tris = np.ascontiguousarray(tris, dtype=np.int64)
        self.ids = np.ascontiguousarray(ids, dtype=np.int32)
        self.h = self.L.cpo_mesh_new(_p(self.nodes), len(self.nodes), _p(self.tris, I64), _p(self.ids, I32),
                                     len(self.ids))
        self.n = self.L.cpo_n_body(self.h)
        self.nw = self.L.cpo_n_wake(self.h)

    def __del__(self):
        try:
            self.L.cpo_mesh_free(self.h)
        except Exception:
            pass

    def body_table(self):
        out = np.zeros((self.n, 18))
        self.L.cpo_body_table(self.h, _p(out))
        return out

    def wake_table(self):
        out = np.zeros((self.nw, 8))
        idx = np.zeros((self.nw, 4), dtype=np.int32)
        coef = np.zeros(self.nw)
        self.L.cpo_wake_table(self.h, _p(out), _p(idx, I32), _p(coef))
        return out, idx, coef

    def clusters(self):
        out = np.zeros((self.n, 32), dtype=np.int32)
        self.L.cpo_clusters(self.h, _p(out, I32))
        return out

    def body_verts(self):
        out = np.zeros((self.n, 9))
        self.L.cpo_body_verts(self.h, _p(out))
        return out

    def wake_verts(self):
        out = np.zeros((self.nw, 9))
        self.L.cpo_wake_verts(self.h, _p(out))
        return out

    def set_inf_coeff(self, rows=None, nthreads=None):
        """Dense A, B as Fortran-ordered arrays (column-major like Eigen): all rows
        (n x n) or the row block rows=(r0, r1) ((r1-r0) x n)."""
        n = self.n
        r0, r1 = (0, n) if rows is None else rows
        A = np.empty((r1 - r0, n), order="F")
        B = np.empty((r1 - r0, n), order="F")
        self.L.cpo_set_inf_coeff(self.h, _p(A), _p(B), r0, r1, nthreads or nthreads_default())
        return A, B

    def case(self, A, B, V=1.0, alpha=5.0, beta=0.0, mach=0.1, Sref=1.0, bref=1.0, cref=1.0, cg=(0, 0, 0),
             nthreads=None):
        n = self.n
        p = CaseParams(V, alpha, beta, mach, Sref, bref, cref, (C.c_double * 3)(*cg))
        r = CaseResult()
        out = {k: np.zeros(n) for k in ("sigma", "mu", "phi", "cp")}
        out["vel"] = np.zeros((n, 3))
        out["wake_mu"] = np.zeros(self.nw)
        A = np.asfortranarray(A)
        B = np.asfortranarray(B)
        self.L.cpo_case_run(self.h, _p(A), _p(B), C.byref(p), _p(out["sigma"]), _p(out["mu"]), _p(out["phi"]),
                            _p(out["vel"]), _p(out["cp"]), _p(out["wake_mu"]), C.byref(r),
                            nthreads or nthreads_default())
        out.update(CL=r.CL, CDi=r.CDi, Fbody=np.array(r.Fbody[:]), Fwind=np.array(r.Fwind[:]),
                   CM=np.array(r.CM[:]), iters=r.iters, error=r.error, converged=bool(r.converged))
        return out

    def post(self, mu, V=1.0, alpha=5.0, beta=0.0, mach=0.1, Sref=1.0, bref=1.0, cref=1.0, cg=(0, 0, 0)):
        n = self.n
        p = CaseParams(V, alpha, beta, mach, Sref, bref, cref, (C.c_double * 3)(*cg))
        r = CaseResult()
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        phi, cp, vel = np.zeros(n), np.zeros(n), np.zeros((n, 3))
        self.L.cpo_case_post(self.h, C.byref(p), _p(mu), _p(phi), _p(vel), _p(cp), C.byref(r))
        return dict(phi=phi, cp=cp, vel=vel, CL=r.CL, CDi=r.CDi, Fbody=np.array(r.Fbody[:]),
                    Fwind=np.array(r.Fwind[:]), CM=np.array(r.CM[:]))

    def spanwise(self, wake=0):
        """The last case's spanwise Trefftz loads of one wake (cpCase::writeSpanwiseData,
        CPanel/cpCase.cpp:910-935): dict of y2b, cl, cdi at the 165 stations."""
        out = {k: np.zeros(512) for k in ("y2b", "cl", "cdi")}
        m = self.L.cpo_spanwise(self.h, wake, _p(out["y2b"]), _p(out["cl"]), _p(out["cdi"]))
        if m < 0:
            raise ValueError("no spanwise loads for wake %d" % wake)
        return {k: v[:m].copy() for k, v in out.items()}


def tri_phi_inf(verts9, poi):
    L = lib()
    v = np.ascontiguousarray(verts9, dtype=np.float64)
    p = np.ascontiguousarray(poi, dtype=np.float64)
    s, d = C.c_double(0), C.c_double(0)
    L.cpo_tri_phi_inf(_p(v), _p(p), C.byref(s), C.byref(d))
    return s.value, d.value


def tri_dub_phi_inf(verts9, poi):
    L = lib()
    v = np.ascontiguousarray(verts9, dtype=np.float64)
    p = np.ascontiguousarray(poi, dtype=np.float64)
    return L.cpo_tri_dub_phi_inf(_p(v), _p(p))


def tri_v_inf(verts9, poi):
    L = lib()
    v = np.ascontiguousarray(verts9, dtype=np.float64)
    p = np.ascontiguousarray(poi, dtype=np.float64)
    vs, vd = np.zeros(3), np.zeros(3)
    L.cpo_tri_v_inf(_p(v), _p(p), _p(vs), _p(vd))
    return vs, vd


def bicgstab(A, b, nthreads=None):
    L = lib()
    A = np.asfortranarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = len(b)
    x = np.zeros(n)
    it, err = C.c_int64(0), C.c_double(0)
    L.cpo_bicgstab(_p(A), n, _p(b), _p(x), np.finfo(float).eps, 2 * n, C.byref(it), C.byref(err),
                   nthreads or nthreads_default())
    return x, it.value, err.value


def tri_dub_v_inf(verts9, poi):
    L = lib()
    v = np.ascontiguousarray(verts9, dtype=np.float64)
    p = np.ascontiguousarray(poi, dtype=np.float64)
    vd = np.zeros(3)
    L.cpo_tri_dub_v_inf(_p(v), _p(p), _p(vd))
    return vd


def panels_velocity(bverts, sigma, mu, wverts, wmu, pts, nthreads=None):
    """Sum of bodyPanel::panelV over body triangles and wakePanel::panelV over wake triangles."""
    L = lib()
    bv = np.ascontiguousarray(bverts, dtype=np.float64).reshape(-1, 9)
    wv = np.ascontiguousarray(wverts, dtype=np.float64).reshape(-1, 9)
    sg = np.ascontiguousarray(sigma, dtype=np.float64)
    m_ = np.ascontiguousarray(mu, dtype=np.float64)
    wm = np.ascontiguousarray(wmu, dtype=np.float64)
    p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(p), 3))
    L.cpo_panels_velocity(_p(bv), _p(sg), _p(m_), len(bv), _p(wv), _p(wm), len(wv), _p(p), len(p), _p(out),
                          nthreads or nthreads_default())
    return out


def point_velocity(bverts, sigma, mu, wverts, wmu, vinf, mach):
    """geometry::pntVelocity (CPanel/geometry.cpp:1239-1253) as a function of one point: the panels'
    velocity plus V_inf, the x component divided by the Prandtl-Glauert factor sqrt(1 - M^2)."""
    pg = math.sqrt(1 - mach ** 2)
    vinf = np.asarray(vinf, dtype=np.float64)

    def f(p):
        v = panels_velocity(bverts, sigma, mu, wverts, wmu, np.asarray(p, dtype=np.float64).reshape(1, 3))[0] + vinf
        v[0] /= pg
        return v
    return f


def streamline(vel, start, speed, x_max, tol, max_points=100000):
    """One off-body streamline as streamline::streamline and streamline::rkf integrate it
    (CPanel/streamline.cpp:20-78): Runge-Kutta-Fehlberg 4(5) from start with a first step of
    0.1 / speed; after each step with a positive error estimate err = |step5 - step4|,
    dt <- dt (tol dt / (2 err))^(1/4); stop once a step ends at x >= x_max.  vel(point) -> velocity.
    Every step start is kept with its velocity.  Returns (points, velocities, ended), ended False
    where max_points stopped the line first."""
    c5 = [16.0 / 135, 0, 6656.0 / 12825, 28561.0 / 56430, -9.0 / 50, 2.0 / 55]
    c4 = [25.0 / 216, 0, 1408.0 / 2565, 2197.0 / 4104, -0.2, 0]
    pts, vels = [], []

    def rkf(x0, dt):
        x = [float(v) for v in x0]
        k = []
        for s in range(6):
            if s == 0:
                y = list(x)
            else:
                k0 = k[0]
                k1 = k[1] if s > 1 else None
                k2 = k[2] if s > 2 else None
                k3 = k[3] if s > 3 else None
                k4 = k[4] if s > 4 else None
                y = []
                for c in range(3):
                    if s == 1:
                        y.append(x[c] + 1.0 / 4 * k0[c])
                    elif s == 2:
                        y.append(x[c] + 1.0 / 32 * (3 * k0[c] + 9.0 * k1[c]))
                    elif s == 3:
                        y.append(x[c] + 1.0 / 2197 * (1932 * k0[c] - 7200 * k1[c] + 7296 * k2[c]))
                    elif s == 4:
                        y.append(x[c] + 439.0 / 216 * k0[c] - 8 * k1[c] + 3680.0 / 513 * k2[c] - 845.0 / 4104 * k3[c])
                    else:
                        y.append(x[c] - 8.0 / 27 * k0[c] + 2 * k1[c] - 3544.0 / 2565 * k2[c] + 1859.0 / 4104 * k3[c]
                                 - 11.0 / 40 * k4[c])
            v = [float(q) for q in vel(np.array(y))]
            if s == 0:
                pts.append(list(x))
                vels.append(v)
            k.append([dt * v[c] for c in range(3)])
        s5, s4 = [], []
        for c in range(3):
            a5 = a4 = 0.0
            for j in range(6):
                a5 += c5[j] * k[j][c]
                a4 += c4[j] * k[j][c]
            s5.append(a5)
            s4.append(a4)
        err = math.sqrt(sum((s5[c] - s4[c]) * (s5[c] - s4[c]) for c in range(3)))
        return [x[c] + s5[c] for c in range(3)], err

    dt = 0.1 / speed
    if max_points < 1:
        return np.zeros((0, 3)), np.zeros((0, 3)), False
    nxt, err = rkf(start, dt)
    ended = True
    while nxt[0] < x_max:
        if len(pts) >= max_points:
            ended = False
            break
        if err > 0:
            dt = dt * math.pow(tol * dt / (2 * err), 0.25)
        nxt, err = rkf(nxt, dt)
    return np.array(pts).reshape(-1, 3), np.array(vels).reshape(-1, 3), ended


def _parts(pos, strength, radius):
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    strength = np.ascontiguousarray(strength, dtype=np.float64).reshape(-1, 3)
    radius = np.ascontiguousarray(radius, dtype=np.float64).reshape(-1)
    return pos, strength, radius


def particles_velocity(pos, strength, radius, pts=None, kernel="gauss"):
    """Direct sums of particle::velInfl.  pts None: on every particle (symmetrised core,
    self skipped); else at the points with the Gaussian or the algebraic kernel."""
    L = lib()
    pos, st, rad = _parts(pos, strength, radius)
    if pts is None:
        out = np.zeros((len(pos), 3))
        L.cpo_vp_direct_velocity(_p(pos), _p(st), _p(rad), len(pos), None, 0, 0, _p(out))
        return out
    p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(p), 3))
    L.cpo_vp_direct_velocity(_p(pos), _p(st), _p(rad), len(pos), _p(p), len(p), 1 if kernel == "gauss" else 2,
                             _p(out))
    return out


def particles_stretch(pos, strength, radius):
    L = lib()
    pos, st, rad = _parts(pos, strength, radius)
    out = np.zeros((len(pos), 3))
    L.cpo_vp_direct_stretch(_p(pos), _p(st), _p(rad), len(pos), _p(out))
    return out


def particles_diffusion(pos, strength, radius):
    L = lib()
    pos, st, rad = _parts(pos, strength, radius)
    out = np.zeros((len(pos), 3))
    L.cpo_vp_direct_diffusion(_p(pos), _p(st), _p(rad), len(pos), _p(out))
    return out


class ParticleTree:
    """particleOctree + particleFMM: insertion-order octree with lumped expansions."""

    NODE_FIELDS = 24

    def __init__(self, pos, strength, radius, max_members=10, theta=0.5):
        L = lib()
        self.pos, self.strength, self.radius = _parts(pos, strength, radius)
        self.h = L.cpo_bh_build(_p(self.pos), _p(self.strength), _p(self.radius), len(self.pos), max_members, theta)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().cpo_bh_free(h)
            self.h = None

    @property
    def n_nodes(self):
        return lib().cpo_bh_num_nodes(self.h)

    @property
    def n_levels(self):
        return lib().cpo_bh_num_levels(self.h)

    def nodes(self):
        out = np.zeros((self.n_nodes, self.NODE_FIELDS))
        lib().cpo_bh_nodes(self.h, _p(out))
        return out

    def leaf_members(self):
        out = np.zeros(len(self.pos), dtype=np.int64)
        lib().cpo_bh_leaf_members(self.h, _p(out, I64))
        return out

    def velocity_points(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(p), 3))
        lib().cpo_bh_velocity(self.h, _p(p), len(p), 0, _p(out))
        return out

    def velocity(self):
        out = np.zeros((len(self.pos), 3))
        lib().cpo_bh_velocity(self.h, None, 0, 1, _p(out))
        return out

    def stretch(self):
        out = np.zeros((len(self.pos), 3))
        lib().cpo_bh_stretch(self.h, _p(out))
        return out

    def diffusion(self):
        out = np.zeros((len(self.pos), 3))
        lib().cpo_bh_diffusion(self.h, _p(out))
        return out


def panels_stretching(bverts, sigma, mu, wverts, wmu, pos, strength):
    """Sum of bodyPanel::partStretching (triangles) and wakePanel::partStretching (quads)."""
    L = lib()
    bv = np.ascontiguousarray(bverts, dtype=np.float64).reshape(-1, 9)
    wv = np.ascontiguousarray(wverts, dtype=np.float64).reshape(-1, 12)
    p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    st = np.ascontiguousarray(strength, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((len(p), 3))
    L.cpo_panels_stretching(_p(bv), _p(np.ascontiguousarray(sigma, dtype=np.float64)),
                            _p(np.ascontiguousarray(mu, dtype=np.float64)), len(bv), _p(wv),
                            _p(np.ascontiguousarray(wmu, dtype=np.float64)), len(wv), _p(p), _p(st), len(p), _p(out))
    return out


class VPCase:
    """cpCaseVP on a body-only mesh: buffer wake, shedding, stretching, AB2 time loop."""

    def __init__(self, nodes, tris, ids, V=1.0, alpha=5.0, beta=0.0, dt=0.0, cref=1.0, accelerate=True, num_steps=10,
                 Sref=1.0, mach=0.0):
        L = lib()
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.tris = np.ascontiguousarray(tris, dtype=np.int64)
        self.ids = np.ascontiguousarray(ids, dtype=np.int32)
        self.h = L.cpo_vpcase_new(_p(self.nodes), len(self.nodes), _p(self.tris, I64), _p(self.ids, I32),
                                  len(self.tris), V, alpha, beta, dt, cref, 1 if accelerate else 0, num_steps)
        if not self.h:
            raise ValueError("mesh has wake panels; the vortex-particle case builds its own")
        L.cpo_vpcase_set_refs(self.h, Sref, mach)

    def trefftz(self, row=0):
        """Trefftz-plane CL, CD of the current state; row > 0 integrates over the particles
        shed at that step in place of the reference's row."""
        out = np.zeros(3)
        lib().cpo_vpcase_trefftz_row(self.h, int(row), _p(out))
        return dict(CL=out[0], CD=out[1], converged=bool(out[2]))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().cpo_vpcase_free(h)
            self.h = None

    def info(self):
        out = np.zeros(7, dtype=np.int64)
        lib().cpo_vpcase_info(self.h, _p(out, I64))
        return dict(n_body=int(out[0]), n_w1=int(out[1]), n_w2=int(out[2]), n_particles=int(out[3]),
                    timestep=int(out[4]), n_nodes=int(out[5]), last_iters=int(out[6]))

    @property
    def dt(self):
        return lib().cpo_vpcase_dt(self.h)

    def wake(self):
        i = self.info()
        w1 = np.zeros((i["n_w1"], 12))
        w2 = np.zeros((i["n_w2"], 12))
        cols = np.zeros((i["n_w1"], 4), dtype=np.int32)
        coef = np.zeros(i["n_w1"])
        lib().cpo_vpcase_wake(self.h, _p(w1), _p(w2), _p(cols, I32), _p(coef))
        return w1, w2, cols, coef

    def matrices(self):
        i = self.info()
        n = i["n_body"]
        A = np.zeros((n, n), order="F")
        B = np.zeros((n, n), order="F")
        Cm = np.zeros((n, i["n_w2"]), order="F")
        lib().cpo_vpcase_matrices(self.h, _p(A), _p(B), _p(Cm))
        return A, B, Cm

    def step(self):
        return lib().cpo_vpcase_step(self.h)

    def particles(self):
        n = self.info()["n_particles"]
        pos, st, rad = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        shed, parent = np.zeros(n, dtype=np.int32), np.zeros(n, dtype=np.int32)
        lib().cpo_vpcase_particles(self.h, _p(pos), _p(st), _p(rad), _p(shed, I32), _p(parent, I32))
        return dict(pos=pos, strength=st, radius=rad, shed_time=shed, parent=parent)

    def strengths(self):
        i = self.info()
        sg, mu = np.zeros(i["n_body"]), np.zeros(i["n_body"])
        m1, m2 = np.zeros(i["n_w1"]), np.zeros(i["n_w2"])
        lib().cpo_vpcase_strengths(self.h, _p(sg), _p(mu), _p(m1), _p(m2))
        return dict(sigma=sg, mu=mu, mu_w1=m1, mu_w2=m2)

    def surface(self, cg=(0.0, 0.0, 0.0), bref=1.0, cref=1.0):
        """cpCaseVP::compVelocity on the current state: phi, V, Cp per panel and the body,
        wind and moment coefficients."""
        n = self.info()["n_body"]
        phi, vel, cp, f = np.zeros(n), np.zeros((n, 3)), np.zeros(n), np.zeros(9)
        cgv = np.ascontiguousarray(cg, dtype=np.float64)
        lib().cpo_vpcase_surface(self.h, _p(cgv), bref, cref, _p(phi), _p(vel), _p(cp), _p(f))
        return dict(phi=phi, vel=vel, cp=cp, Fbody=f[0:3], Fwind=f[3:6], CM=f[6:9])
