"""Vortex-particle operators: host-side mirror of particleOctree / particleFMM / particle.

Tensors are CUDA float64 tensors: positions and strengths (n, 3), radii (n,).
The calls go through include/cpanel_vp.h; there is no CPU fallback.

    tree = ParticleFMM(pos, strength, radius)          # particleOctree::addData + particleFMM::build
    v_pts = tree.barnesHutVel(points)                  # barnesHutVel(POI), CPanel/particleFMM.cpp:65-77
    v, s, d = tree.barnesHut()                         # barnesHutVel(part) / Stretch / Diff, :79-116
    v = particles_velocity(pos, strength, radius)      # direct sums (particle.cpp:31-77)
    s, d = particles_stretch_diff(pos, strength, radius)
    v = panels_velocity(body_verts, sigma, mu, wake_verts, wake_mu, points)
"""
import ctypes as C

import numpy as np

from . import _lib, _shutting_down_now
from ._lib import VEL_ALG, VEL_GAUSS, VEL_GAUSS_SYM

NODE_FIELDS = 24
_KERNELS = {"gauss_sym": VEL_GAUSS_SYM, "gauss": VEL_GAUSS, "alg": VEL_ALG}


def _ctx(ctx):
    from . import Context
    return ctx or Context.default()


def _dev(t, cols=None):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("expected a CUDA tensor")
    t = t.contiguous().to(torch.float64)
    if cols is not None and (t.dim() != 2 or t.shape[1] != cols):
        t = t.reshape(-1, cols)
    return t


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _sync():
    import torch
    torch.cuda.synchronize()


def _precision(p):
    return {"plain": _lib.PLAIN_FP64, "mixed": _lib.MIXED}[p]


class ParticleFMM:
    """Barnes-Hut octree over one particle set (fresh build, as the VP loop does every step)."""

    def __init__(self, pos, strength, radius, max_members=10, theta=0.5, precision="plain", ctx=None):
        self.ctx = _ctx(ctx)
        self.pos, self.strength, self.radius = _dev(pos, 3), _dev(strength, 3), _dev(radius).reshape(-1)
        self.n = self.pos.shape[0]
        h = C.c_void_p()
        _sync()
        self.ctx.check(self.ctx.L.cpg_ptree_build(self.ctx.h, _ptr(self.pos), _ptr(self.strength), _ptr(self.radius),
                                                  self.n, max_members, theta, C.byref(h)), "particle tree")
        self.h = h
        self.set_precision(precision)

    def set_precision(self, precision):
        """"plain": every interaction in FP64; "mixed": far nodes in FP32, leaves (the
        direct near field) in FP64, the same traversal decisions."""
        code = _precision(precision)
        self.ctx.check(self.ctx.L.cpg_ptree_set_precision(self.h, code), "tree precision")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            if not _shutting_down_now():
                self.ctx.L.cpg_ptree_destroy(h)
            self.h = None

    def info(self):
        i = _lib.PTreeInfo()
        self.ctx.check(self.ctx.L.cpg_ptree_info_get(self.h, C.byref(i)), "tree info")
        return {"n_particles": i.n_particles, "n_nodes": i.n_nodes, "n_leaves": i.n_leaves, "n_levels": i.n_levels}

    def numTreeLevels(self):
        return self.info()["n_levels"]

    def nodes(self):
        """(n_nodes, 24) pre-order node table: origin half level leaf n_members exp_pos exp_strength
        exp_radius child0..7."""
        out = np.zeros((self.info()["n_nodes"], NODE_FIELDS))
        self.ctx.check(self.ctx.L.cpg_ptree_table(self.h, out.ctypes.data_as(_lib.D), None), "tree table")
        return out

    def leaf_members(self):
        out = np.zeros(self.n, dtype=np.int64)
        self.ctx.check(self.ctx.L.cpg_ptree_table(self.h, None, out.ctypes.data_as(_lib.I64)), "tree table")
        return out

    def barnesHutVel(self, points):
        import torch
        pts = _dev(points, 3)
        vel = torch.empty_like(pts)
        _sync()
        self.ctx.check(self.ctx.L.cpg_bh_velocity_points(self.h, _ptr(pts), pts.shape[0], _ptr(vel)),
                       "barnesHutVel")
        return vel

    def barnesHut(self, vel=True, stretch=True, diff=True):
        """(velocity, stretching, diffusion) on every particle; None for the ones not asked."""
        import torch
        outs = [torch.empty((self.n, 3), dtype=torch.float64, device=self.pos.device) if w else None
                for w in (vel, stretch, diff)]
        _sync()
        self.ctx.check(self.ctx.L.cpg_bh_particles(self.h, *[_ptr(o) for o in outs]), "barnesHut")
        return tuple(outs)

    def barnesHutVelParticles(self):
        return self.barnesHut(True, False, False)[0]

    def barnesHutStretch(self):
        return self.barnesHut(False, True, False)[1]

    def barnesHutDiff(self):
        return self.barnesHut(False, False, True)[2]


def host_tree(pos, strength, radius, max_members=10):
    """The same octree built on the host from numpy arrays: (node table, leaf members, info)."""
    L = _lib.load()
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    st = np.ascontiguousarray(strength, dtype=np.float64).reshape(-1, 3)
    rad = np.ascontiguousarray(radius, dtype=np.float64).reshape(-1)
    info = _lib.PTreeInfo()
    members = np.zeros(len(pos), dtype=np.int64)
    D = _lib.D
    rc = L.cpg_ptree_host_table(pos.ctypes.data_as(D), st.ctypes.data_as(D), rad.ctypes.data_as(D), len(pos),
                                max_members, None, 0, members.ctypes.data_as(_lib.I64), C.byref(info))
    if rc != 0:
        raise _lib.CpgError(rc, "host tree")
    nodes = np.zeros((info.n_nodes, NODE_FIELDS))
    rc = L.cpg_ptree_host_table(pos.ctypes.data_as(D), st.ctypes.data_as(D), rad.ctypes.data_as(D), len(pos),
                                max_members, nodes.ctypes.data_as(D), info.n_nodes, None, C.byref(info))
    if rc != 0:
        raise _lib.CpgError(rc, "host tree")
    return nodes, members, {"n_particles": info.n_particles, "n_nodes": info.n_nodes, "n_leaves": info.n_leaves,
                            "n_levels": info.n_levels}


def particles_velocity(pos, strength, radius, points=None, kernel="gauss", ctx=None):
    """Direct sum of particle velocity kernels at `points` (or at the particles when None)."""
    import torch
    ctx = _ctx(ctx)
    pos, st, rad = _dev(pos, 3), _dev(strength, 3), _dev(radius).reshape(-1)
    pts = _dev(points, 3) if points is not None else None
    m = pts.shape[0] if pts is not None else pos.shape[0]
    vel = torch.empty((m, 3), dtype=torch.float64, device=pos.device)
    _sync()
    ctx.check(ctx.L.cpg_particles_velocity(ctx.h, _ptr(pos), _ptr(st), _ptr(rad), pos.shape[0], _ptr(pts), m,
                                           _KERNELS[kernel], _ptr(vel)), "particle velocity")
    return vel


def particles_stretch_diff(pos, strength, radius, ctx=None):
    import torch
    ctx = _ctx(ctx)
    pos, st, rad = _dev(pos, 3), _dev(strength, 3), _dev(radius).reshape(-1)
    s = torch.empty_like(pos)
    d = torch.empty_like(pos)
    _sync()
    ctx.check(ctx.L.cpg_particles_stretch_diff(ctx.h, _ptr(pos), _ptr(st), _ptr(rad), pos.shape[0], _ptr(s), _ptr(d)),
              "particle strength update")
    return s, d


class _OperatorPrecision:
    """Sets the context's panel-particle operator precision for one call."""

    def __init__(self, ctx, precision):
        self.ctx, self.code = ctx, _precision(precision)

    def __enter__(self):
        self.ctx.check(self.ctx.L.cpg_set_particle_precision(self.ctx.h, self.code), "operator precision")

    def __exit__(self, *a):
        self.ctx.L.cpg_set_particle_precision(self.ctx.h, _lib.PLAIN_FP64)


def panels_velocity(body_verts, sigma, mu, wake_verts, wake_mu, points, precision="plain", ctx=None):
    """Sum of bodyPanel::panelV (triangles) and wake-triangle dubVInf at points; "mixed"
    evaluates body pairs beyond five panel lengths in FP32."""
    import torch
    ctx = _ctx(ctx)
    bv = _dev(body_verts, 9)
    sg, mu_ = _dev(sigma).reshape(-1), _dev(mu).reshape(-1)
    nw = 0 if wake_verts is None else int(np.prod(wake_verts.shape)) // 9
    wv = _dev(wake_verts, 9) if nw else None
    wm = _dev(wake_mu).reshape(-1) if nw else None
    pts = _dev(points, 3)
    vel = torch.empty_like(pts)
    _sync()
    with _OperatorPrecision(ctx, precision):
        ctx.check(ctx.L.cpg_panels_velocity(ctx.h, _ptr(bv), _ptr(sg), _ptr(mu_), bv.shape[0], _ptr(wv), _ptr(wm), nw,
                                            _ptr(pts), pts.shape[0], _ptr(vel)), "panel velocity")
    return vel


def panels_stretching(body_verts, sigma, mu, wake_verts, wake_mu, pos, strength, precision="plain", ctx=None):
    """Sum of bodyPanel::partStretching (triangles) and wakePanel::partStretching (quads);
    "mixed" evaluates body pairs beyond five panel lengths in FP32."""
    import torch
    ctx = _ctx(ctx)
    bv = _dev(body_verts, 9)
    sg, mu_ = _dev(sigma).reshape(-1), _dev(mu).reshape(-1)
    nw = 0 if wake_verts is None else int(np.prod(wake_verts.shape)) // 12
    wv = _dev(wake_verts, 12) if nw else None
    wm = _dev(wake_mu).reshape(-1) if nw else None
    p, st = _dev(pos, 3), _dev(strength, 3)
    out = torch.empty_like(p)
    _sync()
    with _OperatorPrecision(ctx, precision):
        ctx.check(ctx.L.cpg_panels_stretching(ctx.h, _ptr(bv), _ptr(sg), _ptr(mu_), bv.shape[0], _ptr(wv), _ptr(wm),
                                              nw, _ptr(p), _ptr(st), p.shape[0], _ptr(out)), "panel stretching")
    return out


def vp_topology(nodes, tris, ids, V=1.0, dt=0.0):
    """Host-only buffer wake: dict(counts, dt, w1, w2, w1_idx, w1_coef, w2_parent)."""
    L = _lib.load()
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int64)
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    counts = np.zeros(3, dtype=np.int64)
    dto = C.c_double(0)
    args = (nodes.ctypes.data_as(_lib.D), len(nodes), tris.ctypes.data_as(_lib.I64), ids.ctypes.data_as(_lib.I32),
            len(tris), V, dt, counts.ctypes.data_as(_lib.I64), C.byref(dto))
    rc = L.cpg_vp_topology(*args, None, None, None, None, None)
    if rc != 0:
        raise _lib.CpgError(rc, "vp topology")
    n1, n2 = int(counts[1]), int(counts[2])
    w1, w2 = np.zeros((n1, 12)), np.zeros((n2, 12))
    idx, coef, par = np.zeros((n1, 4), dtype=np.int32), np.zeros(n1), np.zeros(n2, dtype=np.int32)
    L.cpg_vp_topology(*args, w1.ctypes.data_as(_lib.D), w2.ctypes.data_as(_lib.D), idx.ctypes.data_as(_lib.I32),
                      coef.ctypes.data_as(_lib.D), par.ctypes.data_as(_lib.I32))
    return dict(counts=counts, dt=dto.value, w1=w1, w2=w2, w1_idx=idx, w1_coef=coef, w2_parent=par)


class VPCase:
    """cpCaseVP on a body-only mesh, advanced step by step on the GPU."""

    def __init__(self, nodes, tris, ids, V=1.0, alpha=5.0, beta=0.0, dt=0.0, cref=1.0, accelerate=True, Sref=1.0,
                 mach=0.0, precision="plain", run_all_steps=False, ctx=None):
        self.ctx = _ctx(ctx)
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int64)
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        prm = _lib.VPParams(V, alpha, beta, dt, cref, 1 if accelerate else 0, Sref, mach, _precision(precision),
                            1 if run_all_steps else 0)
        h = C.c_void_p()
        self.ctx.check(self.ctx.L.cpg_vpcase_create(self.ctx.h, nodes.ctypes.data_as(_lib.D), len(nodes),
                                                    tris.ctypes.data_as(_lib.I64), ids.ctypes.data_as(_lib.I32),
                                                    len(tris), C.byref(prm), C.byref(h)), "vortex-particle case")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            if not _shutting_down_now():
                self.ctx.L.cpg_vpcase_destroy(h)
            self.h = None

    def info(self):
        i = _lib.VPInfo()
        self.ctx.check(self.ctx.L.cpg_vpcase_info_get(self.h, C.byref(i)), "info")
        return {f: getattr(i, f) for f, _ in _lib.VPInfo._fields_}

    def step(self, n=1):
        self.ctx.check(self.ctx.L.cpg_vpcase_step(self.h, n), "step")
        return self.info()["timestep"]

    def trefftz(self):
        """Trefftz-plane CL, CD of the current state and whether the run has converged."""
        cl, cd, cv = C.c_double(), C.c_double(), C.c_int()
        self.ctx.check(self.ctx.L.cpg_vpcase_trefftz(self.h, C.byref(cl), C.byref(cd), C.byref(cv)), "trefftz")
        return dict(CL=cl.value, CD=cd.value, converged=bool(cv.value))

    def velocities(self, precision="plain", direct=False):
        """Convective velocity of every particle at the current state (n x 3)."""
        n = self.info()["n_particles"]
        out = np.zeros((n, 3))
        self.ctx.check(self.ctx.L.cpg_vpcase_velocities(self.h, _precision(precision), 1 if direct else 0,
                                                        out.ctypes.data_as(_lib.D)), "velocities")
        return out

    def particles(self):
        n = self.info()["n_particles"]
        pos, st, rad = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        shed, par = np.zeros(n, dtype=np.int32), np.zeros(n, dtype=np.int32)
        self.ctx.check(self.ctx.L.cpg_vpcase_particles(self.h, pos.ctypes.data_as(_lib.D), st.ctypes.data_as(_lib.D),
                                                       rad.ctypes.data_as(_lib.D), shed.ctypes.data_as(_lib.I32),
                                                       par.ctypes.data_as(_lib.I32)), "particles")
        return dict(pos=pos, strength=st, radius=rad, shed_time=shed, parent=par)

    def strengths(self):
        i = self.info()
        sg, mu = np.zeros(i["n_body"]), np.zeros(i["n_body"])
        m1, m2 = np.zeros(i["n_w1"]), np.zeros(i["n_w2"])
        self.ctx.check(self.ctx.L.cpg_vpcase_strengths(self.h, sg.ctypes.data_as(_lib.D), mu.ctypes.data_as(_lib.D),
                                                       m1.ctypes.data_as(_lib.D), m2.ctypes.data_as(_lib.D)),
                       "strengths")
        return dict(sigma=sg, mu=mu, mu_w1=m1, mu_w2=m2)

    def surface(self, cg=(0.0, 0.0, 0.0), bref=1.0, cref=1.0):
        """cpCaseVP::compVelocity on the current state (steady case): potential, surface
        velocity and Cp per panel, and the body, wind and moment coefficients."""
        n = self.info()["n_body"]
        phi, vel, cp, f = np.zeros(n), np.zeros((n, 3)), np.zeros(n), np.zeros(9)
        cgv = np.ascontiguousarray(cg, dtype=np.float64)
        self.ctx.check(self.ctx.L.cpg_vpcase_surface(self.h, cgv.ctypes.data_as(_lib.D), bref, cref,
                                                     phi.ctypes.data_as(_lib.D), vel.ctypes.data_as(_lib.D),
                                                     cp.ctypes.data_as(_lib.D), f.ctypes.data_as(_lib.D)), "surface")
        return dict(phi=phi, vel=vel, cp=cp, Fbody=f[0:3], Fwind=f[3:6], CM=f[6:9])

    def matrices(self):
        i = self.info()
        n, n2 = i["n_body"], i["n_w2"]
        A, B, Cm = np.zeros((n, n), order="F"), np.zeros((n, n), order="F"), np.zeros((n, n2), order="F")
        self.ctx.check(self.ctx.L.cpg_vpcase_matrices(self.h, A.ctypes.data_as(_lib.D), B.ctypes.data_as(_lib.D),
                                                      Cm.ctypes.data_as(_lib.D)), "matrices")
        return A, B, Cm
