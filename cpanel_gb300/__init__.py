"""GB300-native steady panel path of CPanel.

Host-side mirror of the reference's operator surface for this path:

  Geometry      geometry::readTri + setInfCoeff/getA/getB (CPanel/geometry.cpp:132-891)
  CpCase        cpCase::run results (CPanel/cpCase.cpp:31-139): getCL/getCD,
                getBodyForces/getWindForces/getMoment, per-panel mu/phi/V/Cp
  solve_cases   many flow conditions on one geometry in one batched call
  panel_phi_inf / dub_phi_inf / panel_v_inf
                bodyPanel::panelPhiInf, panel::dubPhiInf, bodyPanel::panelVInf on
                device arrays

All compute runs in libcpanel_gb300.so (sm_103a); this module only marshals
arguments.  There is no CPU fallback.
"""
import atexit
import os
import ctypes as C
import sys

import numpy as np

from . import _lib
from ._lib import MIXED, PLAIN_FP64, CpgError

__all__ = ["Context", "Geometry", "CpCase", "solve_cases", "topology", "read_tri", "streamlines_field", "panel_phi_inf", "dub_phi_inf",
           "panel_v_inf", "CpgError", "PLAIN_FP64", "MIXED"]

_shutting_down = False


@atexit.register
def _mark_shutdown():
    global _shutting_down
    _shutting_down = True


def _shutting_down_now():
    return _shutting_down or sys.is_finalizing()


_PREC = {"fp64": PLAIN_FP64, "plain": PLAIN_FP64, PLAIN_FP64: PLAIN_FP64, "mixed": MIXED, MIXED: MIXED}


def _p(a, t=_lib.D):
    return a.ctypes.data_as(t)


class Context:
    """One device context (stream + error state).  Thread-compatible, not shared."""

    _default = None

    def __init__(self, device=0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.cpg_create(C.byref(h), device)
        if rc != 0:
            raise CpgError(rc, "cpg_create(device=%d)" % device)
        self.h = h

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def check(self, rc, what=""):
        if rc != 0:
            msg = self.L.cpg_last_error(self.h)
            raise CpgError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def synchronize(self):
        self.check(self.L.cpg_synchronize(self.h), "synchronize")

    def release_spares(self):
        """Free the matrix buffers kept from destroyed geometries (cpg_release_spares)."""
        self.check(self.L.cpg_release_spares(self.h), "release_spares")

    def prof_enable(self, on=True):
        self.check(self.L.cpg_prof_enable(self.h, 1 if on else 0), "prof_enable")

    def prof_read(self):
        p = _lib.Prof()
        self.check(self.L.cpg_prof_read(self.h, C.byref(p)), "prof_read")
        return {name: (p.launches[i], p.ms[i]) for i, name in enumerate(_lib.PROF_CLASSES)}

    def __del__(self):
        if _shutting_down or sys.is_finalizing():
            return  # the CUDA runtime may already be unloaded
        try:
            self.L.cpg_destroy(self.h)
        except Exception:
            pass


def read_tri(path):
    """Cart3D .tri file -> (nodes[n,3], tris[nt,3] 1-based, ids[nt]) (geometry::readTri input format)."""
    with open(path) as f:
        tok = f.read().split()
    nn, nt = int(tok[0]), int(tok[1])
    k = 2
    nodes = np.array(tok[k:k + 3 * nn], dtype=np.float64).reshape(nn, 3)
    k += 3 * nn
    tris = np.array(tok[k:k + 3 * nt], dtype=np.int64).reshape(nt, 3)
    k += 3 * nt
    ids = np.array(tok[k:k + nt], dtype=np.int32)
    return nodes, tris, ids


class Geometry:
    """geometry: .tri topology on the host, panel tables and matrices on the device."""

    def __init__(self, nodes, tris, ids, ctx=None):
        self.ctx = ctx or Context.default()
        L = self.ctx.L
        self._nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self._tris = np.ascontiguousarray(tris, dtype=np.int64)
        self._ids = np.ascontiguousarray(ids, dtype=np.int32)
        h = C.c_void_p()
        self.ctx.check(L.cpg_geometry_create(self.ctx.h, _p(self._nodes), len(self._nodes), _p(self._tris, _lib.I64),
                                             _p(self._ids, _lib.I32), len(self._ids), C.byref(h)),
                       "cpg_geometry_create")
        self.h = h
        info = _lib.GeometryInfo()
        self.ctx.check(L.cpg_geometry_info_get(self.h, C.byref(info)), "info")
        self.info = {f: getattr(info, f) for f, _ in info._fields_}
        self.n = info.n_body
        self.nw = info.n_wake

    @classmethod
    def from_tri(cls, path, ctx=None):
        return cls(*read_tri(path), ctx=ctx)

    def __del__(self):
        if _shutting_down or sys.is_finalizing():
            return
        try:
            self.ctx.L.cpg_geometry_destroy(self.h)
        except Exception:
            pass

    def getNumberOfBodyPanels(self):
        return self.n

    def setInfCoeff(self, precision="fp64"):
        self.ctx.check(self.ctx.L.cpg_set_inf_coeff(self.h, _PREC[precision]), "setInfCoeff")

    def getA(self):
        A = np.empty((self.n, self.n), order="F")
        self.ctx.check(self.ctx.L.cpg_get_A(self.h, _p(A)), "getA")
        return A

    def getB(self):
        B = np.empty((self.n, self.n), order="F")
        self.ctx.check(self.ctx.L.cpg_get_B(self.h, _p(B)), "getB")
        return B

    def tables(self):
        body = np.zeros((self.n, 18))
        wake = np.zeros((self.nw, 8))
        idx = np.zeros((self.nw, 4), dtype=np.int32)
        coef = np.zeros(self.nw)
        cl = np.zeros((self.n, 32), dtype=np.int32)
        self.ctx.check(self.ctx.L.cpg_geometry_tables(self.h, _p(body), _p(wake), _p(idx, _lib.I32), _p(coef),
                                                      _p(cl, _lib.I32)), "tables")
        return dict(body=body, wake=wake, idx4=idx, coef=coef, clusters=cl)


def topology(nodes, tris, ids):
    """Host-only readTri topology tables (no device needed)."""
    L = _lib.load()
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int64)
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    info = _lib.GeometryInfo()
    args = (_p(nodes), len(nodes), _p(tris, _lib.I64), _p(ids, _lib.I32), len(ids), C.byref(info))
    rc = L.cpg_topology(*args, None, None, None, None, None)
    if rc != 0:
        raise CpgError(rc, "cpg_topology")
    n, nw = info.n_body, info.n_wake
    body, wake = np.zeros((n, 18)), np.zeros((nw, 8))
    idx, coef, cl = np.zeros((nw, 4), dtype=np.int32), np.zeros(nw), np.zeros((n, 32), dtype=np.int32)
    rc = L.cpg_topology(*args, _p(body), _p(wake), _p(idx, _lib.I32), _p(coef), _p(cl, _lib.I32))
    if rc != 0:
        raise CpgError(rc, "cpg_topology")
    return dict(info={f: getattr(info, f) for f, _ in info._fields_}, body=body, wake=wake, idx4=idx, coef=coef,
                clusters=cl)


def solve_cases(geom, flows, Sref=1.0, bref=1.0, cref=1.0, cg=(0.0, 0.0, 0.0), precision="fp64", want=None):
    """Run cpCase::run for k flow conditions (V, alpha, beta, mach) on one geometry.

    Returns a dict with per-case arrays (mu, sigma, phi, vel, cp: k x n [x 3]) and
    CL, CDi (k), Fbody, Fwind, CM (k x 3), plus solver statistics.
    """
    flows = [tuple(f) for f in flows]
    k = len(flows)
    fl = (_lib.Flow * k)(*[_lib.Flow(*f) for f in flows])
    refs = _lib.Refs(Sref, bref, cref, (C.c_double * 3)(*cg))
    n = geom.n
    # want=None: every per-panel output; an empty tuple: none (coefficients only)
    want = ("mu", "sigma", "phi", "vel", "cp") if want is None else tuple(want)
    out = {name: np.zeros((k, n)) for name in ("mu", "sigma", "phi", "cp") if name in want}
    if "vel" in want:
        out["vel"] = np.zeros((k, n, 3))
    for name in ("CL", "CDi"):
        out[name] = np.zeros(k)
    for name in ("Fbody", "Fwind", "CM"):
        out[name] = np.zeros((k, 3))
    co = _lib.CaseOut(*[_p(out[f]) if f in out else None for f, _ in _lib.CaseOut._fields_])
    st = _lib.SolveStats()
    rc = geom.ctx.L.cpg_solve_cases(geom.h, fl, k, C.byref(refs), _PREC[precision], C.byref(co), C.byref(st))
    out["stats"] = {f: getattr(st, f) for f, _ in st._fields_}
    out["status"] = rc
    if rc not in (0, 5):
        geom.ctx.check(rc, "solve_cases")
    return out


def spanwise_loads(geom, case=0, wake=0):
    """The spanwise Trefftz-plane loads of one case of the last solve_cases call on geom and one of its
    wakes, as cpCase::writeSpanwiseData scales them (CPanel/cpCase.cpp:910-935): a dict of 2y/b ("y2b"),
    Cl / PG ("cl") and Cdi / PG^2 ("cdi") at the reference's 165 stations."""
    n = C.c_int(512)
    out = {k: np.zeros(512) for k in ("y2b", "cl", "cdi")}
    geom.ctx.check(geom.ctx.L.cpg_spanwise_loads(geom.h, case, wake, _p(out["y2b"]), _p(out["cl"]), _p(out["cdi"]),
                                                 C.byref(n)), "spanwise_loads")
    return {k: v[:n.value].copy() for k, v in out.items()}


class CpCase:
    """cpCase: one flow condition on a geometry (CPanel/cpCase.h:127-136)."""

    def __init__(self, geom, V, alpha, beta, mach, Sref=1.0, bref=1.0, cref=1.0, cg=(0, 0, 0), precision="fp64"):
        self.geom = geom
        self.flow = (V, alpha, beta, mach)
        self.refs = dict(Sref=Sref, bref=bref, cref=cref, cg=cg)
        self.precision = precision
        self.res = None
        self.stab = None
        self.survey = None
        self.lines = None

    def run(self):
        self.res = solve_cases(self.geom, [self.flow], precision=self.precision, **self.refs)
        # the spanwise loads of every wake, read before another solve replaces them
        self.span = [spanwise_loads(self.geom, 0, w) for w in range(self.geom.ctx.L.cpg_trefftz_wakes(self.geom.h))]
        return self.res["status"] == 0

    def getCL(self):
        return self.res["CL"][0]

    def getCD(self):
        return self.res["CDi"][0]

    def getBodyForces(self):
        return self.res["Fbody"][0]

    def getWindForces(self):
        return self.res["Fwind"][0]

    def getMoment(self):
        return self.res["CM"][0]

    def getMu(self):
        return self.res["mu"][0]

    def getCp(self):
        return self.res["cp"][0]

    def getVelocity(self):
        return self.res["vel"][0]

    def stabilityDerivatives(self):
        """cpCase::stabilityDerivatives (CPanel/cpCase.cpp:635-665): the base case and the two
        0.5 deg sub-cases as three right-hand sides of one solve, forward differences per
        radian.  Also runs the base case (its results as run() gives them).  Returns dict(
        dF_dAlpha, dF_dBeta: (CD, CY, CL); dM_dAlpha, dM_dBeta: (roll, pitch, yaw))."""
        g = self.geom
        n = g.n
        res = {name: np.zeros((1, n)) for name in ("mu", "sigma", "phi", "cp")}
        res["vel"] = np.zeros((1, n, 3))
        for name in ("CL", "CDi"):
            res[name] = np.zeros(1)
        for name in ("Fbody", "Fwind", "CM"):
            res[name] = np.zeros((1, 3))
        co = _lib.CaseOut(*[_p(res[f]) for f, _ in _lib.CaseOut._fields_])
        st = _lib.Stability()
        fl = _lib.Flow(*self.flow)
        refs = _lib.Refs(self.refs["Sref"], self.refs["bref"], self.refs["cref"], (C.c_double * 3)(*self.refs["cg"]))
        rc = g.ctx.L.cpg_stability_derivatives(g.h, C.byref(fl), C.byref(refs), _PREC[self.precision], C.byref(co),
                                               C.byref(st))
        if rc not in (0, 5):
            g.ctx.check(rc, "stabilityDerivatives")
        res["status"] = rc
        self.res = res
        self.stab = {k: np.array(getattr(st, k)[:]) for k in ("dF_dAlpha", "dF_dBeta", "dM_dAlpha", "dM_dBeta")}
        return self.stab

    def velocityAtPoints(self, pts):
        """cpCase::velocityAtPoint (CPanel/cpCase.cpp:1007-1021) for many points: the velocity all
        body and wake panels induce (V_inf not included), for this case's strengths."""
        g = self.geom
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        vel = np.zeros_like(pts)
        sig = np.ascontiguousarray(self.res["sigma"][0])
        mu = np.ascontiguousarray(self.res["mu"][0])
        g.ctx.check(g.ctx.L.cpg_volume_velocity(g.h, _p(sig), _p(mu), _p(pts), len(pts), _p(vel)), "velocityAtPoints")
        return vel

    def streamlines(self, starts, x_max, tol=1e-4, max_points=1000):
        """Off-body streamlines (streamline::streamline / rkf, CPanel/streamline.cpp:20-78) from the
        start points (k x 3) to x_max, through geometry::pntVelocity (panels + V_inf, x divided by
        the Prandtl-Glauert factor).  All lines advance together, one batched panel-velocity launch
        per Runge-Kutta stage.  Returns (lines, ended) as streamlines_field does."""
        g = self.geom
        st = np.ascontiguousarray(starts, dtype=np.float64).reshape(-1, 3)
        n = len(st)
        pts = np.zeros((n, max_points, 3))
        vel = np.zeros((n, max_points, 3))
        counts = np.zeros(n, dtype=np.int32)
        ended = np.zeros(n, dtype=np.int32)
        sig = np.ascontiguousarray(self.res["sigma"][0])
        mu = np.ascontiguousarray(self.res["mu"][0])
        fl = _lib.Flow(*[float(x) for x in self.flow])
        g.ctx.check(g.ctx.L.cpg_streamlines(g.h, _p(sig), _p(mu), C.byref(fl), _p(st), n, float(x_max), float(tol),
                                            int(max_points), _p(pts), _p(vel), _p(counts, _lib.I32),
                                            _p(ended, _lib.I32)), "streamlines")
        lines, ended = _streamline_lines(pts, vel, counts, ended)
        self.lines = lines
        return lines, ended

    def vinf(self):
        """V_inf in body axes (cpCase::windToBody, CPanel/cpCase.cpp:142-165)."""
        V, alpha, beta, _ = self.flow
        a, b = np.radians(alpha), np.radians(beta)
        return V * np.array([np.cos(a) * np.cos(b), -np.sin(b), np.sin(a) * np.cos(b)])

    def volumeSurvey(self, bounds, res):
        """cpCase::createVolMesh + populateVolMesh (CPanel/cpCase.cpp:1024-1122): velocity and Cp at
        the cell centres of a structured grid.  Cp is the reference's (|V| / V_inf)^2, as written
        there (not 1 - (|V| / V_inf)^2).  Returns dict(points, cells, centers, velocity, cp)."""
        from . import io
        pts, cells, centers = io.volume_grid(bounds, res)
        vel = self.velocityAtPoints(centers) + self.vinf()
        cp = (np.linalg.norm(vel, axis=1) / self.flow[0]) ** 2
        self.survey = dict(points=pts, cells=cells, centers=centers, velocity=vel, cp=cp)
        return self.survey

    def writeFiles(self, directory=".", geom_file=""):
        """cpCase::writeFiles (CPanel/cpCase.cpp:667-709): the case directory
        V<V>_Mach<M>_alpha<a>_beta<b> under `directory` with surfaceData.vtu, wakeData.vtu (when
        the mesh has wake panels), spanwiseData_Wake<i>.csv per wake, volumeMesh.vtu (after volumeSurvey),
        OffBodyStreamlines.vtu
        (after streamlines; the reference's name for off-body lines, CPanel/cpCase.cpp:626, where
        streamlines.vtu holds its surface streamlines), and
        caseMgr::writeSummary's .CPout (CPanel/CPanelMgr.cpp:89-116) beside it.  Returns the paths
        of surfaceData.vtu and the .CPout."""
        from . import io
        V, alpha, beta, mach = self.flow
        sub = os.path.join(directory, io.case_label(V, mach, alpha, beta))
        os.makedirs(sub, exist_ok=True)
        t = self.geom.tables()
        body = t["body"]
        tris = self.geom._tris[body[:, 17].astype(np.int64)] - 1  # file triangle of each panel, zero-based
        vtu = os.path.join(sub, "surfaceData.vtu")
        io.write_surface_vtu(vtu, self.geom._nodes, tris, self.res["mu"][0], self.res["sigma"][0],
                             self.res["phi"][0], self.res["vel"][0], self.res["cp"][0], body[:, 3:6], body[:, 0:3])
        if self.geom.nw > 0:
            wt = io.wake_tris(self.geom._nodes, self.geom._tris, self.geom._ids)
            wmu, wphi = io.wake_fields(self.res["mu"][0], t["idx4"], t["coef"], t["wake"][:, 0:3], self.vinf())
            io.write_wake_vtu(os.path.join(sub, "wakeData.vtu"), self.geom._nodes, self.geom._tris[wt] - 1, wmu, wphi)
        if self.survey is not None:
            sv = self.survey
            io.write_volume_vtu(os.path.join(sub, "volumeMesh.vtu"), sv["points"], sv["cells"], sv["velocity"],
                                sv["cp"])
        if getattr(self, "lines", None) is not None:
            io.write_streamlines_vtu(os.path.join(sub, "OffBodyStreamlines.vtu"), self.lines)
        for w, span in enumerate(getattr(self, "span", None) or []):  # cpCase.cpp:694
            io.write_spanwise_csv(os.path.join(sub, "spanwiseData_Wake%d.csv" % (w + 1)), span)
        stem = os.path.splitext(os.path.basename(geom_file))[0] if geom_file else "case"
        cpout = os.path.join(directory, stem + ".CPout")
        io.write_cpout(cpout, [dict(V=V, alpha=alpha, beta=beta, mach=mach, CL=self.getCL(), CDi=self.getCD(),
                                    Fbody=self.getBodyForces(), Fwind=self.getWindForces(), CM=self.getMoment(),
                                    stability=self.stab)],
                       geom_file=geom_file, flags=dict(stability_derivatives=self.stab is not None),
                       **self.refs)
        return vtu, cpout


def _streamline_lines(pts, vel, counts, ended):
    lines = [(pts[i, :counts[i]].copy(), vel[i, :counts[i]].copy()) for i in range(len(counts))]
    return lines, ended.astype(bool)


def streamlines_field(fn, speed, starts, x_max, tol=1e-4, max_points=1000):
    """The library's streamline integrator (streamline::streamline / rkf, CPanel/streamline.cpp:20-78)
    through a Python velocity field: fn(points m x 3) -> velocities m x 3, free stream and
    compressibility included.  The first step is 0.1 / speed.  Returns (lines, ended): lines[i] is
    (points, velocities) of every step start of line i; ended[i] is True where the line reached
    x_max (False: max_points cut it short)."""
    L = _lib.load()
    st = np.ascontiguousarray(starts, dtype=np.float64).reshape(-1, 3)
    n = len(st)
    pts = np.zeros((n, max_points, 3))
    vel = np.zeros((n, max_points, 3))
    counts = np.zeros(n, dtype=np.int32)
    ended = np.zeros(n, dtype=np.int32)
    failure = []

    def cb(user, p, m, v):
        try:
            P = np.ctypeslib.as_array(p, shape=(m, 3))
            V = np.ctypeslib.as_array(v, shape=(m, 3))
            V[:] = np.asarray(fn(P.copy()), dtype=np.float64).reshape(m, 3)
            return 0
        except Exception as e:  # reported after the call: an exception cannot cross the C frames
            failure.append(e)
            return 99

    rc = L.cpg_streamlines_field(_lib.VELOCITY_FN(cb), None, float(speed), _p(st), n, float(x_max), float(tol),
                                 int(max_points), _p(pts), _p(vel), _p(counts, _lib.I32), _p(ended, _lib.I32))
    if failure:
        raise failure[0]
    if rc != 0:
        raise CpgError(rc, "cpg_streamlines_field")
    return _streamline_lines(pts, vel, counts, ended)


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr())


def panel_phi_inf(verts, poi, ctx=None):
    """Batched bodyPanel::panelPhiInf on CUDA tensors (m x 9, m x 3) -> (phi_src, phi_dub)."""
    import torch
    ctx = ctx or Context.default()
    verts = verts.contiguous().double()
    poi = poi.contiguous().double()
    m = verts.shape[0]
    src = torch.empty(m, dtype=torch.float64, device=verts.device)
    dub = torch.empty(m, dtype=torch.float64, device=verts.device)
    torch.cuda.synchronize()
    ctx.check(ctx.L.cpg_panel_phi_inf(ctx.h, _dev_ptr(verts), _dev_ptr(poi), m, _dev_ptr(src), _dev_ptr(dub)),
              "panelPhiInf")
    return src, dub


def dub_phi_inf(verts, poi, ctx=None):
    import torch
    ctx = ctx or Context.default()
    verts = verts.contiguous().double()
    poi = poi.contiguous().double()
    m = verts.shape[0]
    dub = torch.empty(m, dtype=torch.float64, device=verts.device)
    torch.cuda.synchronize()
    ctx.check(ctx.L.cpg_dub_phi_inf(ctx.h, _dev_ptr(verts), _dev_ptr(poi), m, _dev_ptr(dub)), "dubPhiInf")
    return dub


def panel_v_inf(verts, poi, ctx=None):
    import torch
    ctx = ctx or Context.default()
    verts = verts.contiguous().double()
    poi = poi.contiguous().double()
    m = verts.shape[0]
    vs = torch.empty((m, 3), dtype=torch.float64, device=verts.device)
    vd = torch.empty((m, 3), dtype=torch.float64, device=verts.device)
    torch.cuda.synchronize()
    ctx.check(ctx.L.cpg_panel_v_inf(ctx.h, _dev_ptr(verts), _dev_ptr(poi), m, _dev_ptr(vs), _dev_ptr(vd)),
              "panelVInf")
    return vs, vd
