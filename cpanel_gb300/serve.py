"""Request loop over include/cpanel_serve.h: steady solves and unsteady vortex-particle
runs of different meshes admitted by device-memory footprint and run concurrently, one
context (stream) per slot.

    srv = Server(slots=4, budget_gb=60, precision="mixed")
    t = srv.submit(nodes, tris, ids, flows=[(1.0, a, 0.0, 0.1) for a in alphas], Sref=..., ...)
    res = srv.wait(t)          # dict(cp=(k, n), CL=(k,), CDi=(k,), info=...)
    u = srv.submit_vp(nodes, tris, ids, nsteps=100, alpha=8.0, Sref=...)
    res = srv.wait(u)          # dict(CL, CD, steps, n_particles, converged, mu=(n,), info=...)
"""
import ctypes as C

import numpy as np

from . import _lib, _shutting_down_now
from ._lib import MIXED, PLAIN_FP64, CpgError

_PREC = {"mixed": MIXED, "fp64": PLAIN_FP64, "plain": PLAIN_FP64, MIXED: MIXED, PLAIN_FP64: PLAIN_FP64}


def footprint(n_body, k, precision="mixed"):
    return int(_lib.load().cpg_server_footprint(n_body, k, _PREC[precision]))


def footprint_vp(n_body, n_w2, nsteps, precision="mixed"):
    return int(_lib.load().cpg_server_footprint_vp(n_body, n_w2, nsteps, _PREC[precision]))


class Server:
    def __init__(self, slots=4, budget_gb=64.0, precision="mixed", device=0):
        self.L = _lib.load()
        self.precision = _PREC[precision]
        prm = _lib.ServerParams(device, slots, budget_gb * 1e9, self.precision)
        h = C.c_void_p()
        rc = self.L.cpg_server_create(C.byref(prm), C.byref(h))
        if rc != 0:
            raise CpgError(rc, "cpg_server_create")
        self.h = h
        self._n = {}

    def close(self):
        if getattr(self, "h", None):
            self.L.cpg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        if not _shutting_down_now():
            self.close()

    def submit(self, nodes, tris, ids, flows, Sref=1.0, bref=1.0, cref=1.0, cg=(0.0, 0.0, 0.0)):
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int64)
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        fl = (_lib.Flow * len(flows))(*[_lib.Flow(*f) for f in flows])
        refs = _lib.Refs(Sref, bref, cref, (C.c_double * 3)(*cg))
        t = C.c_int64(0)
        rc = self.L.cpg_server_submit(self.h, nodes.ctypes.data_as(_lib.D), len(nodes), tris.ctypes.data_as(_lib.I64),
                                      ids.ctypes.data_as(_lib.I32), len(ids), fl, len(flows), C.byref(refs),
                                      C.byref(t))
        if rc != 0:
            raise CpgError(rc, "cpg_server_submit")
        self._n[t.value] = (int(np.count_nonzero(ids <= 1000)), len(flows))
        return t.value

    def submit_vp(self, nodes, tris, ids, nsteps, V=1.0, alpha=5.0, beta=0.0, dt=0.0, cref=1.0, accelerate=True,
                  Sref=1.0, mach=0.0, precision="mixed"):
        """Queue cpCaseVP::run on a body-only mesh for nsteps steps (or until converged)."""
        nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int64)
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        prm = _lib.VPParams(V, alpha, beta, dt, cref, 1 if accelerate else 0, Sref, mach, _PREC[precision])
        t = C.c_int64(0)
        rc = self.L.cpg_server_submit_vp(self.h, nodes.ctypes.data_as(_lib.D), len(nodes),
                                         tris.ctypes.data_as(_lib.I64), ids.ctypes.data_as(_lib.I32), len(ids),
                                         C.byref(prm), nsteps, C.byref(t))
        if rc != 0:
            raise CpgError(rc, "cpg_server_submit_vp")
        self._n[t.value] = ("vp", len(ids))
        return t.value

    def _wait_vp(self, ticket, n_tris):
        res, info = _lib.VPResult(), _lib.RequestInfo()
        mu = np.zeros(n_tris)  # n_body <= n_tris; trimmed below
        rc = self.L.cpg_server_wait_vp(self.h, ticket, C.byref(res), mu.ctypes.data_as(_lib.D), C.byref(info))
        d = {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}
        d["message"] = info.message.decode(errors="replace")
        if rc != 0:
            raise CpgError(rc, "request %d: %s" % (ticket, d["message"]))
        out = {f: getattr(res, f) for f, _ in _lib.VPResult._fields_}
        out["converged"] = bool(out["converged"])
        out["mu"] = mu[:info.n_body]
        out["info"] = d
        return out

    def wait(self, ticket):
        n, k = self._n.pop(ticket)
        if n == "vp":
            return self._wait_vp(ticket, k)
        cp, CL, CDi = np.zeros((k, n)), np.zeros(k), np.zeros(k)
        info = _lib.RequestInfo()
        rc = self.L.cpg_server_wait(self.h, ticket, cp.ctypes.data_as(_lib.D), CL.ctypes.data_as(_lib.D),
                                    CDi.ctypes.data_as(_lib.D), C.byref(info))
        d = {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}
        d["message"] = info.message.decode(errors="replace")
        if rc != 0:
            raise CpgError(rc, "request %d: %s" % (ticket, d["message"]))
        return dict(cp=cp, CL=CL, CDi=CDi, info=d)
