"""Request loop over include/cpanel_serve.h: steady solves of different meshes admitted
by device-memory footprint and run concurrently, one context (stream) per slot.

    srv = Server(slots=4, budget_gb=60, precision="mixed")
    t = srv.submit(nodes, tris, ids, flows=[(1.0, a, 0.0, 0.1) for a in alphas], Sref=..., ...)
    res = srv.wait(t)          # dict(cp=(k, n), CL=(k,), CDi=(k,), info=...)
"""
import ctypes as C

import numpy as np

from . import _lib, _shutting_down_now
from ._lib import MIXED, PLAIN_FP64, CpgError

_PREC = {"mixed": MIXED, "fp64": PLAIN_FP64, "plain": PLAIN_FP64, MIXED: MIXED, PLAIN_FP64: PLAIN_FP64}


def footprint(n_body, k, precision="mixed"):
    return int(_lib.load().cpg_server_footprint(n_body, k, _PREC[precision]))


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

    def wait(self, ticket):
        n, k = self._n.pop(ticket)
        cp, CL, CDi = np.zeros((k, n)), np.zeros(k), np.zeros(k)
        info = _lib.RequestInfo()
        rc = self.L.cpg_server_wait(self.h, ticket, cp.ctypes.data_as(_lib.D), CL.ctypes.data_as(_lib.D),
                                    CDi.ctypes.data_as(_lib.D), C.byref(info))
        d = {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}
        d["message"] = info.message.decode(errors="replace")
        if rc != 0:
            raise CpgError(rc, "request %d: %s" % (ticket, d["message"]))
        return dict(cp=cp, CL=CL, CDi=CDi, info=d)
