"""Many meshes at once (include/cpanel_batch.h): the grouped, persistent mixed-precision
assembly with its work-shape autotuner, and the batch solve of uneven meshes.

The reference solves one mesh per process (geometry::readTri -> setInfCoeff,
CPanel/geometry.cpp:607-621; CPanelMgr::run -> cpCase::run per flow condition,
CPanel/CPanelMgr.cpp:90-167).  Here m meshes share one assembly launch (bit-identical to
each mesh's own); their factorizations and refined solves run either side by side on
worker streams (bit-identical to each mesh alone) or in lockstep, one launch per block
step for all meshes (the same factors up to FP32 rounding, so the refined solutions agree
within the refinement tolerance).
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import CpgError
from . import Context, _p

TUNE = {"off": _lib.TUNE_OFF, "auto": _lib.TUNE_AUTO, "force": _lib.TUNE_FORCE}


def default_shape():
    L = _lib.load()
    s = _lib.GroupShape()
    L.cpg_group_default_shape(C.byref(s))
    return dict(chunks_per_item=s.chunks_per_item, near_band=s.near_band, blocks_per_sm=s.blocks_per_sm)


def _shape(d):
    if d is None:
        return None
    base = default_shape()
    base.update(d)
    return _lib.GroupShape(base["chunks_per_item"], base["near_band"], base["blocks_per_sm"])


def group_schedule(n_body, shape=None):
    """Host-only work queue of the grouped assembly for meshes of n_body panels:
    (items[count, 4] = mesh, row block, first source chunk, chunk count; chunk lengths)."""
    L = _lib.load()
    n = np.ascontiguousarray(n_body, dtype=np.int64)
    cnt = C.c_int64()
    sh = _shape(shape)
    shp = C.byref(sh) if sh is not None else None
    ch = np.zeros(len(n), dtype=np.int64)
    rc = L.cpg_group_schedule(_p(n, _lib.I64), len(n), shp, None, 0, C.byref(cnt), _p(ch, _lib.I64))
    if rc != 0:
        raise CpgError(rc, "cpg_group_schedule")
    items = np.zeros((cnt.value, 4), dtype=np.int32)
    rc = L.cpg_group_schedule(_p(n, _lib.I64), len(n), shp, _p(items, _lib.I32), cnt.value, C.byref(cnt), None)
    if rc != 0:
        raise CpgError(rc, "cpg_group_schedule")
    return items, ch


def _report(r):
    return dict(shape=dict(chunks_per_item=r.shape.chunks_per_item, near_band=r.shape.near_band,
                           blocks_per_sm=r.shape.blocks_per_sm),
                tuned=r.tuned, candidates=r.candidates, items=r.items, pairs=r.pairs, near_pairs=r.near_pairs,
                ms=r.ms)


def set_inf_coeff_grouped(geoms, tune="off", shape=None):
    """geometry::setInfCoeff (mixed precision) for every geometry of ``geoms`` in one grouped,
    persistent launch.  tune: "off" (``shape`` or the default), "auto" (cached per size
    class, else timed now) or "force".  Returns the launch report."""
    if not geoms:
        raise ValueError("no geometries")
    ctx = geoms[0].ctx
    arr = (C.c_void_p * len(geoms))(*[g.h.value for g in geoms])
    rep = _lib.GroupReport()
    sh = _shape(shape)
    ctx.check(ctx.L.cpg_set_inf_coeff_grouped(arr, len(geoms), TUNE[tune], C.byref(sh) if sh is not None else None,
                                              C.byref(rep)), "cpg_set_inf_coeff_grouped")
    return _report(rep)


def lu_factor_grouped(geoms):
    """The mixed path's FP32 LU factorizations of every geometry at once (lockstep block
    steps); the geometries must hold their mixed matrices.  Returns the device time (ms)."""
    if not geoms:
        raise ValueError("no geometries")
    ctx = geoms[0].ctx
    arr = (C.c_void_p * len(geoms))(*[g.h.value for g in geoms])
    ms = C.c_double()
    ctx.check(ctx.L.cpg_lu_factor_grouped(arr, len(geoms), C.byref(ms)), "cpg_lu_factor_grouped")
    return ms.value


def batch_solve(meshes, workers=8, tune="auto", budget_gb=0.0, want=("cp", "CL", "CDi"), lockstep=False,
                ctx=None):
    """Steady mixed-precision solves of many meshes.  lockstep: False = each mesh's LU,
    refined solves and post on its worker (bit-identical to solve_cases); True = a wave's
    factorizations and refined solves together, block step by block step.

    meshes: list of dicts with nodes, tris, ids, flows [(V, alpha, beta, mach), ...] and
    optional Sref, bref, cref, cg.  Returns (results, stats): one dict per mesh with the
    arrays named in ``want`` (cp, mu: k x n_body; CL, CDi: k), status and n_body.  A mesh
    the path rejects only sets its own status; CpgError is raised when no mesh was solved."""
    ctx = ctx or Context.default()
    L = ctx.L
    m = len(meshes)
    keep = []
    arr = (_lib.BatchMesh * m)()
    outs = []
    for i, ms in enumerate(meshes):
        nodes = np.ascontiguousarray(ms["nodes"], dtype=np.float64)
        tris = np.ascontiguousarray(ms["tris"], dtype=np.int64)
        ids = np.ascontiguousarray(ms["ids"], dtype=np.int32)
        flows = [tuple(f) for f in ms["flows"]]
        k = len(flows)
        fl = (_lib.Flow * k)(*[_lib.Flow(*f) for f in flows])
        n_body = int(np.count_nonzero(ids <= 1000))  # upper bound for the output buffers
        o = {}
        if "cp" in want:
            o["cp"] = np.zeros((k, n_body))
        if "mu" in want:
            o["mu"] = np.zeros((k, n_body))
        for name in ("CL", "CDi"):
            if name in want:
                o[name] = np.zeros(k)
        keep += [nodes, tris, ids, fl]
        b = arr[i]
        b.nodes, b.n_nodes = _p(nodes), len(nodes)
        b.tris, b.ids, b.n_tris = _p(tris, _lib.I64), _p(ids, _lib.I32), len(ids)
        b.flows, b.k = fl, k
        b.refs = _lib.Refs(ms.get("Sref", 1.0), ms.get("bref", 1.0), ms.get("cref", 1.0),
                           (C.c_double * 3)(*ms.get("cg", (0.0, 0.0, 0.0))))
        for name in ("cp", "mu", "CL", "CDi"):
            setattr(b, name, _p(o[name]) if name in o else None)
        outs.append(o)
    prm = _lib.BatchParams(workers, TUNE[tune], budget_gb * 1e9, 1 if lockstep else 0)
    st = _lib.BatchStats()
    rc = L.cpg_batch_solve(ctx.h, arr, m, C.byref(prm), C.byref(st))
    res = []
    for i, o in enumerate(outs):
        o["status"] = arr[i].status
        o["n_body"] = arr[i].n_body
        for name in ("cp", "mu"):
            if name in o:  # written packed as k x n_body
                k = o[name].shape[0]
                o[name] = o[name].ravel()[:k * arr[i].n_body].reshape(k, arr[i].n_body)
        res.append(o)
    stats = dict(ms_total=st.ms_total, ms_topology=st.ms_topology, ms_assembly=st.ms_assembly,
                 ms_factor=st.ms_factor, ms_solve=st.ms_solve,
                 waves=st.waves, solves=st.solves, failed=st.failed, group=_report(st.group))
    if rc not in (0, 5) and st.failed >= m:  # nothing solved; single failures are in the statuses
        ctx.check(rc, "cpg_batch_solve")
    return res, stats
