"""CPanel's result files from this library's results (include/cpanel_io.h): the .CPout
summary (caseMgr::writeSummary, CPanel/CPanelMgr.cpp:89-180), surfaceData.vtu
(cpCase::writeBodyData, CPanel/cpCase.cpp:711-763), wakeData.vtu (cpCase::writeWakeData) and
volumeMesh.vtu (cpCase::writeVolMeshData).  Host only: no device is needed.
"""
import ctypes as C
import os
import re

import numpy as np

from . import _lib
from ._lib import CpgError


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_lib.D)


def _unique(vals):
    out = []
    for v in vals:
        if v not in out:
            out.append(v)
    return np.array(out, dtype=np.float64)


def write_cpout(path, cases, geom_file="", Sref=1.0, bref=1.0, cref=1.0, cg=(0.0, 0.0, 0.0), flags=None):
    """cases: dicts with V, alpha, beta, mach, CL, CDi, Fbody (x, y, z), Fwind (x, y, z) and CM
    (roll, pitch, yaw), as solve_cases / CpCase return them, and optionally "stability" (a dict
    of dF_dAlpha, dF_dBeta, dM_dAlpha, dM_dBeta as CpCase.stabilityDerivatives returns it, printed
    as the reference's stability block).  flags: the input flags to echo
    (subsonic_hom, surface_streamlines, stability_derivatives, write_inf_coeff,
    vortex_particles, accelerate_code, unsteady); all OFF by default."""
    L = _lib.load()
    keep = []
    lists = {}
    for key in ("V", "alpha", "beta", "mach"):
        arr, ptr = _d(_unique([float(c[key]) for c in cases]))
        keep.append(arr)
        lists[key] = (ptr, len(arr))
    f = dict(flags or {})
    inp = _lib.CpoutInputs(geom_file.encode(), Sref, bref, cref, (C.c_double * 3)(*cg),
                           lists["V"][0], lists["V"][1], lists["alpha"][0], lists["alpha"][1],
                           lists["beta"][0], lists["beta"][1], lists["mach"][0], lists["mach"][1],
                           *[int(bool(f.get(k, False))) for k in ("subsonic_hom", "surface_streamlines",
                                                                  "stability_derivatives", "write_inf_coeff",
                                                                  "vortex_particles", "accelerate_code",
                                                                  "unsteady")])
    arr = (_lib.CpoutCase * max(1, len(cases)))()
    for i, c in enumerate(cases):
        st = c.get("stability")
        stab = _lib.Stability(*[(C.c_double * 3)(*st[k]) for k in ("dF_dAlpha", "dF_dBeta", "dM_dAlpha",
                                                                     "dM_dBeta")]) if st else _lib.Stability()
        arr[i] = _lib.CpoutCase(_lib.Flow(c["V"], c["alpha"], c["beta"], c["mach"]), c["CL"], c["CDi"],
                                (C.c_double * 3)(*c["Fbody"]), (C.c_double * 3)(*c["Fwind"]),
                                (C.c_double * 3)(*c["CM"]), 1 if st else 0, stab)
    rc = L.cpg_write_cpout(os.fsencode(path), C.byref(inp), arr, len(cases))
    if rc != 0:
        raise CpgError(rc, "cpg_write_cpout(%s)" % path)


def write_surface_vtu(path, nodes, tris, mu, sigma, phi, vel, cp, bez, centers):
    """nodes (n_nodes x 3); tris (n x 3) zero-based node indices of the body panels in matrix
    order; per panel mu, sigma, phi, cp (n) and vel, bez, centers (n x 3)."""
    L = _lib.load()
    t = np.ascontiguousarray(tris, dtype=np.int64)
    arrays = [_d(a) for a in (nodes, mu, sigma, phi, vel, cp, bez, centers)]
    (nd, ndp), (m, mp), (s, sp), (p, pp), (v, vp), (c, cpp), (b, bp), (ce, cep) = arrays
    rc = L.cpg_write_surface_vtu(os.fsencode(path), ndp, len(nd), t.ctypes.data_as(_lib.I64), len(t), mp, sp, pp, vp,
                                 cpp, bp, cep)
    if rc != 0:
        raise CpgError(rc, "cpg_write_surface_vtu(%s)" % path)


def wake_tris(nodes, tris, ids):
    """Zero-based .tri triangle of each wake panel in wPanels order (host topology)."""
    L = _lib.load()
    n_ = np.ascontiguousarray(nodes, dtype=np.float64)
    t_ = np.ascontiguousarray(tris, dtype=np.int64)
    i_ = np.ascontiguousarray(ids, dtype=np.int32)
    out = np.zeros(int(np.count_nonzero(i_ > 1000)), dtype=np.int64)
    rc = L.cpg_topology_wake_tris(n_.ctypes.data_as(_lib.D), len(n_), t_.ctypes.data_as(_lib.I64),
                                  i_.ctypes.data_as(_lib.I32), len(i_), out.ctypes.data_as(_lib.I64))
    if rc != 0:
        raise CpgError(rc, "cpg_topology_wake_tris")
    return out


def wake_fields(mu, idx4, coef, wake_centers, vinf):
    """wakePanel::setMu (CPanel/wakePanel.cpp:94-100) and panel::setPotential (CPanel/panel.cpp:106-111)
    for every wake panel: mu_w = (1 - t) mu_0 + (t - 1) mu_1 + t mu_2 - t mu_3 over the four
    interpolation panels (idx4, t = coef), phi_w = V_inf . c_w - mu_w."""
    mu = np.asarray(mu, dtype=np.float64)
    ix = np.asarray(idx4)
    t = np.asarray(coef, dtype=np.float64)
    mw = (1 - t) * mu[ix[:, 0]] + (t - 1) * mu[ix[:, 1]] + t * mu[ix[:, 2]] - t * mu[ix[:, 3]]
    phi = np.asarray(wake_centers, dtype=np.float64) @ np.asarray(vinf, dtype=np.float64) - mw
    return mw, phi


def write_wake_vtu(path, nodes, tris, mu, phi):
    """wakeData.vtu (cpCase::writeWakeData): tris n_wake x 3 zero-based node indices in wPanels order."""
    L = _lib.load()
    t = np.ascontiguousarray(tris, dtype=np.int64)
    (nd, ndp), (m, mp), (p, pp) = _d(nodes), _d(mu), _d(phi)
    rc = L.cpg_write_wake_vtu(os.fsencode(path), ndp, len(nd), t.ctypes.data_as(_lib.I64), len(t), mp, pp)
    if rc != 0:
        raise CpgError(rc, "cpg_write_wake_vtu(%s)" % path)


def volume_grid(bounds, res):
    """cpCase::createVolMesh (CPanel/cpCase.cpp:1024-1097): the points of an (nX, nY, nZ)-cell grid
    over bounds (x0, xf, y0, yf, z0, zf), x fastest; the cells as 8 point indices (VTK voxel
    order), looping x, then y, then z innermost as the reference does; the cell centres.
    Returns (points, cells, centers)."""
    x0, xf, y0, yf, z0, zf = [float(b) for b in bounds]
    nX, nY, nZ = [int(r) for r in res]
    hx, hy, hz = (xf - x0) / nX, (yf - y0) / nY, (zf - z0) / nZ
    nXp, nYp, nZp = nX + 1, nY + 1, nZ + 1
    k, j, i = np.meshgrid(np.arange(nZp), np.arange(nYp), np.arange(nXp), indexing="ij")
    pts = np.stack([x0 + hx * i.ravel(), y0 + hy * j.ravel(), z0 + hz * k.ravel()], axis=1)
    I, J, K = np.meshgrid(np.arange(nX), np.arange(nY), np.arange(nZ), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    base = K * (nXp * nYp) + J * nXp + I
    cells = np.stack([base, base + 1, base + nXp, base + nXp + 1, base + nXp * nYp, base + nXp * nYp + 1,
                      base + nXp * nYp + nXp, base + nXp * nYp + nXp + 1], axis=1).astype(np.int64)
    centers = pts[cells].mean(axis=1)
    return pts, cells, centers


def write_volume_vtu(path, points, cells, vel, cp):
    """volumeMesh.vtu (cpCase::writeVolMeshData): cell data Velocity and Cp on VTK voxels."""
    L = _lib.load()
    c = np.ascontiguousarray(cells, dtype=np.int64)
    (p, pp), (v, vp), (q, qp) = _d(points), _d(vel), _d(cp)
    rc = L.cpg_write_volume_vtu(os.fsencode(path), pp, len(p), c.ctypes.data_as(_lib.I64), len(c), vp, qp)
    if rc != 0:
        raise CpgError(rc, "cpg_write_volume_vtu(%s)" % path)


def write_streamlines_vtu(path, lines):
    """A streamline file in cpCase::writeBodyStreamlines's layout (CPanel/cpCase.cpp:937-977; CpCase.writeFiles
    writes the off-body lines as OffBodyStreamlines.vtu, the reference's name for them): lines as
    CpCase.streamlines or streamlines_field return them, [(points k x 3, velocities k x 3), ...]; one
    piece per line with point data Velocity and line cells."""
    L = _lib.load()
    n = len(lines)
    width = max([len(p) for p, _ in lines] + [1])
    pts = np.zeros((max(n, 1), width, 3))
    vel = np.zeros((max(n, 1), width, 3))
    counts = np.zeros(max(n, 1), dtype=np.int32)
    for i, (p, v) in enumerate(lines):
        counts[i] = len(p)
        pts[i, :len(p)] = p
        vel[i, :len(p)] = v
    rc = L.cpg_write_streamlines_vtu(os.fsencode(path), pts.ctypes.data_as(_lib.D), vel.ctypes.data_as(_lib.D),
                                     counts.ctypes.data_as(_lib.I32), n, width)
    if rc != 0:
        raise CpgError(rc, "cpg_write_streamlines_vtu(%s)" % path)


def write_spanwise_csv(path, span):
    """spanwiseData_Wake<i>.csv in cpCase::writeSpanwiseData's layout (CPanel/cpCase.cpp:910-935): span as
    spanwise_loads returns it, {"y2b", "cl", "cdi"}."""
    L = _lib.load()
    cols = [np.ascontiguousarray(span[k], dtype=np.float64) for k in ("y2b", "cl", "cdi")]
    rc = L.cpg_write_spanwise_csv(os.fsencode(path), *[c.ctypes.data_as(_lib.D) for c in cols], len(cols[0]))
    if rc != 0:
        raise CpgError(rc, "cpg_write_spanwise_csv(%s)" % path)


def read_vtu_pieces(path):
    """Every piece of an ASCII .vtu file as {array name: array} (points under "Position")."""
    txt = open(path).read()
    out = []
    for piece in re.findall(r"<Piece .*?</Piece>", txt, flags=re.S):
        d = {}
        for m in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)"(?: NumberOfComponents="(\d+)")? Format="ascii">'
                             r'(.*?)</DataArray>', piece, flags=re.S):
            kind, name, comps, body = m.group(1), m.group(2), m.group(3), m.group(4)
            vals = np.array(body.split(), dtype=np.float64 if kind == "Float64" else np.int64)
            ncomp = int(comps) if comps else 1
            d[name] = vals.reshape(-1, ncomp) if ncomp > 1 else vals
        out.append(d)
    return out


def read_vtu_cells(path):
    """The cell data arrays, points and connectivity of an ASCII .vtu file (as written by CPanel
    or by write_surface_vtu): {name: array}."""
    txt = open(path).read()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)"(?: NumberOfComponents="(\d+)")? Format="ascii">'
                         r'(.*?)</DataArray>', txt, flags=re.S):
        kind, name, comps, body = m.group(1), m.group(2), m.group(3), m.group(4)
        vals = np.array(body.split(), dtype=np.float64 if kind == "Float64" else np.int64)
        ncomp = int(comps) if comps else 1
        out[name] = vals.reshape(-1, ncomp) if ncomp > 1 else vals
    return out


def case_label(V, mach, alpha, beta):
    """The case directory name cpCase::writeFiles uses (CPanel/cpCase.cpp:669-670)."""
    def g(x):
        return ("%.6g" % x)
    return "V%s_Mach%s_alpha%s_beta%s" % (g(V), g(mach), g(alpha), g(beta))
