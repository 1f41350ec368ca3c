"""The identity the mixed assembly uses between 3 and 5 panel lengths (CPU, FP64).

For those pairs the mixed path evaluates bodyPanel::panelPhiInf (CPanel/bodyPanel.cpp:132-190)
as: the three vortexPhi edge angles = minus the solid angle 2 atan(N / D) (Van Oosterom and
Strackee) with N = -2 area PN, and each srcSidePhi log term log((A+B+S)/(A+B-S)) = 2 atanh(S/(A+B)).
Here the identity itself is checked in FP64 against the oracle's restatement of the reference
on a jittered wing, for the pairs the kernel accepts (|N / D| >= 1e-6, inside the series' ranges).
"""
import numpy as np

from conftest import small_wing
from oracle import pyoracle as po


def _band(v, poi):
    c = v.mean(axis=0)
    e1, e2 = v[1] - v[0], v[2] - v[0]
    nrm = np.cross(e1, e2)
    area = 0.5 * np.linalg.norm(nrm)
    n = nrm / (2 * area)
    d = poi - c
    PN = d @ n
    a = [poi - v[k] for k in range(3)]
    A = [np.linalg.norm(x) for x in a]
    D = A[0] * A[1] * A[2] + (a[0] @ a[1]) * A[2] + (a[0] @ a[2]) * A[1] + (a[1] @ a[2]) * A[0]
    x = -2 * area * PN / D
    dub = -2 * np.arctan(x)
    src = 0.0
    ts = []
    for k in range(3):
        s = v[(k + 1) % 3] - v[k]
        S = np.linalg.norm(s)
        t = S / (A[k] + A[(k + 1) % 3])
        ts.append(t)
        src += (np.cross(n, s) @ a[k]) * 2 * np.arctanh(t) / S
    src -= PN * dub
    return src / (4 * np.pi), dub / (4 * np.pi), abs(x), max(ts), D


def test_band_identity_matches_the_reference_formulas():
    nodes, tris, ids, info, spec = small_wing(n_chord=16, n_span=9)
    m = po.Mesh(nodes, tris, ids)
    bv = m.body_verts().reshape(-1, 3, 3)
    c = bv.mean(axis=1)
    L = np.max([np.linalg.norm(bv[:, (k + 1) % 3] - bv[:, k], axis=1) for k in range(3)], axis=0)
    rng = np.random.default_rng(3)
    checked = 0
    worst_src = worst_dub = 0.0
    for _ in range(6000):
        i, j = rng.integers(len(c), size=2)
        r = np.linalg.norm(c[i] - c[j]) / L[j]
        if not 3 < r <= 5:
            continue
        src, dub, ax, tmax, D = _band(bv[j], c[i])
        assert D > 0 and ax < 0.02 and tmax < 0.25  # the kernel's series ranges hold in the band
        if ax < 1e-6:
            continue  # nearly coplanar: the kernel takes the FP64 formulas
        s_ref, d_ref = po.tri_phi_inf(bv[j].reshape(9), c[i])
        worst_src = max(worst_src, abs(src - s_ref))
        worst_dub = max(worst_dub, abs(dub - d_ref))
        checked += 1
    assert checked > 500
    assert worst_src < 1e-15 and worst_dub < 1e-14


def test_solid_angle_form_of_the_near_field():
    """Within 3 panel lengths the mixed path keeps FP64 but takes the three vortexPhi edge
    angles as one solid angle, 2 atan2(a0.(a1 x a2), D), from one panel length out (closer
    in the edge sum is kept).  Checked in FP64 against the oracle's edge sum."""
    nodes, tris, ids, info, spec = small_wing(n_chord=16, n_span=9)
    m = po.Mesh(nodes, tris, ids)
    bv = m.body_verts().reshape(-1, 3, 3)
    c = bv.mean(axis=1)
    L = np.max([np.linalg.norm(bv[:, (k + 1) % 3] - bv[:, k], axis=1) for k in range(3)], axis=0)
    rng = np.random.default_rng(4)
    worst, checked = 0.0, 0
    for i in rng.integers(len(c), size=120):
        r = np.linalg.norm(c - c[i], axis=1) / L
        for j in np.where((r >= 1) & (r <= 3))[0][:40]:
            a = [c[i] - bv[j][k] for k in range(3)]
            A = [np.linalg.norm(x) for x in a]
            D = A[0] * A[1] * A[2] + (a[0] @ a[1]) * A[2] + (a[0] @ a[2]) * A[1] + (a[1] @ a[2]) * A[0]
            dub = 2 * np.arctan2(a[0] @ np.cross(a[1], a[2]), D) / (4 * np.pi)
            _, d_ref = po.tri_phi_inf(bv[j].reshape(9), c[i])
            worst = max(worst, abs(dub - d_ref))
            checked += 1
    assert checked > 1000
    assert worst < 1e-12
