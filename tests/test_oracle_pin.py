"""Pin the CPU oracle to the reference's own known answers and fixtures.

* CPanelTests/influenceTests.cpp:598-643 -- phi of a unit triangle at a near and a
  far point (5-6 decimals, printed by the reference's test).
* Connor Cases/4412 -- the full steady case: CL/CDi and surface-integrated forces
  and moments from 4412.CPout (5 decimals), and per-panel doublet, source,
  potential, velocity and Cp from surfaceData-0.vtu (6 significant digits).
"""
import os

import numpy as np
import pytest
from scipy.linalg import lu_factor, lu_solve

from oracle import pyoracle as po

TRI = np.array([1, 0, 0, -1, 1, 0, -1, -1, 0], dtype=np.float64)  # influenceTests.cpp:579-590


def test_near_point_known_answer():
    src, dub = po.tri_phi_inf(TRI, [2, 2, 2])
    assert abs(src - 0.043411) < 1e-5
    assert abs(dub - 0.006645) < 1e-5


def test_far_point_known_answer():
    src, dub = po.tri_phi_inf(TRI, [7, 7, 7])
    assert abs(src - 0.012919) < 1e-5
    assert abs(dub - 0.0005958) < 1e-5


def test_collocation_point_self_term():
    # influenceTests.cpp:664 -- doublet potential -0.5 at the panel's own centroid
    src, dub = po.tri_phi_inf(TRI, [-1.0 / 3, 0, 0])
    assert dub == -0.5


def test_wake_doublet_matches_body_doublet_off_panel():
    for poi in ([2, 2, 2], [0.3, -0.2, 0.5], [7, 7, 7]):
        _, dub = po.tri_phi_inf(TRI, poi)
        assert po.tri_dub_phi_inf(TRI, poi) == pytest.approx(dub, abs=1e-15)


def test_4412_topology_counts(solved4412):
    m, A, B, r = solved4412
    assert m.n == 4824 and m.nw == 172
    bt = m.body_table()
    assert int(bt[:, 11].sum()) == 68  # tip-patch panels, both tips


def test_4412_trefftz_and_forces(solved4412, case4412):
    g = case4412
    m, A, B, r = solved4412
    assert r["converged"]
    assert abs(r["CL"] - float(g["CL"])) <= 5.01e-6
    assert abs(r["CDi"] - float(g["CDi"])) <= 5.01e-6
    CN, CA, CY = g["body_CN_CA_CY"]
    assert abs(r["Fbody"][2] - CN) <= 5.01e-6 and abs(r["Fbody"][0] - CA) <= 5.01e-6
    assert abs(r["Fbody"][1] - CY) <= 5.01e-6
    CLw, CDw, CYw = g["wind_CL_CD_CY"]
    assert abs(r["Fwind"][2] - CLw) <= 5.01e-6 and abs(r["Fwind"][0] - CDw) <= 5.01e-6
    Cm, Cl, Cn = g["Cm_Cl_Cn"]
    assert abs(r["CM"][1] - Cm) <= 5.01e-6 and abs(r["CM"][0] - Cl) <= 5.01e-6 and abs(r["CM"][2] - Cn) <= 5.01e-6


def test_4412_per_panel_fields(solved4412, case4412):
    from scipy.spatial import cKDTree
    g = case4412
    m, A, B, r = solved4412
    c = m.body_table()[:, 0:3]
    d, idx = cKDTree(c).query(g["centroid"].astype(np.float64))
    assert d.max() < 1e-5 and len(np.unique(idx)) == len(idx)
    for name in ("mu", "sigma", "phi", "cp"):
        ref = g[name].astype(np.float64)
        mine = r[name][idx]
        assert np.all(np.abs(mine - ref) <= 6e-6 * np.abs(ref) + 2e-7), name
    vr = g["vel"].astype(np.float64)
    assert np.all(np.abs(r["vel"][idx] - vr) <= 6e-6 * np.abs(vr) + 2e-7)


def test_bicgstab_matches_direct_solve(solved4412):
    m, A, B, r = solved4412
    lu = lu_factor(A)
    rhs = -(B @ r["sigma"])
    x = lu_solve(lu, rhs)
    assert np.abs(x - r["mu"]).max() <= 1e-12 * np.abs(x).max()


def test_doublet_rows_of_closed_body_sum_to_minus_one(case4412):
    g = case4412
    body = g["ids"] < 1000
    m = po.Mesh(g["nodes"], g["tris"][body], g["ids"][body])
    A, _ = m.set_inf_coeff()
    assert np.abs(A.sum(axis=1) + 1).max() < 1e-3


def test_4412AR6_stability_derivatives_match_reference(case4412ar6, solved4412ar6):
    """The reference's 4412AR6 case (Stability_Derivatives 1): CL, CDi, forces, moments and the
    ten stability derivatives of its .CPout, 5 printed decimals each."""
    from conftest import printed_stability
    g = case4412ar6
    r0, st = solved4412ar6
    assert abs(r0["CL"] - float(g["CL"])) <= 5.01e-6 and abs(r0["CDi"] - float(g["CDi"])) <= 5.01e-6
    CN, CA, CY = g["body_CN_CA_CY"]
    assert abs(r0["Fbody"][2] - CN) <= 5.01e-6 and abs(r0["Fbody"][0] - CA) <= 5.01e-6
    Cm, Cl, Cn = g["Cm_Cl_Cn"]
    assert abs(r0["CM"][1] - Cm) <= 5.01e-6 and abs(r0["CM"][0] - Cl) <= 5.01e-6 and abs(r0["CM"][2] - Cn) <= 5.01e-6
    da, db = printed_stability(st)
    assert np.all(np.abs(da - g["d_alpha_CL_CY_Cm_Cl_Cn"]) <= 5.01e-6), da
    assert np.all(np.abs(db - g["d_beta_CL_CY_Cm_Cl_Cn"]) <= 5.01e-6), db



def spanwise_reference():
    """The reference's own spanwiseData_Wake1.csv of the 4412 case (tests/golden/make_golden.py)."""
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "case4412_spanwise.npz"))


def within_printed(ours, ref):
    """|ours - ref| within half a unit of ref's 6th significant digit (1e-12 covers printed zeros)."""
    return np.abs(ours - ref) <= 5e-6 * 1.02 * np.abs(ref) + 1e-12


def test_4412_spanwise_loads_match_reference_csv(solved4412, case4412):
    """cpCase::writeSpanwiseData's columns (CPanel/cpCase.cpp:910-935: 2y/b, Cl / PG, Cdi / PG^2 at
    wake::trefftzPlane's 165 stations) for the reference's 4412 case, within the 6 printed digits
    of its spanwiseData_Wake1.csv."""
    g = case4412
    m, A, B, r = solved4412
    m.post(r["mu"], V=float(g["V"]), alpha=float(g["alpha"]), beta=float(g["beta"]), mach=float(g["mach"]),
           Sref=float(g["Sref"]), bref=float(g["bref"]), cref=float(g["cref"]), cg=tuple(g["cg"]))
    sp, ref = m.spanwise(0), spanwise_reference()
    for k in ("y2b", "cl", "cdi"):
        assert len(sp[k]) == len(ref[k]) == 165
        assert within_printed(sp[k], ref[k]).all(), k
