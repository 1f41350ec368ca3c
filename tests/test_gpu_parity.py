"""GPU parity: the sm_103a library against the CPU oracle, through the C ABI.

Tolerances (from the path's specification):
  * influence coefficients: 1e-12 relative (elementwise, relative to the column's
    largest entry so that exact cancellations near zero are judged fairly);
  * plain FP64 path: mu, Cp, CL, CDi within 1e-10 of the oracle;
  * mixed path: Cp max-abs error <= 1e-5 and CL relative error <= 1e-6 against the
    plain FP64 GPU path.
"""
import os

import numpy as np
import pytest

from conftest import small_wing

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg(built):
    import cpanel_gb300
    return cpanel_gb300


def _matrix_rel_err(X, Xo):
    scale = np.maximum(np.abs(Xo).max(axis=0, keepdims=True), 1e-300)
    return (np.abs(X - Xo) / scale).max()


@pytest.fixture(scope="module")
def small(cg):
    from oracle import pyoracle as po
    nodes, tris, ids, info, spec = small_wing(n_chord=16, n_span=9)
    g = cg.Geometry(nodes, tris, ids)
    m = po.Mesh(nodes, tris, ids)
    Ao, Bo = m.set_inf_coeff()
    refs = dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0.0, 0.0))
    return g, m, Ao, Bo, refs


def test_assembly_fp64_matches_oracle(small):
    g, m, Ao, Bo, refs = small
    g.setInfCoeff("fp64")
    A, B = g.getA(), g.getB()
    assert _matrix_rel_err(A, Ao) < 1e-12
    assert _matrix_rel_err(B, Bo) < 1e-12
    te_cols = np.unique(m.wake_table()[1])
    off_te = np.setdiff1d(np.arange(m.n), te_cols)
    assert np.all(np.diag(A)[off_te] == -0.5)  # self term (trailing-edge columns also carry wake terms)


def test_assembly_fp64_4412_matches_oracle(cg, case4412):
    from oracle import pyoracle as po
    gg = case4412
    g = cg.Geometry(gg["nodes"], gg["tris"].astype(np.int64), gg["ids"])
    g.setInfCoeff("fp64")
    m = po.Mesh(gg["nodes"], gg["tris"], gg["ids"])
    Ao, Bo = m.set_inf_coeff()
    assert _matrix_rel_err(g.getA(), Ao) < 1e-12
    assert _matrix_rel_err(g.getB(), Bo) < 1e-12


def test_assembly_mixed_is_close(small):
    """The mixed matrix (hi + lo): near field within 3 longSide in FP64 (the solid angle in
    one atan2), the exact formulas between 3 and 5 longSide and the far field in
    double-float."""
    g, m, Ao, Bo, refs = small
    g.setInfCoeff("mixed")
    A = g.getA()
    assert _matrix_rel_err(A, Ao) < 1e-11
    assert np.abs(A - Ao).max() < 1e-11


def test_influence_operators_match_oracle(cg):
    import torch
    from oracle import pyoracle as po
    rng = np.random.default_rng(7)
    m = 257
    verts = rng.uniform(-1, 1, (m, 9))
    scale = rng.uniform(0.2, 3.0, (m, 1))
    poi = rng.uniform(-1, 1, (m, 3)) * scale * 4
    poi[:16] = verts[:16].reshape(-1, 3, 3).mean(axis=1)  # self points
    v_t = torch.tensor(verts, device="cuda")
    p_t = torch.tensor(poi, device="cuda")
    s, d = cg.panel_phi_inf(v_t, p_t)
    dw = cg.dub_phi_inf(v_t, p_t)
    vs, vd = cg.panel_v_inf(v_t, p_t)
    s, d, dw, vs, vd = (x.cpu().numpy() for x in (s, d, dw, vs, vd))
    for i in range(m):
        so, do = po.tri_phi_inf(verts[i], poi[i])
        assert s[i] == pytest.approx(so, rel=1e-12, abs=1e-15)
        assert d[i] == pytest.approx(do, rel=1e-12, abs=1e-15)
        assert dw[i] == pytest.approx(po.tri_dub_phi_inf(verts[i], poi[i]), rel=1e-12, abs=1e-15)
        vso, vdo = po.tri_v_inf(verts[i], poi[i])
        assert np.allclose(vs[i], vso, rtol=1e-11, atol=1e-14)
        assert np.allclose(vd[i], vdo, rtol=1e-11, atol=1e-14)


def test_plain_solve_matches_oracle(cg, small):
    g, m, Ao, Bo, refs = small
    flows = [(1.0, 5.0, 0.0, 0.1), (1.0, -2.0, 0.0, 0.1), (1.3, 8.0, 1.0, 0.2)]
    r = cg.solve_cases(g, flows, precision="fp64", **refs)
    assert r["status"] == 0
    for c, f in enumerate(flows):
        o = m.case(Ao, Bo, V=f[0], alpha=f[1], beta=f[2], mach=f[3], **refs)
        assert np.abs(r["sigma"][c] - o["sigma"]).max() < 1e-14
        assert np.abs(r["mu"][c] - o["mu"]).max() < 1e-10
        assert np.abs(r["phi"][c] - o["phi"]).max() < 1e-10
        assert np.abs(r["vel"][c] - o["vel"]).max() < 1e-10
        assert np.abs(r["cp"][c] - o["cp"]).max() < 1e-10
        assert abs(r["CL"][c] - o["CL"]) < 1e-10 and abs(r["CDi"][c] - o["CDi"]) < 1e-10
        assert np.abs(r["Fbody"][c] - o["Fbody"]).max() < 1e-10
        assert np.abs(r["Fwind"][c] - o["Fwind"]).max() < 1e-10
        assert np.abs(r["CM"][c] - o["CM"]).max() < 1e-10


def test_4412_reference_case_on_gpu(cg, case4412):
    gg = case4412
    g = cg.Geometry(gg["nodes"], gg["tris"].astype(np.int64), gg["ids"])
    case = cg.CpCase(g, float(gg["V"]), float(gg["alpha"]), float(gg["beta"]), float(gg["mach"]),
                     Sref=float(gg["Sref"]), bref=float(gg["bref"]), cref=float(gg["cref"]), cg=tuple(gg["cg"]))
    assert case.run()
    assert abs(case.getCL() - float(gg["CL"])) <= 5.01e-6
    assert abs(case.getCD() - float(gg["CDi"])) <= 5.01e-6
    CN, CA, CY = gg["body_CN_CA_CY"]
    assert abs(case.getBodyForces()[2] - CN) <= 5.01e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_4412_spanwise_loads_on_gpu(cg, case4412, precision, tmp_path):
    """cpg_spanwise_loads on the reference's 4412 case: 2y/b, Cl and Cdi at the 165 Trefftz stations
    within the 6 printed digits of the reference's spanwiseData_Wake1.csv (the mixed form with its
    own error added, 1e-7 of each column's largest value), and CpCase.writeFiles' CSV from the plain
    path equal to the reference's file line for line."""
    from test_oracle_pin import spanwise_reference
    gg = case4412
    g = cg.Geometry(gg["nodes"], gg["tris"].astype(np.int64), gg["ids"])
    case = cg.CpCase(g, float(gg["V"]), float(gg["alpha"]), float(gg["beta"]), float(gg["mach"]),
                     Sref=float(gg["Sref"]), bref=float(gg["bref"]), cref=float(gg["cref"]), cg=tuple(gg["cg"]),
                     precision=precision)
    assert case.run()
    ref = spanwise_reference()
    assert len(case.span) == 1
    slack = 1e-7 if precision == "mixed" else 0.0
    for k in ("y2b", "cl", "cdi"):
        ours = case.span[0][k]
        assert len(ours) == 165
        tol = 5e-6 * 1.02 * np.abs(ref[k]) + 1e-12 + slack * np.abs(ref[k]).max()
        assert (np.abs(ours - ref[k]) <= tol).all(), k
    if precision == "fp64":
        case.writeFiles(str(tmp_path), geom_file="4412.tri")
        sub = [d for d in os.listdir(tmp_path) if os.path.isdir(os.path.join(tmp_path, d))][0]
        with open(os.path.join(tmp_path, sub, "spanwiseData_Wake1.csv")) as f:
            assert f.read().splitlines() == list(ref["lines"])


def test_4412_reference_case_mixed_on_gpu(cg, case4412):
    """The reference's own 4412 case (4,824 body panels) through the mixed path: the printed
    CL and CDi (5 decimals) as the plain path reproduces them."""
    gg = case4412
    g = cg.Geometry(gg["nodes"], gg["tris"].astype(np.int64), gg["ids"])
    case = cg.CpCase(g, float(gg["V"]), float(gg["alpha"]), float(gg["beta"]), float(gg["mach"]),
                     Sref=float(gg["Sref"]), bref=float(gg["bref"]), cref=float(gg["cref"]), cg=tuple(gg["cg"]),
                     precision="mixed")
    assert case.run()
    assert abs(case.getCL() - float(gg["CL"])) <= 5.01e-6
    assert abs(case.getCD() - float(gg["CDi"])) <= 5.01e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_4412AR6_stability_derivatives_on_gpu(cg, case4412ar6, precision):
    """cpCase::stabilityDerivatives on the GPU for the reference's 4412AR6 case: the ten printed
    derivatives of its .CPout (5 decimals), the base and both sub-cases solved together."""
    from conftest import printed_stability
    g = case4412ar6
    geo = cg.Geometry(g["nodes"], g["tris"].astype(np.int64), g["ids"])
    case = cg.CpCase(geo, 1.0, 5.0, 0.0, 0.1, Sref=6.0, bref=6.0, cref=1.0, cg=(0.25, 0.0, 0.0), precision=precision)
    st = case.stabilityDerivatives()
    assert abs(case.getCL() - float(g["CL"])) <= 5.01e-6
    da, db = printed_stability(st)
    assert np.all(np.abs(da - g["d_alpha_CL_CY_Cm_Cl_Cn"]) <= 5.01e-6), da
    assert np.all(np.abs(db - g["d_beta_CL_CY_Cm_Cl_Cn"]) <= 5.01e-6), db


def test_volume_survey_matches_oracle(cg, small, tmp_path):
    """cpCase::velocityAtPoint over a volume grid around the wing (plain path): the GPU's panel
    velocities with the wake doublets the library derives, against the oracle's own chain (its
    solve, its wakePanel::setMu, its panelV sums) plus V_inf."""
    from cpanel_gb300 import io
    from oracle import pyoracle as po
    g, m, Ao, Bo, refs = small
    case = cg.CpCase(g, 1.0, 5.0, 0.0, 0.1, precision="fp64", **refs)
    assert case.run()
    sv = case.volumeSurvey((-0.5, 1.5, -1.0, 1.0, -0.5, 0.5), (8, 6, 5))
    o = m.case(Ao, Bo, alpha=5.0, mach=0.1, **refs)
    vo = po.panels_velocity(m.body_verts(), o["sigma"], o["mu"], m.wake_verts(), o["wake_mu"], sv["centers"])
    vo = vo + case.vinf()
    scale = np.abs(vo).max()
    assert np.abs(sv["velocity"] - vo).max() <= 1e-9 * scale
    assert np.allclose(sv["cp"], (np.linalg.norm(vo, axis=1) / 1.0) ** 2, rtol=1e-8)
    vtu, cpout = case.writeFiles(str(tmp_path))
    d = io.read_vtu_cells(os.path.join(os.path.dirname(vtu), "volumeMesh.vtu"))
    assert np.allclose(d["Cp"], sv["cp"], rtol=1e-5)


def test_streamlines_match_oracle(cg, small, tmp_path):
    """streamline::streamline through geometry::pntVelocity around the wing (plain path): the
    library's lockstep integration, one batched panel-velocity launch per Runge-Kutta stage, against
    the oracle integrating each line alone through its own solve and panel sums.  Points agree to
    1e-7: the two velocity sums round differently and the step-size control carries that along."""
    from oracle import pyoracle as po
    g, m, Ao, Bo, refs = small
    case = cg.CpCase(g, 1.0, 5.0, 0.0, 0.1, precision="fp64", **refs)
    assert case.run()
    starts = np.array([[-0.5, 0.3, 0.15], [-0.5, 1.0, -0.3], [-0.5, -0.8, 0.3]])
    lines, ended = case.streamlines(starts, x_max=2.0, tol=1e-4, max_points=400)
    assert ended.all()
    o = m.case(Ao, Bo, alpha=5.0, mach=0.1, **refs)
    vel = po.point_velocity(m.body_verts(), o["sigma"], o["mu"], m.wake_verts(), o["wake_mu"], case.vinf(), 0.1)
    for (p, v), s in zip(lines, starts):
        op, ov, oe = po.streamline(vel, s, 1.0, 2.0, 1e-4, 400)
        assert oe and p.shape == op.shape and len(p) >= 3
        assert np.abs(p - op).max() <= 1e-7
        assert np.abs(v - ov).max() <= 1e-7 * np.abs(ov).max()
    from cpanel_gb300 import io
    vtu, _ = case.writeFiles(str(tmp_path))
    pieces = io.read_vtu_pieces(os.path.join(os.path.dirname(vtu), "OffBodyStreamlines.vtu"))
    assert [len(d["Position"]) for d in pieces] == [len(p) for p, _ in lines]


def test_case_write_files(cg, small, tmp_path):
    """cpCase::writeFiles: the case directory with surfaceData.vtu and the .CPout beside it, read
    back equal to the case's results at the printed precision."""
    import re

    from cpanel_gb300 import io
    g, m, Ao, Bo, refs = small
    case = cg.CpCase(g, 1.0, 5.0, 0.0, 0.1, precision="mixed", **refs)
    assert case.run()
    vtu, cpout = case.writeFiles(str(tmp_path), geom_file="wing.tri")
    assert vtu.endswith(os.path.join("V1_Mach0.1_alpha5_beta0", "surfaceData.vtu"))
    d = io.read_vtu_cells(vtu)
    assert np.allclose(d["Cp"], case.getCp(), rtol=1e-5, atol=1e-6)
    assert np.allclose(d["Doublet Strengths"], case.getMu(), rtol=1e-5, atol=1e-7)
    assert d["connectivity"].reshape(-1, 3).max() < len(d["Position"])
    cl = float(re.search(r"CL = (\S+)", open(cpout).read()).group(1))
    assert abs(cl - case.getCL()) <= 5.01e-6


def test_mixed_matches_plain_within_tolerance(cg, small):
    g, m, Ao, Bo, refs = small
    flows = [(1.0, a, 0.0, 0.1) for a in (-4.0, 0.0, 5.0, 12.0)]
    rp = cg.solve_cases(g, flows, precision="fp64", **refs)
    rm = cg.solve_cases(g, flows, precision="mixed", **refs)
    assert rm["status"] == 0
    assert np.abs(rm["cp"] - rp["cp"]).max() <= 1e-5
    assert np.all(np.abs(rm["CL"] - rp["CL"]) <= 1e-6 * np.abs(rp["CL"]) + 1e-9)


def test_repeated_geometries_reuse_matrix_buffers(cg, small):
    """A destroyed geometry's matrices go to its context's spares and the next geometry of the
    same size takes them: every solve overwrites them completely, so the results repeat bit
    for bit; the spares can be freed at any time."""
    g, m, Ao, Bo, refs = small
    ctx = cg.Context(0)
    flows = [(1.0, a, 0.0, 0.1) for a in (-2.0, 4.0)]
    outs = []
    for _ in range(3):
        ge = cg.Geometry(m.nodes, m.tris, m.ids, ctx=ctx)
        outs.append(cg.solve_cases(ge, flows, precision="mixed", want=("mu", "cp"), **refs))
        del ge
    for o in outs[1:]:
        assert np.array_equal(o["cp"], outs[0]["cp"]) and np.array_equal(o["mu"], outs[0]["mu"])
    ctx.release_spares()
    ge = cg.Geometry(m.nodes, m.tris, m.ids, ctx=ctx)
    o = cg.solve_cases(ge, flows, precision="mixed", want=("cp",), **refs)
    assert np.array_equal(o["cp"], outs[0]["cp"])


def test_mixed_many_right_hand_sides(cg, small):
    """More cases than one column group of the blocked triangular solves (32)."""
    g, m, Ao, Bo, refs = small
    flows = [(1.0, -4.0 + 0.4 * q, 0.5 * (q % 3), 0.1) for q in range(40)]
    rp = cg.solve_cases(g, flows, precision="fp64", **refs)
    rm = cg.solve_cases(g, flows, precision="mixed", **refs)
    assert rm["status"] == 0
    assert np.abs(rm["cp"] - rp["cp"]).max() <= 1e-5
    assert np.all(np.abs(rm["CL"] - rp["CL"]) <= 1e-6 * np.abs(rp["CL"]) + 1e-9)


def test_small_steady_workload_parity(cg):
    """The 3,896-panel NACA 0012 wing (alpha = 5 deg, Mach 0.1): plain GPU vs oracle."""
    from cpanel_gb300 import wing
    from oracle import pyoracle as po
    spec = wing.config_small_steady()
    nodes, tris, ids, info = wing.make_wing(spec)
    g = cg.Geometry(nodes, tris, ids)
    refs = dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0.0, 0.0))
    r = cg.solve_cases(g, [(1.0, 5.0, 0.0, 0.1)], precision="fp64", **refs)
    m = po.Mesh(nodes, tris, ids)
    Ao, Bo = m.set_inf_coeff()
    assert _matrix_rel_err(g.getA(), Ao) < 1e-12
    o = m.case(Ao, Bo, alpha=5.0, mach=0.1, **refs)
    assert np.abs(r["mu"][0] - o["mu"]).max() < 1e-10
    assert np.abs(r["cp"][0] - o["cp"]).max() < 1e-10
    assert abs(r["CL"][0] - o["CL"]) < 1e-10 and abs(r["CDi"][0] - o["CDi"]) < 1e-10
    rm = cg.solve_cases(g, [(1.0, 5.0, 0.0, 0.1)], precision="mixed", **refs)
    assert np.abs(rm["cp"] - r["cp"]).max() <= 1e-5
    assert abs(rm["CL"][0] - r["CL"][0]) <= 1e-6 * abs(r["CL"][0])


def test_multi_rhs_workload_meets_the_metric_bound(cg):
    """The benchmark's own workload at full size: NACA 4412, AR 6, taper 0.6, 80 points per side x
    61 stations (19,272 body panels), 17 alphas from -4 to 12 deg.  The mixed path against the plain
    FP64 GPU path, per alpha: Cp max-abs <= 1e-5 over every panel and CL within 1e-6 relative."""
    from cpanel_gb300 import wing
    spec = wing.config_multi_rhs()
    nodes, tris, ids, info = wing.make_wing(spec)
    g = cg.Geometry(nodes, tris, ids)
    assert g.n > 19000
    refs = dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0.0, 0.0))
    flows = [(1.0, float(a), 0.0, 0.1) for a in range(-4, 13)]
    rm = cg.solve_cases(g, flows, precision="mixed", want=("cp",), **refs)
    rp = cg.solve_cases(g, flows, precision="fp64", want=("cp",), **refs)
    del g
    assert rm["status"] == 0 and rp["status"] == 0
    assert np.all(np.abs(rm["cp"] - rp["cp"]).max(axis=1) <= 1e-5)
    assert np.all(np.abs(rm["CL"] - rp["CL"]) <= 1e-6 * np.abs(rp["CL"]))


def test_invalid_arguments_are_reported(cg):
    g_err = None
    with pytest.raises(cg.CpgError) as e:
        cg.Geometry(np.zeros((3, 3)), np.array([[1, 1, 2]]), np.array([1], dtype=np.int32))
    assert e.value.code == 4
    del g_err
