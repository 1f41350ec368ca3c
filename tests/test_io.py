"""CPanel's result files (include/cpanel_io.h), on the CPU: the reference's 4412 case solved by
the oracle, written as surfaceData.vtu and .CPout by the library's writers, read back and
compared with the reference's own output for that case (surfaceData-0.vtu and 4412.CPout, kept
in tests/golden/case4412.npz) at the precision the reference prints."""
import os
import re

import numpy as np
import pytest


def _panel_tables(g):
    import cpanel_gb300 as cg
    t = cg.topology(g["nodes"], g["tris"].astype(np.int64), g["ids"])
    return t["body"]


def test_surface_vtu_round_trip_matches_reference_output(built, case4412, solved4412, tmp_path):
    from scipy.spatial import cKDTree

    from cpanel_gb300 import io
    g = case4412
    m, A, B, r = solved4412
    body = _panel_tables(g)
    tris = g["tris"].astype(np.int64)[body[:, 17].astype(np.int64)] - 1
    path = str(tmp_path / "surfaceData.vtu")
    io.write_surface_vtu(path, g["nodes"], tris, r["mu"], r["sigma"], r["phi"], r["vel"], r["cp"], body[:, 3:6],
                         body[:, 0:3])
    d = io.read_vtu_cells(path)
    n = len(body)
    assert set(d) == {"Doublet Strengths", "Source Strengths", "Velocity Potential", "Velocity", "Cp", "bezNormals",
                      "xPosition", "yPosition", "zPostition", "Position", "connectivity", "offsets", "types"}
    assert d["connectivity"].size == 3 * n and np.all(d["types"] == 5) and np.all(d["offsets"] == 3 * np.arange(1, n + 1))
    assert np.array_equal(d["connectivity"].reshape(n, 3), tris)
    # the reference's surfaceData-0.vtu, matched by panel centroid, at its 6 significant digits
    c = np.stack([d["xPosition"], d["yPosition"], d["zPostition"]], axis=1)
    dist, idx = cKDTree(c).query(g["centroid"].astype(np.float64))
    assert dist.max() < 1e-5 and len(np.unique(idx)) == len(idx)
    for name, key in (("Doublet Strengths", "mu"), ("Source Strengths", "sigma"), ("Velocity Potential", "phi"),
                      ("Cp", "cp"), ("Velocity", "vel")):
        ref = g[key].astype(np.float64)
        assert np.all(np.abs(d[name][idx] - ref) <= 1.2e-5 * np.abs(ref) + 4e-7), name


def test_cpout_matches_reference_summary(built, case4412, solved4412, tmp_path):
    from cpanel_gb300 import io
    g = case4412
    m, A, B, r = solved4412
    path = str(tmp_path / "4412.CPout")
    io.write_cpout(path, [dict(V=float(g["V"]), alpha=float(g["alpha"]), beta=float(g["beta"]), mach=float(g["mach"]),
                               CL=r["CL"], CDi=r["CDi"], Fbody=r["Fbody"], Fwind=r["Fwind"], CM=r["CM"])],
                   geom_file="4412.tri", Sref=float(g["Sref"]), bref=float(g["bref"]), cref=float(g["cref"]),
                   cg=tuple(float(x) for x in g["cg"]))
    txt = open(path).read()
    lines = txt.split("\n")
    assert lines[0] == "-----------INPUTS-----------"
    assert "              Geometry File -> 4412.tri" in lines
    assert "             Reference Area -> 6 ft^2" in lines
    assert "          Center of Gravity -> [0.25 0 0] ft" in lines
    assert "                      Alpha -> 5 degrees" in lines
    assert "                     Mach # -> 0.1 " in lines
    assert "      Stability Derivatives -> OFF" in lines
    assert "---Case #1---" in lines and "-----------RESULTS-----------" in lines
    assert "\t\t1.000      0.100  5.000   0.000   " in lines
    # the printed coefficients (5 decimals), as in the reference's 4412.CPout
    cl, cdi = re.search(r"\t\t\tCL = (\S+)\tCDi = (\S+)", txt).groups()
    assert abs(float(cl) - float(g["CL"])) < 1.01e-5 and abs(float(cdi) - float(g["CDi"])) < 1.01e-5
    rows = [ln for ln in lines if ln.startswith("\t\t\t               ")]
    body_row = [float(x) for x in rows[0].split()]
    wind_row = [float(x) for x in rows[1].split()]
    assert np.allclose(body_row, g["body_CN_CA_CY"], atol=1.01e-5)
    assert np.allclose(wind_row, g["wind_CL_CD_CY"], atol=1.01e-5)
    i = lines.index("\t\tCm (pitch)  Cl (roll)   Cn (yaw)    ")
    assert np.allclose([float(x) for x in lines[i + 1].split()], g["Cm_Cl_Cn"], atol=1.01e-5)


def test_case_label_follows_the_reference():
    from cpanel_gb300 import io
    assert io.case_label(1.0, 0.1, 5.0, 0.0) == "V1_Mach0.1_alpha5_beta0"
    assert io.case_label(1.0, 0.1, -2.5, 0.5) == "V1_Mach0.1_alpha-2.5_beta0.5"


def test_writers_reject_bad_input(built, tmp_path):
    from cpanel_gb300 import CpgError, io
    nodes = np.zeros((3, 3))
    with pytest.raises(CpgError):  # node index outside the node list
        io.write_surface_vtu(str(tmp_path / "x.vtu"), nodes, np.array([[0, 1, 3]]), *([np.zeros(1)] * 4)[:3],
                             np.zeros((1, 3)), np.zeros(1), np.zeros((1, 3)), np.zeros((1, 3)))
    with pytest.raises(CpgError):  # a directory that does not exist
        io.write_cpout(str(tmp_path / "missing" / "x.CPout"), [])


def test_cpout_stability_block_matches_reference(built, case4412ar6, solved4412ar6, tmp_path):
    """The stability-derivative block of the reference's 4412AR6.CPout, from the oracle's
    derivatives through the writer."""
    from cpanel_gb300 import io
    g = case4412ar6
    r0, st = solved4412ar6
    path = str(tmp_path / "4412AR6.CPout")
    io.write_cpout(path, [dict(V=1.0, alpha=5.0, beta=0.0, mach=0.1, CL=r0["CL"], CDi=r0["CDi"], Fbody=r0["Fbody"],
                               Fwind=r0["Fwind"], CM=r0["CM"], stability=st)],
                   geom_file="4412AR6.tri", Sref=6.0, bref=6.0, cref=1.0, cg=(0.25, 0.0, 0.0),
                   flags=dict(stability_derivatives=True))
    lines = open(path).read().split("\n")
    assert "      Stability Derivatives -> ON" in lines and "\t--Stability Derivatives--" in lines
    i = lines.index("\t\tCL_alpha    CY_alpha    Cm_alpha    Cl_alpha    Cn_alpha    ")
    assert lines[i + 2] == "\t\tCL_beta     CY_beta     Cm_beta     Cl_beta     Cn_beta     "
    assert np.allclose([float(x) for x in lines[i + 1].split()], g["d_alpha_CL_CY_Cm_Cl_Cn"], atol=1.01e-5)
    assert np.allclose([float(x) for x in lines[i + 3].split()], g["d_beta_CL_CY_Cm_Cl_Cn"], atol=1.01e-5)


def test_volume_grid_follows_create_vol_mesh():
    """The grid of cpCase::createVolMesh (CPanel/cpCase.cpp:1024-1097), restated here as its
    loops, against the vectorised io.volume_grid."""
    from cpanel_gb300 import io
    bounds, (nX, nY, nZ) = (-1.0, 2.0, 0.5, 1.5, -0.25, 0.75), (3, 2, 4)
    pts, cells, centers = io.volume_grid(bounds, (nX, nY, nZ))
    x0, xf, y0, yf, z0, zf = bounds
    hx, hy, hz = (xf - x0) / nX, (yf - y0) / nY, (zf - z0) / nZ
    nXp, nYp, nZp = nX + 1, nY + 1, nZ + 1
    ref_pts = [(x0 + hx * i, y0 + hy * j, z0 + hz * k) for k in range(nZp) for j in range(nYp) for i in range(nXp)]
    ref_cells = []
    for i in range(nX):
        for j in range(nY):
            for k in range(nZ):
                b = k * nXp * nYp + j * nXp + i
                t = (k + 1) * nXp * nYp + j * nXp + i
                ref_cells.append([b, b + 1, b + nXp, b + nXp + 1, t, t + 1, t + nXp, t + nXp + 1])
    assert np.allclose(pts, ref_pts, rtol=0, atol=1e-15)
    assert np.array_equal(cells, ref_cells)
    assert np.allclose(centers, np.array(ref_pts)[np.array(ref_cells)].mean(axis=1), rtol=0, atol=1e-15)


def test_volume_vtu_round_trip(built, tmp_path):
    from cpanel_gb300 import io
    pts, cells, centers = io.volume_grid((0, 1, 0, 1, 0, 1), (2, 2, 2))
    vel = np.arange(3 * len(cells), dtype=float).reshape(-1, 3) / 7
    cp = np.linspace(0.5, 1.5, len(cells))
    path = str(tmp_path / "volumeMesh.vtu")
    io.write_volume_vtu(path, pts, cells, vel, cp)
    d = io.read_vtu_cells(path)
    assert np.allclose(d["Velocity"], vel, rtol=1e-5) and np.allclose(d["Cp"], cp, rtol=1e-5)
    assert np.array_equal(d["connectivity"].reshape(-1, 8), cells) and np.all(d["types"] == 11)
    assert np.allclose(d["Position"], pts)


def test_wake_vtu_matches_reference_output(built, case4412, solved4412, tmp_path):
    """wakeData.vtu for the reference's 4412 case from the oracle's body doublets: the wake
    doublets (wakePanel::setMu) and potentials (panel::setPotential) against the reference's
    own wakeData-0.vtu, matched by panel centroid, at its 6 significant digits."""
    from scipy.spatial import cKDTree

    import cpanel_gb300 as cg
    from cpanel_gb300 import io
    from conftest import GOLDEN
    g = case4412
    ref = dict(np.load(os.path.join(GOLDEN, "case4412_wake.npz")))
    m, A, B, r = solved4412
    tri = g["tris"].astype(np.int64)
    t = cg.topology(g["nodes"], tri, g["ids"])
    a = np.radians(float(g["alpha"]))
    vinf = float(g["V"]) * np.array([np.cos(a), 0.0, np.sin(a)])
    wmu, wphi = io.wake_fields(r["mu"], t["idx4"], t["coef"], t["wake"][:, 0:3], vinf)
    assert np.allclose(wmu, r["wake_mu"], rtol=0, atol=1e-14)  # the oracle's own wakePanel::setMu
    wt = io.wake_tris(g["nodes"], tri, g["ids"])
    path = str(tmp_path / "wakeData.vtu")
    io.write_wake_vtu(path, g["nodes"], tri[wt] - 1, wmu, wphi)
    d = io.read_vtu_cells(path)
    con = d["connectivity"].reshape(-1, 3)
    c = d["Position"][con].mean(axis=1)
    assert np.allclose(c, t["wake"][:, 0:3], atol=1e-12)  # the written triangles are the wake panels
    dist, idx = cKDTree(c).query(ref["centroid"].astype(np.float64))
    assert dist.max() < 1e-4 and len(np.unique(idx)) == len(idx) == len(wmu)
    for name, key in (("Doublet Strengths", "mu"), ("Velocity Potential", "phi")):
        want = ref[key].astype(np.float64)
        assert np.all(np.abs(d[name][idx] - want) <= 1.2e-5 * np.abs(want) + 4e-7), name


def test_case_write_files_on_host(built, case4412, solved4412, tmp_path):
    """CpCase.writeFiles itself, on the CPU: a stand-in geometry with the host topology tables
    and the oracle's solution in place of the device results."""
    import cpanel_gb300 as cg
    from cpanel_gb300 import io
    g = case4412
    m, A, B, r = solved4412
    tri = g["tris"].astype(np.int64)
    t = cg.topology(g["nodes"], tri, g["ids"])

    class HostGeometry:
        _nodes, _tris, _ids = g["nodes"], tri, g["ids"]
        n, nw = m.n, m.nw

        def tables(self):
            return t

    case = cg.CpCase.__new__(cg.CpCase)
    case.geom = HostGeometry()
    case.flow = (float(g["V"]), float(g["alpha"]), float(g["beta"]), float(g["mach"]))
    case.refs = dict(Sref=float(g["Sref"]), bref=float(g["bref"]), cref=float(g["cref"]),
                     cg=tuple(float(x) for x in g["cg"]))
    case.precision = "fp64"
    case.stab = None
    case.survey = None
    case.res = {k: np.asarray(r[k])[None] for k in ("mu", "sigma", "phi", "cp", "vel", "Fbody", "Fwind", "CM")}
    case.res.update(CL=np.array([r["CL"]]), CDi=np.array([r["CDi"]]))
    vtu, cpout = case.writeFiles(str(tmp_path), geom_file="4412.tri")
    sub = os.path.dirname(vtu)
    assert os.path.basename(sub) == "V1_Mach0.1_alpha5_beta0" and os.path.basename(cpout) == "4412.CPout"
    d = io.read_vtu_cells(vtu)
    assert np.allclose(d["Cp"], r["cp"], rtol=1e-5, atol=1e-6)
    w = io.read_vtu_cells(os.path.join(sub, "wakeData.vtu"))
    assert np.allclose(w["Doublet Strengths"], r["wake_mu"], rtol=1e-5, atol=1e-7)
    assert "CL = %.5f" % r["CL"] in open(cpout).read()



def test_spanwise_csv_matches_reference_file(built, case4412, solved4412, tmp_path):
    """cpg_write_spanwise_csv on the oracle's loads of the reference's 4412 case writes the reference's
    own spanwiseData_Wake1.csv character for character (cpCase::writeSpanwiseData,
    CPanel/cpCase.cpp:910-935); the fixture's parsed numbers print back to the same text."""
    from cpanel_gb300 import io
    from test_oracle_pin import spanwise_reference
    g = case4412
    m, A, B, r = solved4412
    m.post(r["mu"], V=float(g["V"]), alpha=float(g["alpha"]), beta=float(g["beta"]), mach=float(g["mach"]),
           Sref=float(g["Sref"]), bref=float(g["bref"]), cref=float(g["cref"]), cg=tuple(g["cg"]))
    ref = spanwise_reference()
    ours = tmp_path / "spanwiseData_Wake1.csv"
    io.write_spanwise_csv(str(ours), m.spanwise(0))
    assert ours.read_text().splitlines() == list(ref["lines"])
    back = tmp_path / "fixture.csv"
    io.write_spanwise_csv(str(back), {k: ref[k] for k in ("y2b", "cl", "cdi")})
    assert back.read_text().splitlines() == list(ref["lines"])
