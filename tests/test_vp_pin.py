"""The vortex-particle case pinned to the reference's own unsteady fixture.

`Connor Cases/steadyTest` of the reference: a 3,046-triangle wing without wake panels,
Vortex_Particle_Wake on, alpha 10 deg, Mach 0.1, Accelerate_Code 1 (Barnes-Hut), Time_Step 0
(geometry::calcTimeStep), 40 steps.  The reference wrote per step the particles
(particleData-N.vtu: position, strength, Time Step Shed) and the body strengths
(surfaceData-N.vtu), the final surface pass (Cp, velocity, potential after
cpCaseVP::compVelocity) and the .CPout summary.  tests/golden/make_golden.py extracts them
into tests/golden/steadyTest.npz.  Every value is printed to 6 significant digits (the
.CPout to 5 decimals), so a value matches when it lies within half a unit of its last
printed digit.

This file runs the CPU oracle (test infrastructure) through the whole case; the GPU case
is held to the same fixture in tests/test_vp_gpu.py.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "steadyTest.npz")


def printed_match(ours, ref, rel=5e-6, slack=0.0):
    """|ours - ref| within half a unit in the 6th significant digit of ref (float32 storage of
    the fixture adds 6e-8 relative; 1e-12 absolute covers printed zeros), plus slack x max|ref|
    (a reduced-precision form's own error, relative to the array's largest value)."""
    ours, ref = np.asarray(ours, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    tol = rel * 1.02 * np.abs(ref) + 1e-12 + slack * np.abs(ref).max()
    return np.abs(ours - ref) <= tol


def run_case(make_case, fix):
    """Run the fixture's case step by step; returns the states the fixture keeps."""
    case = make_case(fix)
    part_steps = set(int(s) for s in fix["part_steps"])
    body_steps = set(int(s) for s in fix["body_steps"])
    out = {"counts": []}
    for s in range(1, int(fix["steps"]) + 1):
        case.step()
        p = case.particles()
        out["counts"].append(len(p["pos"]))
        if s in part_steps:
            out["part_%d" % s] = p
        if s in body_steps:
            out["body_%d" % s] = case.strengths()
    out["case"] = case
    return out


def oracle_case(fix):
    return po.VPCase(fix["nodes"], fix["tris"], fix["ids"], V=float(fix["V"]), alpha=float(fix["alpha"]),
                     beta=float(fix["beta"]), dt=float(fix["dt"]), cref=float(fix["cref"]),
                     accelerate=bool(fix["accelerate"]), num_steps=int(fix["steps"]), Sref=float(fix["Sref"]),
                     mach=float(fix["mach"]))


def check_against_fixture(run, fix, slack=0.0):
    # shedding: particle count after every step and the shedding step of every particle, exact
    assert run["counts"] == [int(c) for c in fix["n_particles"]]
    last = run["part_%d" % int(fix["steps"])]
    assert np.array_equal(last["shed_time"], fix["shed_step"].astype(np.int32))
    # particle positions and strengths after the kept steps
    for s in fix["part_steps"]:
        p = run["part_%d" % s]
        assert printed_match(p["pos"], fix["part_pos_%d" % s], slack=slack).all(), "positions at step %d" % s
        assert printed_match(p["strength"], fix["part_str_%d" % s], slack=slack).all(), "strengths at step %d" % s
    # body doublet and source strengths after the kept steps
    for s in fix["body_steps"]:
        b = run["body_%d" % s]
        assert printed_match(b["mu"], fix["mu_%d" % s], slack=slack).all(), "doublets at step %d" % s
        assert printed_match(b["sigma"], fix["sigma_%d" % s], slack=slack).all(), "sources at step %d" % s


def check_surface(sf, fix, slack=0.0):
    assert printed_match(sf["cp"], fix["cp_final"], slack=slack).all()
    assert printed_match(sf["vel"], fix["vel_final"], slack=slack).all()
    assert printed_match(sf["phi"], fix["phi_final"], slack=slack).all()
    # the .CPout's surface-integrated coefficients, 5 decimals
    body = [sf["Fbody"][2], sf["Fbody"][0], sf["Fbody"][1]]   # CN CA CY
    wind = [sf["Fwind"][2], sf["Fwind"][0], sf["Fwind"][1]]   # CL CD CY
    mom = [sf["CM"][1], sf["CM"][0], sf["CM"][2]]             # Cm Cl Cn
    for ours, ref in ((body, fix["body_CN_CA_CY"]), (wind, fix["wind_CL_CD_CY"]), (mom, fix["Cm_Cl_Cn"])):
        assert np.all(np.abs(np.array(ours) - ref) <= 0.5e-5 + 1e-12 + slack), (ours, ref)


@pytest.fixture(scope="module")
def fix():
    return np.load(FIX)


@pytest.fixture(scope="module")
def oracle_run(fix):
    po.lib()
    return run_case(oracle_case, fix)


def test_oracle_vp_loop_matches_reference_particles_and_strengths(oracle_run, fix):
    check_against_fixture(oracle_run, fix)


def test_oracle_vp_surface_matches_reference_final_state(oracle_run, fix):
    sf = oracle_run["case"].surface(cg=fix["cg"], bref=float(fix["bref"]), cref=float(fix["cref"]))
    check_surface(sf, fix)


def test_oracle_vp_trefftz_against_printed(oracle_run, fix):
    """The printed Trefftz CL (1.10020) is the integral over the particle row shed at step 20;
    the source's row formula (wake::trefftzPlaneVP, CPanel/wake.cpp:194-198: ceil_even(40) / 2
    + 2 = 22) gives 1.10125.  The printed CDi (0.06869) comes from neither row: its downwash
    term differs from the source's (particles only, |w_z|)."""
    S = oracle_run["case"]
    t20 = S.trefftz(row=20)
    assert abs(t20["CL"] - float(fix["CL"])) <= 0.5e-5
    t = S.trefftz()
    assert abs(t["CL"] - float(fix["CL"])) < 2e-3 and t["CL"] != pytest.approx(t20["CL"], abs=1e-5)
    assert abs(t["CD"] - float(fix["CDi"])) / float(fix["CDi"]) < 0.15
