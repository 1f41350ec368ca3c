"""The C++ drop-in shim (include/cpanel_shim.hpp) from a compiled C++ caller.

tests/shim/shim_test.cpp includes only the shim header and links libcpanel_gb300.so; it runs
the reference's unit-triangle known answers, the reference's 4412 case through
geometry::readTri / setInfCoeff / getA / getB and cpCase::solveMatrixEq (against the case's
own surfaceData-0.vtu and .CPout, tests/golden/case4412.npz), and the particle operators
against the CPU oracle.  The CPU test checks that the program compiles and links; the GPU test
runs it.
"""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _compile(out_dir):
    from cpanel_gb300 import build
    lib = build.build()
    exe = os.path.join(str(out_dir), "shim_test")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(build.CUDA, "include"), os.path.join(HERE, "shim", "shim_test.cpp"), "-o", exe,
           "-L" + os.path.dirname(lib), "-lcpanel_gb300", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_shim_program_compiles_and_links(built, tmp_path):
    exe = _compile(tmp_path)
    assert os.path.getsize(exe) > 0


def _write_inputs(d, case4412):
    g = case4412
    nodes, tris, ids = g["nodes"], g["tris"], g["ids"]
    with open(os.path.join(d, "mesh4412.tri"), "w") as f:  # Cart3D .tri, as readTri reads it
        f.write("%d %d\n" % (len(nodes), len(tris)))
        for p in nodes:
            f.write("%.17g %.17g %.17g\n" % tuple(p))
        for t in tris:
            f.write("%d %d %d\n" % tuple(t))
        for s in ids:
            f.write("%d\n" % s)
    head = [len(g["mu"]), g["V"], g["alpha"], g["beta"], g["mach"], g["Sref"], g["bref"], g["cref"], *g["cg"],
            g["CL"], g["CDi"]]
    np.concatenate([np.array(head, dtype=np.float64), g["mu"].astype(np.float64),
                    g["cp"].astype(np.float64)]).tofile(os.path.join(d, "case4412.bin"))
    from oracle import pyoracle as po
    rng = np.random.default_rng(17)
    n, m = 600, 40
    pos = np.concatenate([rng.normal(size=(n // 2, 3)) * 0.3, rng.normal(size=(n - n // 2, 3)) + 2.0])
    st = rng.normal(size=(n, 3)) * 0.01
    rad = rng.uniform(0.02, 0.08, n)
    pts = rng.normal(size=(m, 3)) * 1.5
    t = po.ParticleTree(pos, st, rad, max_members=10, theta=0.5)
    pair = [po.particles_velocity(pos[:2], st[:2], rad[:2])[1], po.particles_stretch(pos[:2], st[:2], rad[:2])[0],
            po.particles_diffusion(pos[:2], st[:2], rad[:2])[0],
            po.particles_velocity(pos[:1], st[:1], rad[:1], pts=pts[:1], kernel="gauss")[0],
            po.particles_velocity(pos[:1], st[:1], rad[:1], pts=pts[:1], kernel="alg")[0]]
    np.concatenate([np.array([n, m], dtype=np.float64), pos.ravel(), st.ravel(), rad, pts.ravel(),
                    t.velocity_points(pts).ravel(), t.velocity().ravel(), t.stretch().ravel(),
                    t.diffusion().ravel(), np.concatenate(pair)]).tofile(os.path.join(d, "particles.bin"))


@pytest.mark.gpu
def test_shim_program_runs_the_reference_cases(built, case4412, tmp_path):
    exe = _compile(tmp_path)
    _write_inputs(str(tmp_path), case4412)
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "shim ok" in r.stdout and "FAIL" not in r.stdout
