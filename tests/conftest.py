import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def case4412():
    return dict(np.load(os.path.join(GOLDEN, "case4412.npz")))


@pytest.fixture(scope="session")
def solved4412(case4412):
    """The reference's 4412 case through the CPU oracle: (mesh, A, B, results)."""
    from oracle import pyoracle as po
    g = case4412
    m = po.Mesh(g["nodes"], g["tris"], g["ids"])
    A, B = m.set_inf_coeff()
    r = m.case(A, B, V=float(g["V"]), alpha=float(g["alpha"]), beta=float(g["beta"]), mach=float(g["mach"]),
               Sref=float(g["Sref"]), bref=float(g["bref"]), cref=float(g["cref"]), cg=tuple(g["cg"]))
    return m, A, B, r


def small_wing(n_chord=12, n_span=6, alpha=5.0, wake_len=30.0, **kw):
    from cpanel_gb300 import wing
    spec = wing.WingSpec(m=kw.pop("m", 0.0), t=kw.pop("t", 0.12), root_chord=1.0, span=kw.pop("span", 4.0),
                         taper=kw.pop("taper", 1.0), sweep_deg=kw.pop("sweep", 0.0), n_chord=n_chord, n_span=n_span,
                         wake_len=wake_len, wake_dir=wing.wake_dir_for(alpha), **kw)
    nodes, tris, ids, info = wing.make_wing(spec)
    return nodes, tris, ids, info, spec


@pytest.fixture(scope="session")
def case4412ar6():
    return dict(np.load(os.path.join(GOLDEN, "case4412AR6.npz")))


def stability_from_cases(r0, ra, rb):
    """cpCase::stabilityDerivatives's forward differences (CPanel/cpCase.cpp:635-665) from the
    base case and its alpha + 0.5 and beta + 0.5 deg sub-cases."""
    d = 0.5 * np.pi / 180

    def F(r):
        f = np.array(r["Fwind"], dtype=float)
        f[2], f[0] = r["CL"], r["CDi"]
        return f
    return dict(dF_dAlpha=(F(ra) - F(r0)) / d, dF_dBeta=(F(rb) - F(r0)) / d,
                dM_dAlpha=(np.array(ra["CM"]) - r0["CM"]) / d, dM_dBeta=(np.array(rb["CM"]) - r0["CM"]) / d)


def printed_stability(st):
    """(CL, CY, Cm, Cl, Cn) rows for alpha and beta, in the reference's printed order."""
    return (np.array([st["dF_dAlpha"][2], st["dF_dAlpha"][1], st["dM_dAlpha"][1], st["dM_dAlpha"][0],
                      st["dM_dAlpha"][2]]),
            np.array([st["dF_dBeta"][2], st["dF_dBeta"][1], st["dM_dBeta"][1], st["dM_dBeta"][0],
                      st["dM_dBeta"][2]]))


@pytest.fixture(scope="session")
def solved4412ar6(case4412ar6):
    """The reference's 4412AR6 case (stability derivatives on) through the CPU oracle:
    (base results, stability derivatives)."""
    from oracle import pyoracle as po
    g = case4412ar6
    m = po.Mesh(g["nodes"], g["tris"], g["ids"])
    A, B = m.set_inf_coeff()
    kw = dict(V=float(g["V"]), mach=float(g["mach"]), Sref=float(g["Sref"]), bref=float(g["bref"]),
              cref=float(g["cref"]), cg=tuple(g["cg"]))
    a, b = float(g["alpha"]), float(g["beta"])
    r0 = m.case(A, B, alpha=a, beta=b, **kw)
    ra = m.case(A, B, alpha=a + 0.5, beta=b, **kw)
    rb = m.case(A, B, alpha=a, beta=b + 0.5, **kw)
    return r0, stability_from_cases(r0, ra, rb)

