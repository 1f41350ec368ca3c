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
