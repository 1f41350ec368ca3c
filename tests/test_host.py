"""Host-side checks that need no GPU: the C-ABI library, the product's readTri
topology against the oracle (bit for bit), and the synthetic wing generator."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, small_wing


def _declared_symbols():
    syms = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(cpg_[A-Za-z0-9_]+)\s*\(", txt):
            syms.add(m.group(1))
    return syms


def test_library_exports_every_declared_symbol(built):
    from cpanel_gb300 import _lib
    L = _lib.load()
    declared = _declared_symbols()
    assert declared, "no declarations found"
    for s in declared:
        assert hasattr(L, s), s
    assert declared == set(_lib.EXPORTS)
    assert L.cpg_compiled_arch() == 103


def test_no_device_is_an_error_not_a_fallback(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    import cpanel_gb300 as cg
    with pytest.raises(cg.CpgError) as e:
        cg.Context(0)
    assert e.value.code == 7


def _compare_topology(nodes, tris, ids):
    import cpanel_gb300 as cg
    from oracle import pyoracle as po
    t = cg.topology(nodes, tris, ids)
    m = po.Mesh(nodes, tris, ids)
    ow, oi, oc = m.wake_table()
    assert t["info"]["n_body"] == m.n and t["info"]["n_wake"] == m.nw
    assert np.array_equal(t["body"], m.body_table())
    assert np.array_equal(t["wake"], ow)
    assert np.array_equal(t["idx4"], oi)
    assert np.array_equal(t["coef"], oc)
    assert np.array_equal(t["clusters"], m.clusters())
    return t


def test_topology_4412_matches_oracle(built, case4412):
    g = case4412
    t = _compare_topology(g["nodes"], g["tris"].astype(np.int64), g["ids"])
    assert t["info"]["n_tip"] == 68 and t["info"]["n_wakelines"] == 20


@pytest.mark.parametrize("which", ["small", "multi", "rand5"])
def test_topology_synthetic_matches_oracle(built, which):
    from cpanel_gb300 import wing
    spec = {"small": wing.config_small_steady, "multi": wing.config_multi_rhs,
            "rand5": lambda: wing.config_random(5)}[which]()
    nodes, tris, ids, info = wing.make_wing(spec)
    t = _compare_topology(nodes, tris, ids)
    assert t["info"]["n_tip"] == 0
    assert t["info"]["n_wakelines"] == spec.n_span - 1


def test_topology_from_many_threads_is_unchanged(built):
    """Meshes built from several host threads at once share the builder's thread pool (each call
    queues its slices and runs some itself): every table equals the one built alone."""
    import threading

    import cpanel_gb300 as cg
    from cpanel_gb300 import wing
    meshes = [wing.make_wing(wing.config_random(20261203 + s))[:3] for s in range(3)]
    alone = [cg.topology(*m) for m in meshes]
    got = [None] * 6
    errs = []

    def run(i):
        try:
            got[i] = cg.topology(*meshes[i % 3])
        except Exception as e:  # reported below
            errs.append(e)

    ts = [threading.Thread(target=run, args=(i,)) for i in range(6)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs
    for i, t in enumerate(got):
        ref = alone[i % 3]
        assert t["info"] == ref["info"]
        for key in ("body", "wake", "idx4", "coef", "clusters"):
            assert np.array_equal(t[key], ref[key]), key


def test_bad_mesh_is_reported(built):
    import cpanel_gb300 as cg
    nodes = np.zeros((3, 3))
    tris = np.array([[1, 1, 2]])
    with pytest.raises(cg.CpgError) as e:
        cg.topology(nodes, tris, np.array([1], dtype=np.int32))
    assert e.value.code == 4
    with pytest.raises(cg.CpgError):
        cg.topology(nodes, np.array([[1, 2, 9]]), np.array([1], dtype=np.int32))


def test_generator_counts_match_the_workloads():
    from cpanel_gb300 import wing
    n1 = wing.make_wing(wing.config_small_steady())[3]
    # 3,744 surface triangles and two paired tip caps of 2 x (2 x 40 - 4) / 2 triangles each
    assert n1["n_surface"] == 4 * 39 * 24 and n1["n_body"] == 3744 + 2 * (2 * 40 - 4) and n1["n_wake"] == 48
    n2 = wing.make_wing(wing.config_multi_rhs())[3]
    assert 19000 <= n2["n_body"] <= 19400
    for s in range(8):
        info = wing.make_wing(wing.config_random(20261203 + s))[3]
        assert 1000 <= info["n_surface"] + 0 and info["n_body"] <= 12600


def test_generator_closed_outward_surface():
    from oracle import pyoracle as po
    nodes, tris, ids, info, spec = small_wing(wake_len=0.0)
    m = po.Mesh(nodes, tris, ids)
    A, _ = m.set_inf_coeff()
    assert np.abs(A.sum(axis=1) + 1).max() < 1e-3  # closed, normals outward
    bt = m.body_table()
    assert bt[:, 11].sum() == 0  # no accidental tip-patch flags
