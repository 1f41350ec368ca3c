"""The allocation-free assembly entry point, through the C ABI.

cpg_set_inf_coeff_noalloc is for callers that may not allocate device memory while
the panel path runs (graph capture, a borrowed memory pool, real-time loops).  It
must give the same A and B as the ordinary cpg_set_inf_coeff path (to the 1e-12
relative tolerance the assembly tests use), on two calls in a row that share its
fixed scratch array.  This file sorts last so that a stop-at-first-failure run has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_wing

pytestmark = pytest.mark.gpu


def _rel_err(X, Xo):
    scale = np.maximum(np.abs(Xo).max(axis=0, keepdims=True), 1e-300)
    return (np.abs(X - Xo) / scale).max()


def test_no_alloc_assembly_matches_geometry_path(built):
    import torch

    import cpanel_gb300 as cg
    from cpanel_gb300 import _lib
    from oracle import pyoracle as po

    L = _lib.load()
    nodes, tris, ids, info, spec = small_wing(n_chord=14, n_span=8)
    g = cg.Geometry(nodes, tris, ids)
    g.setInfCoeff("fp64")
    A_ref, B_ref = g.getA(), g.getB()
    n, nw = g.n, g.nw

    # panel vertices in matrix order and the wake interpolation tables
    m = po.Mesh(nodes, tris, ids)
    _, idx4, coef = m.wake_table()
    bv = torch.tensor(m.body_verts(), device="cuda")
    wv = torch.tensor(m.wake_verts(), device="cuda")
    wi = torch.tensor(idx4, device="cuda")
    wc = torch.tensor(coef, device="cuda")
    A = torch.empty((n, n), dtype=torch.float64, device="cuda")  # column-major: A[j, i] holds A(i, j)
    B = torch.empty((n, n), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        A.fill_(float("nan"))
        B.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = L.cpg_set_inf_coeff_noalloc(C.c_void_p(bv.data_ptr()), n, C.c_void_p(wv.data_ptr()),
                                         C.c_void_p(wi.data_ptr()), C.c_void_p(wc.data_ptr()), nw,
                                         C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
                                         C.c_void_p(stream.cuda_stream))
        assert rc == 0, "call %d returned %d" % (call, rc)
        torch.cuda.synchronize()
        An = A.cpu().numpy().T  # back to (row i, column j)
        Bn = B.cpu().numpy().T
        assert np.isfinite(An).all() and np.isfinite(Bn).all()
        assert _rel_err(An, A_ref) < 1e-12, "call %d: A differs" % call
        assert _rel_err(Bn, B_ref) < 1e-12, "call %d: B differs" % call


def test_no_alloc_rejects_oversized_input(built):
    from cpanel_gb300 import _lib
    L = _lib.load()
    rc = L.cpg_set_inf_coeff_noalloc(C.c_void_p(1), 16385, None, None, None, 0, C.c_void_p(1), C.c_void_p(1), None)
    assert rc == 1  # CPG_E_INVALID, nothing launched
    rc = L.cpg_set_inf_coeff_noalloc(C.c_void_p(1), 16000, C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), 385,
                                     C.c_void_p(1), C.c_void_p(1), None)
    assert rc == 1
