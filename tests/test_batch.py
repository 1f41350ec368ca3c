"""Many meshes at once (include/cpanel_batch.h).

Host: the grouped launch's work queue covers every (mesh, row block, source chunk) of
every mesh exactly once, for every work shape.
GPU: the grouped, persistent assembly gives the same bits as the single-mesh assembly
for every work shape (given, tuned, or with geometries of two contexts in one launch),
and the batch solve gives each mesh the results of its own cpg_solve_cases (mixed
precision): within 1e-12 with each mesh on its worker, and within the bounds written at
the lockstep test with the lockstep factorizations and solves; in one wave or split into
several.
"""
import numpy as np
import pytest

from conftest import small_wing

SHAPES = [None, dict(chunks_per_item=1, near_band=0, blocks_per_sm=1),
          dict(chunks_per_item=8, near_band=4, blocks_per_sm=2), dict(chunks_per_item=16, near_band=64)]


@pytest.mark.parametrize("shape", SHAPES)
def test_group_schedule_covers_every_block_once(built, shape):
    from cpanel_gb300 import batch
    ns = [129, 300, 1000, 4000, 12000, 2]
    items, ch = batch.group_schedule(ns, shape)
    seen = {}
    for q, bx, by, g in items:
        assert g >= 1
        for c in range(by, by + g):
            key = (int(q), int(bx), c)
            assert key not in seen, key
            seen[key] = True
    for q, n in enumerate(ns):
        nbx = (n + 127) // 128
        nby = (n + ch[q] - 1) // ch[q]
        assert ch[q] % 32 == 0
        for bx in range(nbx):
            for c in range(nby):
                assert (q, bx, c) in seen
    assert len(seen) == sum(((n + 127) // 128) * ((n + c - 1) // c) for n, c in zip(ns, ch))
    sh = dict(batch.default_shape())
    sh.update(shape or {})
    # near items (row and source ranges within near_band chunk lengths) hold one chunk
    for q, bx, by, g in items:
        r0, r1 = 128 * bx, min(ns[q], 128 * (bx + 1))
        for c in range(by, by + g):
            c0, c1 = c * ch[q], min(ns[q], (c + 1) * ch[q])
            gap = c0 - r1 if c0 >= r1 else (r0 - c1 if r0 >= c1 else 0)
            if g > 1:
                assert gap > sh["near_band"] * ch[q]
        assert g <= sh["chunks_per_item"]


def test_group_schedule_rejects_bad_shapes(built):
    from cpanel_gb300 import CpgError, batch
    for bad in (dict(chunks_per_item=0), dict(near_band=-1), dict(chunks_per_item=17)):
        with pytest.raises(CpgError):
            batch.group_schedule([1000], bad)
    with pytest.raises(CpgError):
        batch.group_schedule([0], None)


def _wings():
    out = []
    for q, (nc, ns, taper, m) in enumerate([(10, 6, 1.0, 0.0), (24, 12, 0.6, 0.04), (14, 8, 0.8, 0.02),
                                             (30, 14, 0.5, 0.03), (12, 5, 0.7, 0.0)]):
        nodes, tris, ids, info, spec = small_wing(n_chord=nc, n_span=ns, taper=taper, m=m, seed=q)
        flows = [(1.0, -2.0 + 4.0 * j + 0.5 * q, 0.0, 0.1) for j in range(3)]
        out.append(dict(nodes=nodes, tris=tris, ids=ids, flows=flows, Sref=info["area"], bref=spec.span, cref=1.0,
                        cg=(0.25, 0.0, 0.0)))
    return out


@pytest.fixture(scope="module")
def per_mesh(built):
    """Each wing alone: single-mesh mixed assembly and its solve."""
    import cpanel_gb300 as cg
    res = []
    for w in _wings():
        g = cg.Geometry(w["nodes"], w["tris"], w["ids"])
        g.setInfCoeff("mixed")
        A = g.getA()
        out = cg.solve_cases(g, w["flows"], Sref=w["Sref"], bref=w["bref"], cref=w["cref"], cg=w["cg"],
                             precision="mixed", want=("mu", "cp"))
        res.append(dict(A=A, cp=out["cp"], mu=out["mu"], CL=out["CL"], CDi=out["CDi"],
                        near=out["stats"]["n_near"]))
        del g
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
def test_grouped_assembly_is_bit_identical(per_mesh, shape):
    import cpanel_gb300 as cg
    from cpanel_gb300 import batch
    ws = _wings()
    geoms = [cg.Geometry(w["nodes"], w["tris"], w["ids"]) for w in ws]
    rep = batch.set_inf_coeff_grouped(geoms, tune="off", shape=shape)
    assert rep["pairs"] == sum(g.n * g.n for g in geoms)
    assert rep["near_pairs"] == sum(r["near"] for r in per_mesh)
    for g, r in zip(geoms, per_mesh):
        assert np.array_equal(g.getA(), r["A"])


@pytest.mark.gpu
def test_grouped_assembly_tuned_and_across_contexts(per_mesh):
    import cpanel_gb300 as cg
    from cpanel_gb300 import batch
    ws = _wings()
    c2 = cg.Context(0)
    geoms = [cg.Geometry(w["nodes"], w["tris"], w["ids"], ctx=(c2 if q % 2 else None)) for q, w in enumerate(ws)]
    rep = batch.set_inf_coeff_grouped(geoms, tune="force")
    assert rep["tuned"] == 1 and rep["candidates"] >= 5
    for g, r in zip(geoms, per_mesh):
        assert np.array_equal(g.getA(), r["A"])
    rep2 = batch.set_inf_coeff_grouped(geoms, tune="auto")
    assert rep2["tuned"] == 2 and rep2["shape"] == rep["shape"]
    for q, (g, r, w) in enumerate(zip(geoms, per_mesh, ws)):
        assert np.array_equal(g.getA(), r["A"])
        out = cg.solve_cases(g, w["flows"], Sref=w["Sref"], bref=w["bref"], cref=w["cref"], cg=w["cg"],
                             precision="mixed", want=("cp",))
        assert np.allclose(out["cp"], r["cp"], rtol=0, atol=1e-12)
        assert np.allclose(out["CL"], r["CL"], rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("budget_gb", [0.0, 1e-6])
def test_batch_solve_matches_each_mesh_alone(per_mesh, budget_gb):
    """Factorizations on the workers: the same kernels as each mesh alone."""
    from cpanel_gb300 import batch
    ws = _wings()
    res, st = batch.batch_solve(ws, workers=3, tune="auto", budget_gb=budget_gb, want=("cp", "mu", "CL", "CDi"),
                                lockstep=False)
    assert st["failed"] == 0 and st["solves"] == sum(len(w["flows"]) for w in ws)
    assert st["waves"] == (1 if budget_gb == 0.0 else len(ws))
    for o, r in zip(res, per_mesh):
        assert o["status"] == 0
        assert o["cp"].shape == r["cp"].shape
        assert np.allclose(o["mu"], r["mu"], rtol=0, atol=1e-12 * np.abs(r["mu"]).max())
        assert np.allclose(o["cp"], r["cp"], rtol=0, atol=1e-12)
        assert np.allclose(o["CL"], r["CL"], rtol=1e-12, atol=0)
        assert np.allclose(o["CDi"], r["CDi"], rtol=1e-12, atol=0)


# Lockstep factorizations and refined solves against each mesh's own: both refine to
# relative residual 1e-12 from FP32 factors that differ in rounding, so the solutions agree
# to about cond(A) 1e-12
# in mu; the CHTLS velocity weights (order 1/h at the clustered trailing edge) amplify that
# in Cp.  Bounds: mu 1e-9 relative to max |mu|, Cp 1e-7 absolute, CL and CDi 1e-8 relative
# (the path's own bar against the plain FP64 path is Cp 1e-5 and CL 1e-6).
@pytest.mark.gpu
@pytest.mark.parametrize("budget_gb", [0.0, 1e-6])
def test_batch_solve_lockstep_factorization(per_mesh, budget_gb):
    from cpanel_gb300 import batch
    ws = _wings()
    res, st = batch.batch_solve(ws, workers=3, tune="auto", budget_gb=budget_gb, want=("cp", "mu", "CL", "CDi"),
                                lockstep=True)
    assert st["failed"] == 0 and st["ms_factor"] > 0
    worst = {}
    for o, r in zip(res, per_mesh):
        assert o["status"] == 0
        worst["mu"] = max(worst.get("mu", 0), np.abs(o["mu"] - r["mu"]).max() / np.abs(r["mu"]).max())
        worst["cp"] = max(worst.get("cp", 0), np.abs(o["cp"] - r["cp"]).max())
        worst["CL"] = max(worst.get("CL", 0), (np.abs(o["CL"] - r["CL"]) / np.abs(r["CL"])).max())
        worst["CDi"] = max(worst.get("CDi", 0), (np.abs(o["CDi"] - r["CDi"]) / np.abs(r["CDi"])).max())
    assert st["waves"] == (1 if budget_gb == 0.0 else len(ws))
    print("lockstep vs per-mesh:", worst)
    assert worst["mu"] < 1e-9 and worst["cp"] < 1e-7 and worst["CL"] < 1e-8 and worst["CDi"] < 1e-8


@pytest.mark.gpu
def test_lockstep_factorization_then_solve_cases(per_mesh):
    import cpanel_gb300 as cg
    from cpanel_gb300 import batch
    ws = _wings()
    geoms = [cg.Geometry(w["nodes"], w["tris"], w["ids"]) for w in ws]
    with pytest.raises(cg.CpgError):
        batch.lu_factor_grouped(geoms)  # no mixed matrix yet
    batch.set_inf_coeff_grouped(geoms)
    assert batch.lu_factor_grouped(geoms) > 0
    for g, r, w in zip(geoms, per_mesh, ws):
        out = cg.solve_cases(g, w["flows"], Sref=w["Sref"], bref=w["bref"], cref=w["cref"], cg=w["cg"],
                             precision="mixed", want=("cp",))
        assert out["stats"]["residual_max"] <= 1e-12
        assert np.abs(out["cp"] - r["cp"]).max() < 1e-7


@pytest.mark.gpu
@pytest.mark.parametrize("lockstep", [False, True])
def test_batch_solve_isolates_a_bad_mesh(per_mesh, lockstep):
    """A mesh the path rejects fails alone; the others are solved as before."""
    from cpanel_gb300 import batch
    ws = _wings()
    bad = dict(ws[1])
    bad["tris"] = bad["tris"][:1]  # one body triangle: fewer than two body panels
    bad["ids"] = bad["ids"][:1]
    res, st = batch.batch_solve([ws[0], bad, ws[2]], workers=2, lockstep=lockstep, want=("cp", "CL"))
    assert st["failed"] == 1 and res[1]["status"] == 4  # CPG_E_BAD_MESH
    for o, r in zip([res[0], res[2]], [per_mesh[0], per_mesh[2]]):
        assert o["status"] == 0
        assert np.abs(o["cp"] - r["cp"]).max() < 1e-7
        assert np.allclose(o["CL"], r["CL"], rtol=1e-8, atol=0)


@pytest.mark.gpu
def test_batch_meets_the_metric_bound_on_config_wings(built):
    """Four of the uneven-batch wings (the benchmark's seeds: 20261203 + 0, 16, 32, 48, 8 alphas
    each) through the lockstep batch path against the plain FP64 path: Cp max-abs <= 1e-5 over
    every panel, tip caps included, and CL within 1e-6 relative, the metric's bounds."""
    import cpanel_gb300 as cg
    from cpanel_gb300 import batch, wing
    meshes = []
    for i in (0, 16, 32, 48):
        spec = wing.config_random(20261203 + i)
        nodes, tris, ids, info = wing.make_wing(spec)
        rng = np.random.default_rng(20261203 + i)
        flows = [(1.0, float(a), 0.0, 0.1) for a in rng.uniform(-2, 10, 8)]
        meshes.append(dict(nodes=nodes, tris=tris, ids=ids, flows=flows, Sref=info["area"], bref=spec.span,
                           cref=1.0, cg=(0.25, 0.0, 0.0)))
    res, st = batch.batch_solve(meshes, workers=4, tune="auto", lockstep=True, want=("cp", "CL", "CDi"))
    assert st["failed"] == 0
    for mesh, o in zip(meshes, res):
        g = cg.Geometry(mesh["nodes"], mesh["tris"], mesh["ids"])
        ref = cg.solve_cases(g, mesh["flows"], Sref=mesh["Sref"], bref=mesh["bref"], cref=mesh["cref"],
                             cg=mesh["cg"], precision="fp64", want=("cp",))
        del g
        assert np.abs(o["cp"] - ref["cp"]).max() <= 1e-5
        assert (np.abs(o["CL"] - ref["CL"]) / np.abs(ref["CL"])).max() <= 1e-6
