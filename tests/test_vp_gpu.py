"""Vortex-particle and panel-velocity operators on the GPU against the CPU oracle.

Tolerances (FP64 on both sides; CUDA's erf/exp/atan2/log against glibc's):
  sums of pair kernels: max |gpu - oracle| <= 1e-12 x max |oracle|
  Barnes-Hut: the same bound; every far-field decision is taken on bit-identical
  expansions and rounded identically, so no node is treated differently.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rel(a, b):
    return float(np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300))


def _cuda(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _np(t):
    return t.cpu().numpy()


def _cloud(n, seed, clustered=False):
    rng = np.random.default_rng(seed)
    if clustered:
        pos = np.concatenate([rng.normal(size=(n // 2, 3)) * 0.05, rng.normal(size=(n - n // 2, 3)) + 3.0])
    else:
        pos = rng.normal(size=(n, 3))
    st = rng.normal(size=(n, 3)) * 0.01
    rad = rng.uniform(0.02, 0.08, n)
    return pos, st, rad


@pytest.mark.parametrize("kernel", ["gauss", "alg"])
def test_direct_velocity_at_points(built, kernel):
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(1500, 1)
    rng = np.random.default_rng(2)
    pts = np.concatenate([rng.normal(size=(400, 3)), pos[:20]])
    ref = po.particles_velocity(pos, st, rad, pts, kernel=kernel)
    got = _np(vp.particles_velocity(_cuda(pos), _cuda(st), _cuda(rad), _cuda(pts), kernel=kernel))
    assert _rel(got, ref) < TOL


@pytest.mark.parametrize("n,m", [(9001, 7), (20000, 300), (130, 1)])
def test_direct_velocity_few_points_many_particles(built, n, m):
    """Few targets over many sources (the Trefftz-plane downwash): the source ranges are
    summed by separate blocks and added in order; the sum is the oracle's to 1e-12."""
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(n, 40 + m)
    pts = np.random.default_rng(41).normal(size=(m, 3))
    ref = po.particles_velocity(pos, st, rad, pts, kernel="gauss")
    got = _np(vp.particles_velocity(_cuda(pos), _cuda(st), _cuda(rad), _cuda(pts), kernel="gauss"))
    assert _rel(got, ref) < TOL


def test_direct_velocity_on_particles(built):
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(1200, 3)
    ref = po.particles_velocity(pos, st, rad)  # velInfl(particle*), self skipped
    got = _np(vp.particles_velocity(_cuda(pos), _cuda(st), _cuda(rad), None, kernel="gauss_sym"))
    assert _rel(got, ref) < TOL
    ref = po.particles_velocity(pos, st, rad, pos, kernel="gauss")  # the VP loop's direct branch
    got = _np(vp.particles_velocity(_cuda(pos), _cuda(st), _cuda(rad), None, kernel="gauss"))
    assert _rel(got, ref) < TOL


def test_direct_stretch_and_diffusion(built):
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(1000, 4)
    pos *= 0.2  # many pairs inside the 5 r stretching cut-off
    s, d = vp.particles_stretch_diff(_cuda(pos), _cuda(st), _cuda(rad))
    assert _rel(_np(s), po.particles_stretch(pos, st, rad)) < TOL
    assert _rel(_np(d), po.particles_diffusion(pos, st, rad)) < TOL


@pytest.mark.parametrize("n,clustered,mm", [(4000, False, 10), (3000, True, 10), (2000, False, 4)])
def test_barnes_hut_matches_oracle(built, n, clustered, mm):
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(n, 5 + n, clustered)
    if not clustered:
        pos *= 0.3
    ref = po.ParticleTree(pos, st, rad, max_members=mm)
    tree = vp.ParticleFMM(_cuda(pos), _cuda(st), _cuda(rad), max_members=mm)
    assert np.array_equal(tree.nodes(), ref.nodes())
    assert np.array_equal(tree.leaf_members(), ref.leaf_members())
    v, s, d = tree.barnesHut()
    assert _rel(_np(v), ref.velocity()) < TOL
    assert _rel(_np(s), ref.stretch()) < TOL
    assert _rel(_np(d), ref.diffusion()) < TOL
    # one output at a time takes the same path
    assert _rel(_np(tree.barnesHutStretch()), ref.stretch()) < TOL
    rng = np.random.default_rng(n)
    pts = np.concatenate([rng.normal(size=(500, 3)), pos[:10]])
    assert _rel(_np(tree.barnesHutVel(_cuda(pts))), ref.velocity_points(pts)) < TOL


def test_barnes_hut_small_and_empty(built):
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(8, 9)  # root stays a leaf: the reference's traversal returns zero
    tree = vp.ParticleFMM(_cuda(pos), _cuda(st), _cuda(rad))
    v, s, d = tree.barnesHut()
    assert float(v.abs().max()) == 0 and float(s.abs().max()) == 0 and float(d.abs().max()) == 0
    assert float(tree.barnesHutVel(_cuda(pos)).abs().max()) == 0
    empty = vp.ParticleFMM(_cuda(np.zeros((0, 3))), _cuda(np.zeros((0, 3))), _cuda(np.zeros(0)))
    assert empty.info()["n_nodes"] == 0
    assert tuple(empty.barnesHutVel(_cuda(np.zeros((4, 3)))).shape) == (4, 3)


def test_panels_velocity_matches_oracle(built):
    from conftest import small_wing

    from cpanel_gb300 import vp
    nodes, tris, ids, info, spec = small_wing(n_chord=10, n_span=5)
    m = po.Mesh(nodes, tris, ids)
    bv, wv = m.body_verts(), m.wake_verts()
    rng = np.random.default_rng(12)
    sigma = rng.normal(size=len(bv))
    mu = rng.normal(size=len(bv))
    wmu = rng.normal(size=len(wv))
    c = bv.reshape(-1, 3, 3).mean(axis=1)
    pts = np.concatenate([rng.normal(size=(300, 3)) * [1.0, 2.0, 0.3] + [0.5, 0, 0],  # near and on the surface
                          c[:50] + 1e-3, rng.normal(size=(100, 3)) * 20])              # and far away
    ref = po.panels_velocity(bv, sigma, mu, wv, wmu, pts)
    got = _np(vp.panels_velocity(_cuda(bv), _cuda(sigma), _cuda(mu), _cuda(wv), _cuda(wmu), _cuda(pts)))
    err = np.abs(got - ref).max(axis=1) / np.maximum(np.abs(ref).max(axis=1), 1.0)
    assert err.max() < 1e-10
    # body panels only
    ref = po.panels_velocity(bv, sigma, mu, np.zeros((0, 9)), np.zeros(0), pts)
    got = _np(vp.panels_velocity(_cuda(bv), _cuda(sigma), _cuda(mu), None, None, _cuda(pts)))
    err = np.abs(got - ref).max(axis=1) / np.maximum(np.abs(ref).max(axis=1), 1.0)
    assert err.max() < 1e-10


# ---- vortex-particle case ----

def _vp_wing(n_chord=8, n_span=6, taper=1.0, sweep=0.0):
    from cpanel_gb300 import wing
    spec = wing.WingSpec(m=0.04, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=taper, sweep_deg=sweep,
                         n_chord=n_chord, n_span=n_span, wake_len=10.0, wake_dir=wing.wake_dir_for(8.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    return nodes, tris[keep], ids[keep]


def test_panels_stretching_matches_oracle(built):
    from cpanel_gb300 import vp
    nodes, tris, ids = _vp_wing(10, 7)
    m = po.Mesh(nodes, tris, ids)
    bv = m.body_verts()
    T = vp.vp_topology(nodes, tris, ids)
    wv = T["w1"]
    rng = np.random.default_rng(21)
    sigma, mu, wmu = rng.normal(size=len(bv)), rng.normal(size=len(bv)), rng.normal(size=len(wv))
    c = bv.reshape(-1, 3, 3).mean(axis=1)
    pos = np.concatenate([c[::3] + rng.normal(size=(len(c[::3]), 3)) * 0.05,        # near the surface
                          rng.normal(size=(150, 3)) * [2.0, 2.0, 0.5] + [1.2, 0, 0],  # near the buffer wake
                          rng.normal(size=(50, 3)) * 10])                            # far field
    st = rng.normal(size=pos.shape) * 0.01
    ref = po.panels_stretching(bv, sigma, mu, wv, wmu, pos, st)
    got = _np(vp.panels_stretching(_cuda(bv), _cuda(sigma), _cuda(mu), _cuda(wv), _cuda(wmu), _cuda(pos), _cuda(st)))
    scale = np.maximum(np.abs(ref).max(axis=1), 1e-6)
    assert (np.abs(got - ref).max(axis=1) / scale).max() < 1e-9


def test_vp_matrices_match_oracle(built):
    from cpanel_gb300 import vp
    nodes, tris, ids = _vp_wing(10, 7, 0.7, 10.0)
    S = po.VPCase(nodes, tris, ids, V=1.0, alpha=8.0)
    G = vp.VPCase(nodes, tris, ids, V=1.0, alpha=8.0)
    Ao, Bo, Co = S.matrices()
    Ag, Bg, Cg = G.matrices()
    for X, Y in ((Ag, Ao), (Bg, Bo), (Cg, Co)):
        assert np.abs(X - Y).max() <= 1e-12 * np.abs(Y).max()


@pytest.mark.parametrize("accelerate", [True, False])
def test_vp_time_loop_matches_oracle(built, accelerate):
    """Nine steps of cpCaseVP::run: shedding order exact, state to 1e-9 relative."""
    from cpanel_gb300 import vp
    nodes, tris, ids = _vp_wing(8, 6)
    S = po.VPCase(nodes, tris, ids, V=1.0, alpha=8.0, accelerate=accelerate)
    G = vp.VPCase(nodes, tris, ids, V=1.0, alpha=8.0, accelerate=accelerate)
    for step in range(9):
        S.step()
        G.step()
        po_, pg = S.particles(), G.particles()
        assert len(pg["pos"]) == len(po_["pos"])
        assert np.array_equal(pg["shed_time"], po_["shed_time"]) and np.array_equal(pg["parent"], po_["parent"])
        if len(po_["pos"]):
            for key in ("pos", "strength", "radius"):
                ref = po_[key]
                assert np.abs(pg[key] - ref).max() <= 1e-9 * max(np.abs(ref).max(), 1e-12), (step, key)
        so, sg = S.strengths(), G.strengths()
        for key in ("sigma", "mu", "mu_w1", "mu_w2"):
            assert np.abs(sg[key] - so[key]).max() <= 1e-9 * max(np.abs(so[key]).max(), 1e-12), (step, key)


def test_vp_trefftz_and_early_stop_match_oracle(built):
    """Trefftz plane of the particle row (wake::trefftzPlaneVP) after every step, and the
    convergence stop of cpCaseVP::solutionConvergence at the same step."""
    from cpanel_gb300 import vp, wing
    spec = wing.WingSpec(m=0.0, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=1.0, sweep_deg=0.0, n_chord=6,
                         n_span=4, wake_len=10.0, wake_dir=wing.wake_dir_for(4.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    tris, ids = tris[keep], ids[keep]
    S = po.VPCase(nodes, tris, ids, V=1.0, alpha=4.0, Sref=info["area"], mach=0.2)
    G = vp.VPCase(nodes, tris, ids, V=1.0, alpha=4.0, Sref=info["area"], mach=0.2)
    for step in range(70):
        ts_o, ts_g = S.step(), G.step()
        assert ts_o == ts_g
        to, tg = S.trefftz(), G.trefftz()
        assert tg["converged"] == to["converged"], step
        for key in ("CL", "CD"):
            assert abs(tg[key] - to[key]) <= 1e-9 * max(abs(to[key]), 1e-12), (step, key)
    assert to["converged"] and S.info()["timestep"] < 70
    assert G.info()["timestep"] == S.info()["timestep"]


# ---- mixed precision: FP32 far field, FP64 near field, same decisions ----
MIXED_TOL = 1e-5  # max |mixed - FP64| / max |FP64|, per output


@pytest.mark.parametrize("clustered", [False, True])
def test_barnes_hut_mixed_precision(built, clustered):
    from cpanel_gb300 import vp
    pos, st, rad = _cloud(5000, 31, clustered)
    if not clustered:
        pos *= 0.3
    tree = vp.ParticleFMM(_cuda(pos), _cuda(st), _cuda(rad))
    ref = [_np(x) for x in tree.barnesHut()]
    rng = np.random.default_rng(32)
    pts = _cuda(np.concatenate([rng.normal(size=(800, 3)), pos[:10]]))
    ref_pts = _np(tree.barnesHutVel(pts))
    tree.set_precision("mixed")
    got = [_np(x) for x in tree.barnesHut()]
    for r, g in zip(ref, got):
        assert _rel(g, r) < MIXED_TOL
        assert _rel(g, r) > 0 or np.abs(r).max() == 0  # the far field did run in FP32
    assert _rel(_np(tree.barnesHutVel(pts)), ref_pts) < MIXED_TOL
    # single outputs take the same decisions
    assert _rel(_np(tree.barnesHutStretch()), ref[1]) < MIXED_TOL


def test_panel_operators_mixed_precision(built):
    from cpanel_gb300 import vp
    nodes, tris, ids = _vp_wing(10, 7)
    m = po.Mesh(nodes, tris, ids)
    bv = m.body_verts()
    T = vp.vp_topology(nodes, tris, ids)
    wv = T["w1"]
    rng = np.random.default_rng(41)
    sigma, mu, wmu = rng.normal(size=len(bv)), rng.normal(size=len(bv)), rng.normal(size=len(wv))
    c = bv.reshape(-1, 3, 3).mean(axis=1)
    pos = np.concatenate([c[::3] + rng.normal(size=(len(c[::3]), 3)) * 0.05,
                          rng.normal(size=(3000, 3)) * [3.0, 2.0, 0.5] + [2.0, 0, 0],
                          rng.normal(size=(500, 3)) * 10])
    st = rng.normal(size=pos.shape) * 0.01
    args = (_cuda(bv), _cuda(sigma), _cuda(mu))
    for wverts, wm in ((None, None), (m.wake_verts(), rng.normal(size=len(m.wake_verts())))):
        w = (None, None) if wverts is None else (_cuda(wverts), _cuda(wm))
        ref = _np(vp.panels_velocity(*args, *w, _cuda(pos)))
        got = _np(vp.panels_velocity(*args, *w, _cuda(pos), precision="mixed"))
        assert 0 < _rel(got, ref) < MIXED_TOL
    ref = _np(vp.panels_stretching(*args, _cuda(wv), _cuda(wmu), _cuda(pos), _cuda(st)))
    got = _np(vp.panels_stretching(*args, _cuda(wv), _cuda(wmu), _cuda(pos), _cuda(st), precision="mixed"))
    assert 0 < _rel(got, ref) < MIXED_TOL


def test_vp_mixed_velocities_and_loop(built):
    """Particle velocities of one state in both precisions (and against the FP64 direct
    sum), then the mixed loop against the FP64 loop: same shedding, close states."""
    from cpanel_gb300 import vp
    nodes, tris, ids = _vp_wing(8, 6)
    P = vp.VPCase(nodes, tris, ids, V=1.0, alpha=8.0)
    M = vp.VPCase(nodes, tris, ids, V=1.0, alpha=8.0, precision="mixed")
    for step in range(14):
        P.step()
        M.step()
    vp64 = P.velocities("plain")
    vp32 = P.velocities("mixed")
    vdir = P.velocities("plain", direct=True)
    assert _rel(vp32, vp64) < MIXED_TOL
    per = np.linalg.norm(vp32 - vp64, axis=1) / np.linalg.norm(vp64, axis=1)
    assert per.max() < MIXED_TOL
    assert _rel(vdir, vp64) < 1e-2  # the octree's own approximation, for scale
    pp, pm = P.particles(), M.particles()
    assert np.array_equal(pp["shed_time"], pm["shed_time"]) and np.array_equal(pp["parent"], pm["parent"])
    assert _rel(pm["pos"], pp["pos"]) < 1e-6
    assert _rel(pm["strength"], pp["strength"]) < 1e-4
    sp, sm = P.strengths(), M.strengths()
    assert _rel(sm["mu"], sp["mu"]) < 1e-5
    assert M.info()["solve_fallbacks"] == 0
    tp, tm = P.trefftz(), M.trefftz()
    assert abs(tm["CL"] - tp["CL"]) <= 1e-5 * abs(tp["CL"])


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_vp_case_matches_reference_steady_test(built, precision):
    """The GPU vortex-particle case on the reference's own Connor Cases/steadyTest (40 steps,
    Barnes-Hut): particle counts and shedding steps exact; particle positions and strengths,
    body doublets and sources at the kept steps, and the final Cp, velocity and potential
    per panel within the reference's 6 printed digits; the surface-integrated coefficients
    within its 5 printed decimals.  The mixed form is held to the same digits plus its own
    arithmetic error, 5e-8 of each array's largest value (tiny strength components, 1e-4 of the
    largest, carry it above half a printed digit)."""
    from cpanel_gb300 import vp
    from test_vp_pin import FIX, check_against_fixture, check_surface, run_case
    fix = np.load(FIX)

    def gpu_case(f):
        return vp.VPCase(f["nodes"], f["tris"], f["ids"], V=float(f["V"]), alpha=float(f["alpha"]),
                         beta=float(f["beta"]), dt=float(f["dt"]), cref=float(f["cref"]),
                         accelerate=bool(f["accelerate"]), Sref=float(f["Sref"]), mach=float(f["mach"]),
                         precision=precision)

    slack = 5e-8 if precision == "mixed" else 0.0
    run = run_case(gpu_case, fix)
    check_against_fixture(run, fix, slack)
    sf = run["case"].surface(cg=fix["cg"], bref=float(fix["bref"]), cref=float(fix["cref"]))
    check_surface(sf, fix, slack)
