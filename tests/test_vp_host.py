"""Vortex-particle operators, host side (no GPU).

- The oracle's pair kernels against an independent numpy/scipy restatement of
  CPanel/particle.cpp:31-140 and against the singular Biot-Savart limit.
- The reference's own octree tests (octree/tests/octree_test.cpp:47-362), ported to
  the oracle's insertion-order tree.
- The product's host octree builder (recursive partition) against the oracle's
  insertion-order tree, bit for bit, including clustered and coincident points.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

CORE = 1.5  # particle::coreOverlap, CPanel/particle.h:32
NU = 1.983e-5  # CPanel/particle.cpp:126


def _np_K(rho):
    from scipy.special import erf
    return (1 / (4 * np.pi * rho) * erf(rho / np.sqrt(2)) - 1 / (2 * np.pi) ** 1.5 * np.exp(-0.5 * rho * rho)) / rho**2


def _np_vel_poi(pos, st, rad, pts):
    """particle::velInfl(POI), CPanel/particle.cpp:60-77, summed over all particles."""
    out = np.zeros((len(pts), 3))
    for j in range(len(pos)):
        d = pts - pos[j]
        r = np.linalg.norm(d, axis=1)
        sig = CORE * rad[j]
        with np.errstate(divide="ignore", invalid="ignore"):
            v = (-1 / sig**3 * _np_K(r / sig))[:, None] * np.cross(d, st[j])
        v[r == 0] = 0
        out += v
    return out


def _np_vel_alg(pos, st, rad, pts):
    """particle::velInflAlgSmooth, CPanel/particle.cpp:31-38."""
    out = np.zeros((len(pts), 3))
    for j in range(len(pos)):
        d = pts - pos[j]
        r = np.linalg.norm(d, axis=1)
        sig = CORE * rad[j]
        f = -1 / (4 * np.pi) * (r**2 + 2.5 * sig**2) / (r**2 + sig**2) ** 2.5
        out += f[:, None] * np.cross(d, st[j])
    return out


def _np_stretch_diff(pos, st, rad):
    """cpCaseVP.cpp:504-516: particles[i]->vortexStretching(particles[j]) and viscousDiffusion."""
    n = len(pos)
    S = np.zeros((n, 3))
    Dv = np.zeros((n, 3))
    for i in range(n):
        for j in range(n):
            if i == j:
                continue
            d = pos[i] - pos[j]
            dn = np.linalg.norm(d)
            sig = np.sqrt((CORE * rad[i]) ** 2 + (CORE * rad[j]) ** 2) / np.sqrt(2)
            rho = dn / sig
            Vi, Vj = 4 * np.pi / 3 * rad[i] ** 3, 4 * np.pi / 3 * rad[j] ** 3
            xi_d = 1 / ((2 * np.pi) ** 1.5 * rho**3) * np.exp(-rho * rho / 2)
            Dv[i] += 2 * NU / sig**2 * xi_d * (Vi * st[j] - Vj * st[i])
            if dn > 5 * rad[i]:
                continue
            from scipy.special import erf
            xi = 1 / (2 * np.pi) ** 1.5 * np.exp(-rho * rho / 2)
            G = 1 / (4 * np.pi * rho) * erf(rho / np.sqrt(2))
            K = (G - xi) / rho**2
            F = (3 * K - xi) / rho**2
            M = K * np.eye(3) - 1 / sig**2 * F * np.outer(d, d)
            a = st[j]
            At = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
            S[i] += (1 / sig**3 * At @ M) @ st[i]
    return S, Dv


@pytest.fixture(scope="module")
def cloud():
    rng = np.random.default_rng(11)
    n = 150
    pos = rng.normal(size=(n, 3)) * 0.3
    st = rng.normal(size=(n, 3)) * 0.01
    rad = rng.uniform(0.02, 0.08, n)
    pts = np.concatenate([rng.normal(size=(40, 3)) * 0.5, pos[:5]])  # includes on-particle points
    return pos, st, rad, pts


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_oracle_pair_kernels_match_numpy_restatement(cloud):
    pos, st, rad, pts = cloud
    assert _rel(po.particles_velocity(pos, st, rad, pts, kernel="gauss"), _np_vel_poi(pos, st, rad, pts)) < 1e-12
    assert _rel(po.particles_velocity(pos, st, rad, pts, kernel="alg"), _np_vel_alg(pos, st, rad, pts)) < 1e-12
    S, Dv = _np_stretch_diff(pos, st, rad)
    assert _rel(po.particles_stretch(pos, st, rad), S) < 1e-12
    assert _rel(po.particles_diffusion(pos, st, rad), Dv) < 1e-12


def test_kernels_tend_to_biot_savart_far_away():
    # K(rho) -> 1/(4 pi rho^3): u -> -(d x alpha)/(4 pi |d|^3) for both smoothings
    pos = np.zeros((1, 3))
    st = np.array([[0.0, 0.0, 1.0]])
    rad = np.array([1e-3])
    pts = np.array([[50.0, 0.0, 0.0], [0.0, 30.0, 0.0], [10.0, 20.0, 5.0]])
    d = pts - pos[0]
    bs = -np.cross(d, st[0]) / (4 * np.pi * np.linalg.norm(d, axis=1)[:, None] ** 3)
    for k in ("gauss", "alg"):
        assert _rel(po.particles_velocity(pos, st, rad, pts, kernel=k), bs) < 1e-9


def test_self_term_is_zero_at_the_particle():
    pos = np.array([[0.1, 0.2, 0.3]])
    st = np.array([[1.0, 2.0, 3.0]])
    v = po.particles_velocity(pos, st, np.array([0.05]), pos, kernel="gauss")
    assert np.all(v == 0)


# ---- reference octree tests (octree/tests/octree_test.cpp), on the oracle's tree ----

def _grid():
    return np.array([[i, j, k] for i in range(3) for j in range(3) for k in range(3)], dtype=float)


def _tree(pos, max_members=10):
    pos = np.asarray(pos, dtype=float)
    return po.ParticleTree(pos, np.ones_like(pos), np.full(len(pos), 0.1), max_members=max_members)


def test_octree_construction_root():
    # OctreeTest.AddData (:305-333): root origin (1,1,1), no parent; half = 0.51 x extent
    t = _tree(_grid())
    nd = t.nodes()
    assert np.all(nd[0, 0:3] == 1.0)
    assert np.all(nd[0, 3:6] == 0.51 * 2.0)
    assert nd[0, 6] == 1  # OctreeNodeTest.Construction: level 1
    assert len(t.leaf_members()) == 27


def test_octree_add_member_splits_after_max():
    # OctreeNodeTest.AddMember (:78-113): leaf while count <= maxMembers, split after
    g = _grid()
    for k in range(1, 28):
        t = _tree(g[:k])
        nd = t.nodes()
        assert bool(nd[0, 7]) == (k <= 10), k
        assert sorted(t.leaf_members()) == list(range(k))
        assert int(nd[nd[:, 7] == 1, 8].sum()) == k


def test_octree_child_containing_point():
    # OctreeNodeTest.NodeContainingMember (:115-187): corner points around the root
    # origin land in children 0..7 (x>o: 4, y>o: 2, z>o: 1)
    g = _grid()
    corners = []
    for c in range(8):
        corners.append([1 + (1 if c & 4 else -1), 1 + (1 if c & 2 else -1), 1 + (1 if c & 1 else -1)])
    pts = np.concatenate([g, np.array(corners, dtype=float)])
    t = _tree(pts)
    nd = t.nodes()
    children = nd[0, 16:24].astype(int)
    members = t.leaf_members()
    # walk the pre-order table: members of the subtree of each root child
    leaf_rows = np.where(nd[:, 7] == 1)[0]
    offsets = np.concatenate([[0], np.cumsum(nd[leaf_rows, 8].astype(int))])
    owner = {}
    for li, row in enumerate(leaf_rows):
        for p in members[offsets[li]:offsets[li + 1]]:
            owner[int(p)] = row
    skip = {}
    for c in range(8):
        ci = children[c]
        if ci < 0:
            continue
        nxt = [children[k] for k in range(c + 1, 8) if children[k] >= 0]
        skip[c] = (ci, nxt[0] if nxt else len(nd))
    for c in range(8):
        lo, hi = skip[c]
        assert lo <= owner[27 + c] < hi, c


def test_octree_levels_and_expansions():
    # particleFMM::computeMultExp: every non-root node has an expansion with
    # strength = sum of member strengths and radius |half|*2*1.5
    rng = np.random.default_rng(3)
    pos = rng.normal(size=(500, 3))
    st = rng.normal(size=(500, 3))
    t = po.ParticleTree(pos, st, np.full(500, 0.05))
    nd = t.nodes()
    members = t.leaf_members()
    assert t.n_levels == int(nd[:, 6].max())
    leaf_rows = np.where(nd[:, 7] == 1)[0]
    off = 0
    for row in leaf_rows:
        k = int(nd[row, 8])
        if row > 0:
            ms = members[off:off + k]
            assert np.allclose(nd[row, 12:15], st[ms].sum(axis=0), rtol=1e-13, atol=1e-13)
            w = np.linalg.norm(st[ms], axis=1)
            assert np.allclose(nd[row, 9:12], (pos[ms] * w[:, None]).sum(0) / w.sum(), rtol=1e-12, atol=1e-12)
        off += k
    assert np.allclose(nd[1:, 15], np.linalg.norm(nd[1:, 3:6], axis=1) * 3.0, rtol=1e-15)


def test_barnes_hut_returns_zero_when_root_is_a_leaf():
    # the traversal starts from the root's children (particleFMM.cpp:65-77)
    rng = np.random.default_rng(4)
    pos = rng.normal(size=(7, 3))
    t = po.ParticleTree(pos, rng.normal(size=(7, 3)), np.full(7, 0.1))
    assert np.all(t.velocity() == 0)
    assert np.all(t.velocity_points(rng.normal(size=(3, 3))) == 0)


def test_barnes_hut_tends_to_direct_as_theta_shrinks():
    rng = np.random.default_rng(5)
    pos = rng.normal(size=(400, 3))
    st = rng.normal(size=(400, 3)) * 0.01
    rad = np.full(400, 0.05)
    pts = rng.normal(size=(30, 3)) * 2
    exact = po.particles_velocity(pos, st, rad, pts, kernel="alg")
    t = po.ParticleTree(pos, st, rad, theta=1e-6)
    assert _rel(t.velocity_points(pts), exact) < 1e-12


# ---- product host builder vs the oracle's insertion-order tree ----

def _sets():
    rng = np.random.default_rng(7)
    yield "grid", _grid()
    yield "few", rng.normal(size=(5, 3))
    yield "eleven", rng.normal(size=(11, 3))
    yield "gauss3000", rng.normal(size=(3000, 3))
    yield "clustered", np.concatenate([rng.normal(size=(1000, 3)) * 0.01, rng.normal(size=(1000, 3)) + 5])
    yield "coincident", np.repeat(rng.normal(size=(20, 3)), 20, axis=0)  # reaches the level cap
    yield "flat", np.c_[rng.uniform(size=(800, 2)), np.zeros(800)]  # zero extent in z


@pytest.mark.parametrize("name,pos", list(_sets()), ids=[n for n, _ in _sets()])
def test_product_tree_matches_oracle_bit_for_bit(built, name, pos):
    from cpanel_gb300 import vp
    rng = np.random.default_rng(len(pos))
    st = rng.normal(size=pos.shape)
    rad = rng.uniform(0.01, 0.1, len(pos))
    for mm in (10, 3):
        t = po.ParticleTree(pos, st, rad, max_members=mm)
        nodes, members, info = vp.host_tree(pos, st, rad, max_members=mm)
        assert info["n_nodes"] == t.n_nodes and info["n_levels"] == t.n_levels
        assert np.array_equal(nodes, t.nodes())
        assert np.array_equal(members, t.leaf_members())


def test_dub_v_inf_single_triangle():
    # panel::dubVInf vs the body panel's doublet velocity: the same mathematics with the
    # edge vector formed differently; both agree to rounding
    v9 = np.array([1.0, 0, 0, -1, 1, 0, -1, -1, 0])
    for poi in ([2.0, 2.0, 2.0], [7.0, 7.0, 7.0], [0.1, 0.0, 0.05]):
        vs, vd = po.tri_v_inf(v9, poi)
        assert np.allclose(po.tri_dub_v_inf(v9, poi), vd, rtol=1e-12, atol=1e-15)


# ---- vortex-particle case: the buffer wake built by the product vs the oracle ----

def _vp_wing(n_chord=8, n_span=6, taper=1.0, sweep=0.0):
    from cpanel_gb300 import wing
    spec = wing.WingSpec(m=0.04, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=taper, sweep_deg=sweep,
                         n_chord=n_chord, n_span=n_span, wake_len=10.0, wake_dir=wing.wake_dir_for(8.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000  # the VP case takes a body-only mesh (CPanel/geometry.cpp:270-277)
    return nodes, tris[keep], ids[keep]


@pytest.mark.parametrize("shape", [(8, 6, 1.0, 0.0), (10, 9, 0.7, 10.0), (14, 7, 0.6, 20.0)])
def test_vp_buffer_wake_matches_oracle_bit_for_bit(built, shape):
    from cpanel_gb300 import vp
    nodes, tris, ids = _vp_wing(*shape)
    S = po.VPCase(nodes, tris, ids, V=1.0, alpha=8.0)
    w1, w2, cols, coef = S.wake()
    T = vp.vp_topology(nodes, tris, ids, V=1.0)
    assert T["dt"] == S.dt
    assert np.array_equal(T["w1"], w1) and np.array_equal(T["w2"], w2)
    assert np.array_equal(T["w1_idx"], cols) and np.array_equal(T["w1_coef"], coef)
    # one first-row and one second-row quad per trailing-edge edge, second row behind the first
    assert len(w1) == len(w2) == S.info()["n_w1"]
    assert np.all(w2.reshape(-1, 4, 3)[:, :, 0].mean(1) > w1.reshape(-1, 4, 3)[:, :, 0].mean(1))


def test_vp_mesh_with_wake_panels_is_rejected(built):
    from cpanel_gb300 import vp, wing
    spec = wing.WingSpec(m=0.0, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=1.0, sweep_deg=0.0, n_chord=8,
                         n_span=6, wake_len=10.0, wake_dir=wing.wake_dir_for(5.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    with pytest.raises(ValueError):
        po.VPCase(nodes, tris, ids)
    with pytest.raises(Exception):
        vp.vp_topology(nodes, tris, ids)


def test_vp_oracle_sheds_one_particle_per_te_edge_in_panel_order():
    nodes, tris, ids = _vp_wing()
    S = po.VPCase(nodes, tris, ids, V=1.0, alpha=8.0, accelerate=True)
    n2 = S.info()["n_w2"]
    for _ in range(6):
        S.step()
    p = S.particles()
    # steps 1-2 shed nothing; from step 3 every second-row panel sheds once per step, in order
    assert len(p["pos"]) == 4 * n2
    assert list(p["shed_time"]) == [t for t in range(3, 7) for _ in range(n2)]
    assert list(p["parent"]) == list(range(n2)) * 4
    assert np.all(np.isfinite(p["pos"])) and np.all(p["radius"] > 0)


def test_oracle_vp_converges_and_stops():
    """cpCaseVP::solutionConvergence on the oracle: no Trefftz check before step 5, the
    stop once CL and CD change by < 0.01 %, and no further steps after it."""
    from cpanel_gb300 import wing
    spec = wing.WingSpec(m=0.0, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=1.0, sweep_deg=0.0, n_chord=6,
                         n_span=4, wake_len=10.0, wake_dir=wing.wake_dir_for(4.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    S = po.VPCase(nodes, tris[keep], ids[keep], V=1.0, alpha=4.0, Sref=info["area"])
    hist = []
    for _ in range(80):
        ts = S.step()
        t = S.trefftz()
        hist.append((ts, t["CL"], t["CD"], t["converged"]))
        if t["converged"]:
            break
    ts, CL, CD, conv = hist[-1]
    assert conv and 5 < ts < 80
    assert not any(h[3] for h in hist[:-1])
    prev = hist[-2]
    assert abs(CL - prev[1]) < 1e-4 * abs(prev[1]) and abs(CD - prev[2]) < 1e-4 * abs(prev[2])
    assert S.step() == ts and S.info()["n_particles"] == 3 * (ts - 2)
