"""Seeded synthetic NACA 4-digit wings written as Cart3D .tri arrays.

CPanel reads meshes from OpenVSP-style .tri files (CPanel/geometry.cpp:132-629); no
synthetic meshes ship with it, so this module builds them.  The layout follows the
conventions readTri relies on:

* body triangles first (surface id 1), wake triangles last (id 1001);
* wake nodes are appended after every body node, with the trailing-edge nodes
  duplicated so that geometry::correctWakeConnectivity merges them
  (CPanel/geometry.cpp:218-244,631-667);
* triangles are ordered (p0,p1,p2) with (p1-p0)x(p2-p0) pointing out of the body
  (panel::setGeom, CPanel/panel.cpp:53-61);
* the trailing edge is closed (thickness coefficient -0.1036) so upper and lower
  trailing-edge nodes coincide and share one node;
* closed tips pair the upper and lower nodes of each chord station: a strip of
  quads between consecutive stations, each split on its shorter diagonal, with one
  triangle at the leading and one at the trailing edge (no added node).  A fan from
  a centroid node would put long slivers (area/longSide^2 ~ 1e-3) beside the
  cosine-clustered trailing edge, whose CHTLS fits turn 1e-10 changes of the
  doublet strengths into Cp changes of order 0.1.

Each quad between two span stations is split on one fixed diagonal.  Every wake
trailing-edge quad sheds one flat quad of `wake_len` chords along `wake_dir`.

Every node carries a seeded jitter of 1e-4 of its local spacing.  Without it the strips of an
untwisted wing and the caps are exactly planar, and two reference heuristics
that real OpenVSP meshes never trip on a wing surface would fire: the on-edge
branch of panel::vortexPhi (CPanel/panel.cpp:722-733) for exactly coplanar
target/source pairs (doublet row sums then miss -1 by up to 0.5), and the
tip-patch test of bodyPanel::setTipFlag (CPanel/bodyPanel.cpp:58-95).
"""
import math
from dataclasses import dataclass

import numpy as np


@dataclass
class WingSpec:
    m: float = 0.0          # max camber (fraction of chord)
    p: float = 0.4          # camber position
    t: float = 0.12         # thickness
    root_chord: float = 1.0
    span: float = 4.0       # tip to tip
    taper: float = 1.0
    sweep_deg: float = 0.0  # leading-edge sweep
    n_chord: int = 40       # points per side, leading and trailing edge shared
    n_span: int = 25        # span stations
    wake_len: float = 30.0  # in root chords
    wake_dir: tuple = (1.0, 0.0, 0.0)
    tips: bool = True
    jitter: float = 1e-4    # seeded node jitter, as a fraction of the local node spacing
    seed: int = 0


def naca4_surface(m, p, t, x):
    """Upper and lower (x, z) of a NACA 4-digit section with a closed trailing edge."""
    yt = 5 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3 - 0.1036 * x ** 4)
    if m > 0:
        yc = np.where(x < p, m / p ** 2 * (2 * p * x - x ** 2), m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * x - x ** 2))
        dyc = np.where(x < p, 2 * m / p ** 2 * (p - x), 2 * m / (1 - p) ** 2 * (p - x))
    else:
        yc = np.zeros_like(x)
        dyc = np.zeros_like(x)
    th = np.arctan(dyc)
    xu, zu = x - yt * np.sin(th), yc + yt * np.cos(th)
    xl, zl = x + yt * np.sin(th), yc - yt * np.cos(th)
    return xu, zu, xl, zl


def make_wing(spec: WingSpec):
    """Return (nodes[n,3] float64, tris[nt,3] int64 1-based, ids[nt] int32, info dict)."""
    N, S = spec.n_chord, spec.n_span
    x = 0.5 * (1 - np.cos(np.pi * np.arange(N) / (N - 1)))
    xu, zu, xl, zl = naca4_surface(spec.m, spec.p, spec.t, x)
    # ring: upper TE -> LE (i = N-1 .. 0), then lower i = 1 .. N-2 (lower TE == upper TE)
    rx = np.concatenate([xu[::-1], xl[1:N - 1]])
    rz = np.concatenate([zu[::-1], zl[1:N - 1]])
    rx[0], rz[0] = 1.0, 0.0 + (zu[-1] + zl[-1]) * 0.5
    R = len(rx)  # 2(N-1)
    half = spec.span / 2
    ys = np.linspace(-half, half, S)
    tan_sw = math.tan(math.radians(spec.sweep_deg))
    nodes = []
    for y in ys:
        eta = abs(y) / half
        c = spec.root_chord * (1 - (1 - spec.taper) * eta)
        xle = abs(y) * tan_sw
        for k in range(R):
            nodes.append((xle + c * rx[k], y, c * rz[k]))
    nodes = np.array(nodes, dtype=np.float64)
    node = lambda j, k: j * R + (k % R)
    rng = np.random.default_rng(spec.seed)
    if spec.jitter > 0:
        # break the exact coplanarity of the ruled surface strips: each node moves by
        # up to `jitter` times its shortest distance to a ring or span neighbour
        P = nodes.reshape(S, R, 3)
        dk = np.minimum(np.linalg.norm(P - np.roll(P, 1, axis=1), axis=2),
                        np.linalg.norm(P - np.roll(P, -1, axis=1), axis=2))
        dy = np.full((S, R), np.inf)
        dy[1:] = np.minimum(dy[1:], np.linalg.norm(P[1:] - P[:-1], axis=2))
        dy[:-1] = np.minimum(dy[:-1], np.linalg.norm(P[1:] - P[:-1], axis=2))
        h = np.minimum(dk, dy).reshape(-1, 1)
        nodes = nodes + spec.jitter * h * rng.uniform(-1, 1, nodes.shape)
    tris = []
    for j in range(S - 1):
        # each span strip lists its ring from the trailing edge over the lower side first, so the
        # first triangle that names a trailing-edge edge is the lower one, as in the OpenVSP meshes
        # of the reference's cases: the vortex-particle buffer wake takes its upper/lower panels
        # from that edge's node order (edge::checkTE against the buffer quads' normals)
        for k in reversed(range(R)):
            a, b = node(j, k), node(j, k + 1)
            c, d = node(j + 1, k + 1), node(j + 1, k)
            tris.append((a, d, c))
            tris.append((a, c, b))
    n_surf = len(tris)
    if spec.tips:
        for j, right in ((0, False), (S - 1, True)):
            for t in _cap_triangles(nodes, [node(j, k) for k in range(R)], N):
                # outward: +y on the right tip, -y on the left
                p0, p1, p2 = nodes[t[0]], nodes[t[1]], nodes[t[2]]
                ny = np.cross(p1 - p0, p2 - p0)[1]
                tris.append(t if (ny > 0) == right else (t[0], t[2], t[1]))
    n_body = len(tris)
    ids = [1] * n_body
    # wake: duplicated TE nodes then the downstream nodes (appended after body nodes)
    if spec.wake_len > 0:
        d = np.asarray(spec.wake_dir, dtype=np.float64)
        d = d / np.linalg.norm(d)
        te = np.array([nodes[node(j, 0)] for j in range(S)])
        base = len(nodes)
        far = te + spec.wake_len * spec.root_chord * d
        nodes = np.vstack([nodes, te, far])
        for j in range(S - 1):
            t0, t1 = base + j, base + j + 1
            f0, f1 = base + S + j, base + S + j + 1
            tris.append((t0, f0, f1))
            tris.append((t0, f1, t1))
            ids += [1001, 1001]
    tris = np.array(tris, dtype=np.int64) + 1
    info = dict(n_body=n_body, n_surface=n_surf, n_wake=len(tris) - n_body, n_te=S - 1,
                span=spec.span, area=_planform_area(spec))
    return nodes, tris, np.array(ids, dtype=np.int32), info


def _cap_triangles(nodes, ring, N):
    """Triangles closing one tip section: upper and lower nodes of the same chord station are
    paired, so the cap is a strip of quads between consecutive stations (each split on its
    shorter diagonal) with one triangle at the leading and one at the trailing edge.  ring
    lists the section's node indices from the trailing edge over the upper side to the
    leading edge (position N - 1) and back over the lower side."""
    up = [ring[N - 1 - i] for i in range(N)]               # chord station i, 0 = leading edge
    lo = [ring[N - 1]] + [ring[N - 1 + i] for i in range(1, N - 1)] + [ring[0]]
    out = [(up[0], up[1], lo[1])]
    for i in range(1, N - 2):
        a, b, c, d = up[i], up[i + 1], lo[i + 1], lo[i]
        if np.linalg.norm(nodes[a] - nodes[c]) <= np.linalg.norm(nodes[b] - nodes[d]):
            out += [(a, b, c), (a, c, d)]
        else:
            out += [(a, b, d), (b, c, d)]
    out.append((up[N - 2], up[N - 1], lo[N - 2]))
    return out


def _planform_area(spec):
    return spec.span * spec.root_chord * (1 + spec.taper) / 2


def wake_dir_for(alpha_deg, beta_deg=0.0):
    """Freestream direction in body axes (cpCase::windToBody, CPanel/cpCase.cpp:142-165)."""
    a, b = math.radians(alpha_deg), math.radians(beta_deg)
    return (math.cos(a) * math.cos(b), -math.sin(b), math.sin(a) * math.cos(b))


def config_small_steady():
    """Rectangular NACA 0012 wing, chord 1, span 4, 40 points per side, 25 stations,
    wake 30 chords along Vinf at alpha = 5 deg."""
    return WingSpec(m=0.0, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=1.0, sweep_deg=0.0, n_chord=40,
                    n_span=25, wake_len=30.0, wake_dir=wake_dir_for(5.0))


def config_multi_rhs():
    """NACA 4412 tapered wing: AR 6, root chord 1, taper 0.6, no sweep, 80 points per
    side, 61 stations (about 19.3k triangles); wake fixed along +x body axis so one
    matrix serves all 17 angles of attack."""
    taper = 0.6
    span = 6 * 1.0 * (1 + taper) / 2  # AR = b^2/S with S = b*c_r*(1+taper)/2
    return WingSpec(m=0.04, p=0.4, t=0.12, root_chord=1.0, span=span, taper=taper, sweep_deg=0.0, n_chord=80,
                    n_span=61, wake_len=30.0, wake_dir=(1.0, 0.0, 0.0))


def config_random(seed):
    """One wing of the uneven batch: seeded NACA section and planform."""
    rng = np.random.default_rng(seed)
    m = rng.uniform(0, 0.06)
    p = rng.uniform(0.2, 0.5)
    t = rng.uniform(0.08, 0.18)
    ar = rng.uniform(3, 10)
    taper = rng.uniform(0.3, 1.0)
    sweep = rng.uniform(0, 35)
    for _ in range(100):
        nc = int(rng.integers(20, 101))
        ns = int(rng.integers(15, 61))
        ntri = 4 * (nc - 1) * (ns - 1) + 2 * (2 * nc - 4)
        if 1000 <= ntri <= 12000:
            break
    span = ar * 1.0 * (1 + taper) / 2
    return WingSpec(m=m, p=p, t=t, root_chord=1.0, span=span, taper=taper, sweep_deg=sweep, n_chord=nc, n_span=ns,
                    wake_len=30.0, wake_dir=(1.0, 0.0, 0.0))
