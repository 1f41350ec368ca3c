"""Off-body streamlines (streamline::streamline / rkf, CPanel/streamline.cpp:20-78): the library's
lockstep integrator against the oracle's one-line-at-a-time restatement.  Host only: the velocity
field is an analytic one passed through the C ABI's callback; the panel field on the device is
covered in tests/test_gpu_parity.py."""
import numpy as np
import pytest

from oracle import pyoracle as po


@pytest.fixture(scope="module")
def cg(built):
    import cpanel_gb300
    return cpanel_gb300


def rankine(U=1.0, Q=0.4, c=(0.3, 0.0, 0.0)):
    """Uniform flow U along x plus a point source of strength Q at c (a Rankine half-body)."""
    c = np.asarray(c, dtype=np.float64)

    def f(p):
        p = np.asarray(p, dtype=np.float64).reshape(-1, 3)
        r = p - c
        d = np.linalg.norm(r, axis=1, keepdims=True)
        v = Q / (4 * np.pi) * r / d ** 3
        v[:, 0] += U
        return v
    return f


STARTS = np.array([[-1.0, 0.05, 0.02], [-1.0, -0.2, 0.1], [-0.8, 0.0, 0.3], [-1.2, 0.4, -0.25]])


def test_matches_oracle_line_by_line(cg):
    """Every line's points and velocities equal the oracle's sequential integration of that line."""
    f = rankine()
    lines, ended = cg.streamlines_field(f, 1.0, STARTS, x_max=2.0, tol=1e-5, max_points=2000)
    assert ended.all()
    for (p, v), s in zip(lines, STARTS):
        op, ov, oe = po.streamline(lambda q: f(q)[0], s, 1.0, 2.0, 1e-5, 2000)
        assert oe
        assert p.shape == op.shape and len(p) >= 5
        np.testing.assert_allclose(p, op, rtol=0, atol=1e-12)
        np.testing.assert_allclose(v, ov, rtol=0, atol=1e-12)
        assert p[-1, 0] < 2.0  # the last step start is before x_max; the step from it ends past it


def test_lines_are_independent_of_their_batch(cg):
    """Advancing lines together changes nothing: each line alone gives the same bits."""
    f = rankine()
    together, _ = cg.streamlines_field(f, 1.0, STARTS, x_max=1.5, tol=1e-4, max_points=500)
    for i, s in enumerate(STARTS):
        alone, _ = cg.streamlines_field(f, 1.0, s[None], x_max=1.5, tol=1e-4, max_points=500)
        assert alone[0][0].tobytes() == together[i][0].tobytes()
        assert alone[0][1].tobytes() == together[i][1].tobytes()


def test_uniform_flow_steps_are_exact(cg):
    """In a uniform stream the error estimate is zero, so the step keeps its first size 0.1 / |V|."""
    V = np.array([2.0, 0.0, 0.5])
    lines, ended = cg.streamlines_field(lambda p: np.tile(V, (len(p), 1)), np.linalg.norm(V),
                                        [[0.0, 0.0, 0.0]], x_max=1.0, tol=1e-4, max_points=100)
    p, v = lines[0]
    dt = 0.1 / np.linalg.norm(V)
    assert ended[0]
    assert np.allclose(p, np.arange(len(p))[:, None] * dt * V, atol=1e-13)
    assert p[-1, 0] < 1.0 <= p[-1, 0] + dt * V[0] + 1e-12
    assert np.allclose(v, V)


def test_max_points_cuts_a_line_short(cg):
    """A line out of room stops with ended False; its points are the first ones of the full line."""
    f = rankine()
    full, e_full = cg.streamlines_field(f, 1.0, STARTS[:2], x_max=2.0, tol=1e-5, max_points=2000)
    short, e_short = cg.streamlines_field(f, 1.0, STARTS[:2], x_max=2.0, tol=1e-5, max_points=7)
    assert e_full.all() and not e_short.any()
    for (p, v), (pf, vf) in zip(short, full):
        assert len(p) == 7
        assert p.tobytes() == pf[:7].tobytes() and v.tobytes() == vf[:7].tobytes()
    op, ov, oe = po.streamline(lambda q: f(q)[0], STARTS[0], 1.0, 2.0, 1e-5, 7)
    assert not oe and len(op) == 7


def test_errors_reach_the_caller(cg):
    """A failing velocity field stops the integration and its exception reaches the caller; bad
    arguments are refused."""
    def bad(p):
        raise ValueError("field failed")
    with pytest.raises(ValueError, match="field failed"):
        cg.streamlines_field(bad, 1.0, STARTS, x_max=2.0)
    with pytest.raises(cg.CpgError):
        cg.streamlines_field(rankine(), 0.0, STARTS, x_max=2.0)
    with pytest.raises(cg.CpgError):
        cg.streamlines_field(rankine(), 1.0, STARTS, x_max=2.0, tol=0.0)
    lines, ended = cg.streamlines_field(rankine(), 1.0, np.zeros((0, 3)), x_max=2.0)
    assert lines == [] and len(ended) == 0


def test_streamlines_vtu_round_trip(cg, tmp_path):
    """streamlines.vtu as cpCase::writeBodyStreamlines lays it out: one piece per line, its points
    with point data Velocity and line cells (j, j + 1), read back at the printed precision."""
    from cpanel_gb300 import io
    lines, _ = cg.streamlines_field(rankine(), 1.0, STARTS, x_max=2.0, tol=1e-5, max_points=2000)
    path = str(tmp_path / "streamlines.vtu")
    io.write_streamlines_vtu(path, lines)
    pieces = io.read_vtu_pieces(path)
    assert len(pieces) == len(lines)
    for d, (p, v) in zip(pieces, lines):
        k = len(p)
        assert np.allclose(d["Position"], p, rtol=1e-5, atol=1e-6)
        assert np.allclose(d["Velocity"], v, rtol=1e-5, atol=1e-6)
        assert d["connectivity"].tolist() == [q for j in range(k - 1) for q in (j, j + 1)]
        assert d["offsets"].tolist() == [2 * (j + 1) for j in range(k - 1)]
        assert d["types"].tolist() == [3] * (k - 1)
    from cpanel_gb300._lib import I32
    bad = np.array([5], dtype=np.int32)  # more points than max_points: refused before the file is opened
    assert cg._lib.load().cpg_write_streamlines_vtu(path.encode(), None, None, bad.ctypes.data_as(I32), 1, 2) == 1
