"""Request loop (include/cpanel_serve.h): admission rule on the host, and on the GPU
each request's result alone against the same request in a concurrent mix."""
import numpy as np
import pytest

from conftest import small_wing


def test_footprint_rule(built):
    from cpanel_gb300 import serve
    a = serve.footprint(10000, 8, "mixed")
    b = serve.footprint(20000, 8, "mixed")
    assert a > 12 * 10000**2 and b > 4 * (a - (256 << 20)) * 0.9
    assert serve.footprint(10000, 8, "plain") > 16 * 10000**2


def test_server_refuses_without_device_or_budget(built):
    import torch
    from cpanel_gb300 import CpgError, serve
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(CpgError):
        serve.Server(slots=2, budget_gb=1.0)


def _mix():
    out = []
    for q, (nc, ns, taper) in enumerate([(10, 6, 1.0), (14, 8, 0.6), (12, 5, 0.8), (16, 9, 0.5), (10, 7, 0.7),
                                          (18, 6, 1.0)]):
        nodes, tris, ids, info, spec = small_wing(n_chord=nc, n_span=ns, taper=taper, m=0.02 * (q % 3), seed=q)
        flows = [(1.0, -2.0 + 3.0 * j + 0.5 * q, 0.0, 0.1) for j in range(4)]
        out.append((nodes, tris, ids, flows, dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0, 0))))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "plain"])
def test_results_alone_equal_results_in_the_mix(built, precision):
    from cpanel_gb300 import serve
    reqs = _mix()
    srv = serve.Server(slots=4, budget_gb=40.0, precision=precision)
    alone = []
    for nodes, tris, ids, flows, refs in reqs:  # one at a time
        alone.append(srv.wait(srv.submit(nodes, tris, ids, flows, **refs)))
    tickets = [srv.submit(nodes, tris, ids, flows, **refs) for nodes, tris, ids, flows, refs in reqs * 2]
    mixed = [srv.wait(t) for t in tickets]
    srv.close()
    assert max(r["info"]["running_at_start"] for r in mixed) > 1  # the mix did overlap
    for q, r in enumerate(mixed):
        a = alone[q % len(reqs)]
        assert np.abs(r["cp"] - a["cp"]).max() <= 1e-12
        assert np.all(np.abs(r["CL"] - a["CL"]) <= 1e-12 * np.abs(a["CL"]) + 1e-15)
        assert np.all(np.abs(r["CDi"] - a["CDi"]) <= 1e-12 * np.abs(a["CDi"]) + 1e-15)


@pytest.mark.gpu
def test_admission_by_budget_serialises_large_requests(built):
    from cpanel_gb300 import serve
    reqs = _mix()[:3]
    big = max(serve.footprint(int(np.count_nonzero(ids <= 1000)), 4) for _, _, ids, _, _ in reqs)
    srv = serve.Server(slots=4, budget_gb=1.5 * big / 1e9)  # room for one request at a time
    tickets = [srv.submit(nodes, tris, ids, flows, **refs) for nodes, tris, ids, flows, refs in reqs]
    res = [srv.wait(t) for t in tickets]
    srv.close()
    assert all(r["info"]["running_at_start"] == 1 for r in res)
    assert all(r["info"]["status"] == 0 for r in res)


def test_footprint_rule_unsteady(built):
    from cpanel_gb300 import serve
    a = serve.footprint_vp(4000, 40, 100, "plain")
    b = serve.footprint_vp(4000, 40, 100, "mixed")
    assert a > 16 * 4000**2 + 8 * 4000 * 40 and b > a + 12 * 4000**2
    assert serve.footprint_vp(4000, 40, 200, "plain") > a


@pytest.mark.gpu
def test_unsteady_requests_alone_equal_in_the_mix(built):
    """Vortex-particle runs beside steady solves: the same particles, strengths and
    Trefftz plane as when run alone."""
    from cpanel_gb300 import serve, wing
    spec = wing.WingSpec(m=0.02, p=0.4, t=0.12, root_chord=1.0, span=4.0, taper=0.8, sweep_deg=0.0, n_chord=10,
                         n_span=6, wake_len=10.0, wake_dir=(1.0, 0.0, 0.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    tris, ids = tris[keep], ids[keep]
    steady = _mix()[:3]
    srv = serve.Server(slots=4, budget_gb=40.0, precision="mixed")
    alone = {p: srv.wait(srv.submit_vp(nodes, tris, ids, 12, alpha=6.0, Sref=info["area"], precision=p))
             for p in ("plain", "mixed")}
    tickets = []
    for p in ("plain", "mixed"):
        tickets += [srv.submit(*r[:4], **r[4]) for r in steady]
        tickets.append((p, srv.submit_vp(nodes, tris, ids, 12, alpha=6.0, Sref=info["area"], precision=p)))
    res = [(t[0], srv.wait(t[1])) if isinstance(t, tuple) else (None, srv.wait(t)) for t in tickets]
    srv.close()
    for p, r in res:
        if p is None:
            continue
        a = alone[p]
        assert r["steps"] == a["steps"] == 12 and r["n_particles"] == a["n_particles"] > 0
        assert np.abs(r["mu"] - a["mu"]).max() <= 1e-12 * np.abs(a["mu"]).max()
        assert abs(r["CL"] - a["CL"]) <= 1e-12 * abs(a["CL"]) and abs(r["CD"] - a["CD"]) <= 1e-12 * abs(a["CD"])
    assert max(r["info"]["running_at_start"] for _, r in res) > 1
    assert abs(alone["mixed"]["CL"] - alone["plain"]["CL"]) <= 1e-6 * abs(alone["plain"]["CL"])
