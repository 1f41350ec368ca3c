#!/usr/bin/env python
"""Steady solves/s of the GB300 panel path (CPanel hot path) on one or more GPUs.

Workload: NACA 4412 tapered wing, AR 6, taper 0.6, 80 cosine-spaced points per side
x 61 span stations (19,276 body triangles, 120 wake triangles), Mach 0.1, 17
angles of attack -4..12 deg on one geometry.  A step is one full sweep on the
performance (mixed) path: influence assembly, preconditioner set-up, the 17
refined solves and post-processing (CHTLS velocity, Cp, forces, Trefftz CL/CDi).
`value` counts solves (mesh x alpha) per second with the mesh tables resident on
the device; `e2e` repeats the step through the C ABI from host arrays (readTri
topology, uploads and result copies inside the timed region).

Accuracy is checked once, outside the timing, against the plain FP64 GPU path
(the reference method in FP64), whose own throughput is reported beside it.
Multi-GPU: replicas (each rank runs the full workload on its GPU), weak scaling.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import platform
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import ctypes as C
from ctypes import c_double as C_double

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALPHAS = [float(a) for a in range(-4, 13)]
MACH = 0.1
PLAIN_RUNS = 3
METRIC = "steady solves/s + p50/p99 latency at Cp err<=1e-5 vs FP64 plain GPU path"
# BiCGSTAB (Eigen semantics, tol = eps) iterations of the plain FP64 path on this
# mesh, measured on the GPU; used only by the CPU cost model below.
PLAIN_ITERS = 372


def max_over_ranks(t, dist=None, device="cuda"):
    """The slowest rank's time (every rank runs the whole workload on its own GPU: replicas,
    weak scaling); t itself on one rank."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return t
    import torch
    tt = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def workload(name="multi_rhs"):
    """multi_rhs: the benchmark wing.  mid: the same wing with 25 span stations
    (7,876 panels; matrices still larger than L2), used for profiler captures."""
    import dataclasses

    from cpanel_gb300 import wing
    spec = wing.config_multi_rhs()
    if name == "mid":
        spec = dataclasses.replace(spec, n_span=25)
    nodes, tris, ids, info = wing.make_wing(spec)
    refs = dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0.0, 0.0))
    return spec, nodes, tris, ids, info, refs


def config_dict(info, name="multi_rhs"):
    stations = {"multi_rhs": 61, "mid": 25}[name]
    return {"workload": "NACA4412 tapered AR6 wing, 80 pts/side x %d stations, 17 alphas (-4..12 deg)" % stations,
            "body_panels": info["n_body"], "wake_panels": info["n_wake"], "alphas": len(ALPHAS), "mach": MACH,
            "precision": "mixed: df32 far field + FP64 near field, FP32 LU + refinement to 1e-12",
            "l2": "inputs larger than L2 (A = 2 x 1.49 GB)", "parallelism": "replicas"}


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_tensor_peak():
    """Dense 16-bit tensor throughput in TFLOP/s: (burst, sustained, source)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), float(p.get("bf16_tflops_sustained", p["bf16_tflops"])), "measured"
    except Exception:
        return 1900.0, 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_cost_model(nodes, tris, ids, refs, nthreads):
    """CPU oracle (C++ restatement of the reference path) on a bounded sample of the
    same workload: assembly of 1/8 of the matrix rows (all columns), one FP64
    matvec over those rows, and one full post-processing pass.  The 17-alpha sweep
    time is assembled from them: 8*t_asm + 17*(2*PLAIN_ITERS*8*t_mv + t_post)."""
    from oracle import pyoracle as po
    t0 = time.perf_counter()
    m = po.Mesh(nodes, tris, ids)
    t_topo = time.perf_counter() - t0
    n = m.n
    rows = n // 8
    t0 = time.perf_counter()
    A, B = m.set_inf_coeff(rows=(0, rows), nthreads=nthreads)
    t_asm = time.perf_counter() - t0
    blk = np.ascontiguousarray(A)
    x = np.random.default_rng(0).standard_normal(n)
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        blk @ x
    t_mv = (time.perf_counter() - t0) / reps
    mu = np.random.default_rng(1).standard_normal(n) * 0.1
    t0 = time.perf_counter()
    m.post(mu, alpha=5.0, mach=MACH, **refs)
    t_post = time.perf_counter() - t0
    k = len(ALPHAS)
    t_sweep = t_topo + 8 * t_asm + k * (2 * PLAIN_ITERS * 8 * t_mv + t_post)
    sample = ("oracle on %d threads: assembly of %d/%d rows x8, FP64 matvec of those rows x8 x 2 x %d "
              "BiCGSTAB iterations (plain-path count), full post-processing; sample wall %.1fs"
              % (nthreads, rows, n, PLAIN_ITERS, t_topo + t_asm + reps * t_mv + t_post))
    return k / t_sweep, sample


def _mesh_ok(nodes, tris, ids):
    """The host topology check of cpg_geometry_create (no device use)."""
    from cpanel_gb300 import _lib
    L = _lib.load()
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int64)
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    info = _lib.GeometryInfo()
    return L.cpg_topology(nodes.ctypes.data_as(_lib.D), len(nodes), tris.ctypes.data_as(_lib.I64),
                          ids.ctypes.data_as(_lib.I32), len(ids), C.byref(info), None, None, None, None, None) == 0


def _wing_with(ntri_target, rng, **kw):
    """A seeded NACA wing with about ntri_target body triangles (for the request mix);
    draws again when the generator made a mesh whose topology the path rejects (a tip
    panel at the trailing edge without a usable CHTLS neighbourhood)."""
    for _ in range(20):
        out = _draw_wing(ntri_target, rng)
        if _mesh_ok(*out[:3]):
            return out
    raise RuntimeError("no valid wing drawn")


def _draw_wing(ntri_target, rng):
    from cpanel_gb300 import wing
    nc = int(rng.integers(20, 101))
    ns = int(max(15, min(400, round(ntri_target / (4.0 * (nc - 1)) + 1))))
    taper = float(rng.uniform(0.3, 1.0))
    span = float(rng.uniform(3, 10)) * (1 + taper) / 2
    spec = wing.WingSpec(m=float(rng.uniform(0, 0.06)), p=float(rng.uniform(0.2, 0.5)), t=float(rng.uniform(0.08, 0.18)),
                         root_chord=1.0, span=span, taper=taper, sweep_deg=float(rng.uniform(0, 35)), n_chord=nc,
                         n_span=ns, wake_len=30.0, wake_dir=(1.0, 0.0, 0.0), seed=int(rng.integers(1 << 30)))
    nodes, tris, ids, info = wing.make_wing(spec)
    return nodes, tris, ids, dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0.0, 0.0))


def batched_and_served():
    """The uneven batch (64 seeded wings x 8 alphas) through the grouped batch solve
    (include/cpanel_batch.h) and, for comparison, through the request loop with 8 slots; and
    a bounded sample of the served stream (Poisson arrivals, 50 req/s, steady wings of
    1k-40k triangles and ~10% unsteady 100-step particle-wake runs on ~4k-triangle wings)
    through the request loop (include/cpanel_serve.h) with 4 slots, mixed precision."""
    from cpanel_gb300 import serve, wing
    out = {}
    # ---- the uneven batch: 64 wings x 8 alphas
    wings = []
    for i in range(64):
        spec = wing.config_random(20261203 + i)
        nodes, tris, ids, info = wing.make_wing(spec)
        rng = np.random.default_rng(20261203 + i)
        flows = [(1.0, float(a), 0.0, MACH) for a in rng.uniform(-2, 10, 8)]
        wings.append((nodes, tris, ids, flows, dict(Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0, 0)),
                      int(np.count_nonzero(ids <= 1000))))
    nsol = sum(len(w[3]) for w in wings)
    label = ("64 seeded NACA wings (config_random, seeds 20261203+i), %d-%d body panels, 8 alphas each"
             % (min(w[5] for w in wings), max(w[5] for w in wings)))
    # grouped batch (include/cpanel_batch.h): one persistent assembly launch for all 64 meshes,
    # work shape from the autotuner (tuned during the warm-up call, cached for the timed one)
    from cpanel_gb300 import batch
    meshes = [dict(nodes=n_, tris=t_, ids=i_, flows=f_, **r_) for n_, t_, i_, f_, r_, _ in wings]
    _, st_warm = batch.batch_solve(meshes, workers=8, tune="auto", lockstep=True)
    t0 = time.perf_counter()
    bres, st = batch.batch_solve(meshes, workers=8, tune="auto", lockstep=True, want=("cp", "CL", "CDi"))
    wall = time.perf_counter() - t0
    # accuracy against the plain FP64 GPU path on a sample of the batch (outside the timing)
    import cpanel_gb300 as cg
    acc = {"meshes": [0, 16, 32, 48], "cp_max_abs": 0.0, "CL_max_rel": 0.0, "CDi_max_rel": 0.0}
    for q in acc["meshes"]:
        g = cg.Geometry(meshes[q]["nodes"], meshes[q]["tris"], meshes[q]["ids"])
        ref = cg.solve_cases(g, meshes[q]["flows"], Sref=meshes[q]["Sref"], bref=meshes[q]["bref"],
                             cref=meshes[q]["cref"], cg=meshes[q]["cg"], precision="fp64", want=("cp",))
        del g
        acc["cp_max_abs"] = max(acc["cp_max_abs"], float(np.abs(bres[q]["cp"] - ref["cp"]).max()))
        acc["CL_max_rel"] = max(acc["CL_max_rel"], float((np.abs(bres[q]["CL"] - ref["CL"]) / np.abs(ref["CL"])).max()))
        acc["CDi_max_rel"] = max(acc["CDi_max_rel"],
                                 float((np.abs(bres[q]["CDi"] - ref["CDi"]) / np.abs(ref["CDi"])).max()))
    acc["within_bound"] = acc["cp_max_abs"] <= 1e-5 and acc["CL_max_rel"] <= 1e-6
    acc["note"] = "every panel of 4 of the 64 wings, all 8 alphas each; bound Cp max-abs <= 1e-5, CL rel <= 1e-6"
    out["batched_uneven"] = {
        "workload": label, "solves": nsol, "wall_s": wall, "solves_per_s": nsol / wall,
        "ms_topology": st["ms_topology"], "ms_grouped_assembly": st["ms_assembly"],
        "ms_lockstep_factorization": st["ms_factor"], "ms_lockstep_solves_and_post": st["ms_solve"],
        "accuracy_vs_plain_fp64": acc,
        "grouped_launch": {"items": st["group"]["items"], "pairs": st["group"]["pairs"],
                           "near_pairs_fp64": st["group"]["near_pairs"], "shape": st["group"]["shape"],
                           "tuned_in_warmup": st_warm["group"]["tuned"] == 1,
                           "candidates_timed": st_warm["group"]["candidates"],
                           "gpairs_per_s": st["group"]["pairs"] / st["group"]["ms"] / 1e6},
        "workers": 8,
        "how": "cpg_batch_solve(lockstep=1): topology and post tables on 8 worker threads, one grouped persistent "
               "assembly launch, the 64 LU factorizations in lockstep (one diagonal-block launch per block step for "
               "all meshes), the 64 x 8 refined solves in lockstep (one launch per substitution block step), each "
               "mesh's residuals and post on its worker's stream"}
    # the same 64 wings through the request loop (one assembly launch per mesh), for comparison
    srv = serve.Server(slots=8, budget_gb=160.0, precision="mixed")
    srv.wait(srv.submit(*wings[0][:4], **wings[0][4]))  # warm-up: kernels, cuBLAS plans, workspaces
    t0 = time.perf_counter()
    tickets = [srv.submit(n_, t_, i_, f_, **r_) for n_, t_, i_, f_, r_, _ in wings]
    res = [srv.wait(t) for t in tickets]
    wall = time.perf_counter() - t0
    srv.close()
    out["batched_uneven_request_loop"] = {
        "workload": label, "solves": nsol, "wall_s": wall, "solves_per_s": nsol / wall,
        "p50_ms": float(np.percentile([r["info"]["total_ms"] for r in res], 50)),
        "max_concurrent": max(r["info"]["running_at_start"] for r in res), "slots": 8,
        "how": "all submitted at once to the request loop; each request is assembly + LU + 8 refined solves + post"}
    # ---- the served stream (bounded sample): steady requests and ~10% unsteady particle-wake runs
    rng = np.random.default_rng(7)
    nreq = 32
    gaps = rng.exponential(1.0 / 50.0, nreq)
    reqs = []
    for q in range(nreq):
        if q % 10 == 5:  # unsteady: 100 steps on a ~4k-triangle wing, body panels only
            nodes, tris, ids, refs = _wing_with(4000.0, rng)
            keep = ids < 1000
            reqs.append(("vp", nodes, tris[keep], ids[keep], refs))
        else:
            nodes, tris, ids, refs = _wing_with(float(rng.uniform(1000, 40000)), rng)
            flows = [(1.0, float(a), 0.0, MACH) for a in rng.uniform(-2, 10, 4)]
            reqs.append(("steady", nodes, tris, ids, flows, refs))

    def submit(srv, r):
        if r[0] == "vp":
            return srv.submit_vp(r[1], r[2], r[3], 100, alpha=8.0, dt=0.05, Sref=r[4]["Sref"], precision="mixed")
        return srv.submit(*r[1:5], **r[5])

    srv = serve.Server(slots=4, budget_gb=160.0, precision="mixed")
    srv.wait(submit(srv, reqs[0]))  # warm-up
    srv.wait(srv.submit_vp(*reqs[5][1:4], 4, alpha=8.0, dt=0.05, precision="mixed"))
    tickets = []
    t0 = time.perf_counter()
    for q in range(nreq):
        time.sleep(gaps[q])
        tickets.append(submit(srv, reqs[q]))
    res = [srv.wait(t) for t in tickets]
    wall = time.perf_counter() - t0
    srv.close()
    kinds = [r[0] for r in reqs]
    lat = [r["info"]["total_ms"] for r in res]
    lat_s = [l for l, k in zip(lat, kinds) if k == "steady"]
    lat_u = [l for l, k in zip(lat, kinds) if k == "vp"]
    nsol = sum(len(r[4]) for r in reqs if r[0] == "steady")
    nb = [r["info"]["n_body"] for r, k in zip(res, kinds) if k == "steady"]
    out["serving"] = {
        "workload": "%d requests, Poisson arrivals at 50 req/s (seed 7): %d steady (NACA wings of %d-%d body panels, "
                    "4 alphas each) and %d unsteady (vortex-particle wake, 100 steps of dt 0.05, alpha 8, "
                    "%d-%d body panels, mixed precision)"
                    % (nreq, len(lat_s), min(nb), max(nb), len(lat_u),
                       min(r["info"]["n_body"] for r, k in zip(res, kinds) if k == "vp"),
                       max(r["info"]["n_body"] for r, k in zip(res, kinds) if k == "vp")),
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "steady_p50_ms": float(np.percentile(lat_s, 50)), "steady_p99_ms": float(np.percentile(lat_s, 99)),
        "unsteady_p50_ms": float(np.percentile(lat_u, 50)), "unsteady_max_ms": float(max(lat_u)),
        "unsteady_particles": [int(r["n_particles"]) for r, k in zip(res, kinds) if k == "vp"],
        "steady_solves_per_s": nsol / wall, "wall_s": wall, "slots": 4,
        "max_concurrent": max(r["info"]["running_at_start"] for r in res),
        "latency": "submit -> results on the host (steady: topology, uploads, assembly, LU, solves, post; "
                   "unsteady: buffer wake, matrices, LU, 100 steps)"}

    # ---- the same stream's first steady requests served in each precision (config 5: against the plain
    # FP64 GPU path): same arrival gaps, same slots
    sub = [q for q in range(nreq) if reqs[q][0] == "steady"][:8]
    comp = {}
    for prec in ("mixed", "plain"):
        srv = serve.Server(slots=4, budget_gb=160.0, precision=prec)
        srv.wait(submit(srv, reqs[sub[0]]))  # warm-up
        tickets = []
        t0 = time.perf_counter()
        for q in sub:
            time.sleep(gaps[q])
            tickets.append(submit(srv, reqs[q]))
        res = [srv.wait(t) for t in tickets]
        wall = time.perf_counter() - t0
        srv.close()
        lat = [r["info"]["total_ms"] for r in res]
        comp[prec] = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                      "solves_per_s": sum(len(reqs[q][4]) for q in sub) / wall, "wall_s": wall}
    nbs = [int(res_i["info"]["n_body"]) for res_i in res]
    out["serving_vs_plain_fp64"] = {
        "workload": "the served stream's first %d steady requests (%d-%d body panels, 4 alphas each) at the same "
                    "arrival gaps, 4 slots, served once in each precision" % (len(sub), min(nbs), max(nbs)),
        "mixed": comp["mixed"], "plain_fp64": comp["plain"],
        "speedup_solves_per_s": comp["mixed"]["solves_per_s"] / comp["plain"]["solves_per_s"],
        "p50_ratio_plain_over_mixed": comp["plain"]["p50_ms"] / comp["mixed"]["p50_ms"]}
    return out


def vortex_particles(steps=20):
    """Unsteady vortex-particle wake (bounded sample): NACA 4412 AR 6 wing of 8,216 body triangles without wake
    panels, alpha 8 deg, dt 0.05, Barnes-Hut on: the first `steps` steps of the VP loop in
    FP64 and in the mixed form (FP32 far fields, FP64 near fields, FP32 LU refined in
    FP64), the particle-velocity check of the final state (mixed and FP64 octree against
    the FP64 direct sum), then the particle operators on 40,000 particles spread behind
    the wing in both precisions."""
    import torch

    from cpanel_gb300 import vp, wing
    spec = wing.WingSpec(m=0.04, p=0.4, t=0.12, root_chord=1.0, span=6 * (1 + 0.6) / 2, taper=0.6, sweep_deg=0.0,
                         n_chord=80, n_span=26, wake_len=30.0, wake_dir=(1.0, 0.0, 0.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    tris, ids = tris[keep], ids[keep]

    def rel(a, b):
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    loops, cases = {}, {}
    for prec in ("plain", "mixed"):
        t0 = time.perf_counter()
        S = vp.VPCase(nodes, tris, ids, V=1.0, alpha=8.0, dt=0.05, accelerate=True, Sref=info["area"], precision=prec)
        S.step(3)
        torch.cuda.synchronize()
        t_setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        S.step(steps)
        torch.cuda.synchronize()
        t_loop = time.perf_counter() - t0
        inf = S.info()
        done = inf["timestep"] - 3  # fewer than `steps` once the Trefftz check has converged
        tz = S.trefftz()
        loops[prec] = {"steps": done, "ms_per_step": t_loop / max(done, 1) * 1e3, "setup_and_first_3_steps_s": t_setup,
                       "particles_at_end": inf["n_particles"], "trefftz_CL": tz["CL"], "trefftz_CD": tz["CD"],
                       "converged": tz["converged"], "solve_fallbacks": inf["solve_fallbacks"]}
        cases[prec] = S
    P = cases["plain"]
    v64, v32, vdir = P.velocities("plain"), P.velocities("mixed"), P.velocities("plain", direct=True)
    check = {"particles": int(len(v64)), "mixed_vs_plain_octree": rel(v32, v64),
             "plain_octree_vs_fp64_direct": rel(v64, vdir), "mixed_vs_fp64_direct": rel(v32, vdir),
             "what": "max |dv| / max |v| over the convective particle velocities (Vinf + particles + panels)"}
    pm, pp = cases["mixed"].particles(), P.particles()
    drift = {"same_shedding": bool(np.array_equal(pm["shed_time"], pp["shed_time"])
                                   and np.array_equal(pm["parent"], pp["parent"])),
             "pos_rel": rel(pm["pos"], pp["pos"]), "strength_rel": rel(pm["strength"], pp["strength"]),
             "CL_rel": abs(loops["mixed"]["trefftz_CL"] - loops["plain"]["trefftz_CL"]) / abs(loops["plain"]["trefftz_CL"])}
    del cases, P
    # operators at 40k particles
    rng = np.random.default_rng(4)
    n = 40000
    pos = np.c_[rng.uniform(1.0, 15.0, n), rng.uniform(-2.4, 2.4, n), rng.normal(0, 0.3, n)]
    Pt = torch.tensor(pos, device="cuda")
    A = torch.tensor(rng.normal(size=(n, 3)) * 0.01, device="cuda")
    R = torch.full((n,), 0.05, dtype=torch.float64, device="cuda")
    verts = np.asarray(nodes)[np.asarray(tris) - 1].reshape(-1, 9)
    BV = torch.tensor(verts, device="cuda")
    SG = torch.tensor(rng.normal(size=len(verts)), device="cuda")
    MU = torch.tensor(rng.normal(size=len(verts)), device="cuda")

    def timed(f, reps=2):
        f()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            f()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps * 1e3

    pairs = float(n) * len(verts)
    ops, outs = {}, {}
    tree = vp.ParticleFMM(Pt, A, R)
    for prec in ("plain", "mixed"):
        tree.set_precision(prec)
        o = {"barnes_hut_vel_stretch_diff_ms": timed(lambda: tree.barnesHut(True, True, True))}
        o["panel_velocity_ms"] = timed(lambda: vp.panels_velocity(BV, SG, MU, None, None, Pt, precision=prec), 1)
        o["panel_stretching_ms"] = timed(lambda: vp.panels_stretching(BV, SG, MU, None, None, Pt, A, precision=prec), 1)
        o["panel_velocity_pairs_per_s"] = pairs / (o["panel_velocity_ms"] * 1e-3)
        o["panel_stretching_pairs_per_s"] = pairs / (o["panel_stretching_ms"] * 1e-3)
        ops[prec] = o
        outs[prec] = [x.cpu().numpy() for x in tree.barnesHut(True, True, True)] + [
            vp.panels_velocity(BV, SG, MU, None, None, Pt, precision=prec).cpu().numpy(),
            vp.panels_stretching(BV, SG, MU, None, None, Pt, A, precision=prec).cpu().numpy()]
    names = ("bh_velocity", "bh_stretching", "bh_diffusion", "panel_velocity", "panel_stretching")
    ops["mixed_vs_plain_rel"] = {k: rel(outs["mixed"][i], outs["plain"][i]) for i, k in enumerate(names)}
    ops["tree_build_ms"] = timed(lambda: vp.ParticleFMM(Pt, A, R))
    del tree, Pt, A, R, BV, SG, MU
    at_scale = vp_config4_at_scale()
    return {"vp_unsteady": {
        "workload": "NACA 4412 AR 6 taper 0.6, %d body triangles, no wake panels, alpha 8 deg, dt 0.05, "
                    "Barnes-Hut theta 0.5" % len(verts),
        "loop": loops, "first_step": 4,
        "what": "cpg_vpcase_step: convection, shedding, strength update, octree, source strengths, solve "
                "(plain: FP64 BiCGSTAB; mixed: FP32 LU refined in FP64), Trefftz-plane convergence check",
        "velocity_check": check, "mixed_vs_plain_state": drift,
        "operators_40k_particles": ops, "config4_300_steps": at_scale}}


def config4_wing():
    """The unsteady workload's wing: NACA 4412, AR 6, taper 0.6, 21 points per side x 101 stations
    (8,076 body triangles, 100 trailing-edge edges: 100 particles shed per step), no wake panels."""
    from cpanel_gb300 import wing
    spec = wing.WingSpec(m=0.04, p=0.4, t=0.12, root_chord=1.0, span=6 * (1 + 0.6) / 2, taper=0.6, sweep_deg=0.0,
                         n_chord=21, n_span=101, wake_len=30.0, wake_dir=(1.0, 0.0, 0.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    return nodes, tris[keep], ids[keep], info


def vp_config4_at_scale(steps=300, chunk=50):
    """The unsteady workload at its stated scale, mixed form: impulsive start at alpha 8 deg, dt
    0.05, 300 steps with the Trefftz-plane early stop off, one particle per trailing-edge edge
    per step (~29.8k particles at the end); ms per step and particle count per `chunk` steps,
    then the convective velocities of the final state: the mixed octree against the FP64
    octree (the arithmetic error of the mixed form) and both against the FP64 direct sum."""
    import torch

    from cpanel_gb300 import vp
    nodes, tris, ids, info = config4_wing()
    t0 = time.perf_counter()
    S = vp.VPCase(nodes, tris, ids, V=1.0, alpha=8.0, dt=0.05, accelerate=True, Sref=info["area"],
                  precision="mixed", run_all_steps=True)
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    rows, done = [], 0
    t_all = time.perf_counter()
    while done < steps:
        k = min(chunk, steps - done)
        t0 = time.perf_counter()
        S.step(k)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        done += k
        rows.append({"to_step": done, "particles": S.info()["n_particles"], "ms_per_step": dt / k * 1e3})
    wall = time.perf_counter() - t_all
    inf = S.info()
    tz = S.trefftz()

    def rel(a, b):
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    t0 = time.perf_counter()
    v32, v64, vdir = S.velocities("mixed"), S.velocities("plain"), S.velocities("plain", direct=True)
    t_check = time.perf_counter() - t0
    return {"workload": "NACA 4412 AR 6 taper 0.6, %d body triangles (21 points per side x 101 stations), "
                        "alpha 8 deg, dt 0.05, Barnes-Hut theta 0.5, mixed form" % inf["n_body"],
            "steps": inf["timestep"], "particles_at_end": inf["n_particles"], "wall_s": wall,
            "setup_s": setup, "ms_per_step_by_chunk": rows, "trefftz_CL": tz["CL"], "trefftz_CD": tz["CD"],
            "trefftz_check_fired": tz["converged"], "solve_fallbacks": inf["solve_fallbacks"],
            "velocity_check": {"particles": int(len(v32)), "mixed_vs_fp64_octree": rel(v32, v64),
                               "fp64_octree_vs_fp64_direct": rel(v64, vdir), "mixed_vs_fp64_direct": rel(v32, vdir),
                               "check_s": t_check,
                               "what": "max |dv| / max |v| over the convective particle velocities"}}


def vp_loop_only(precision, steps):
    """The vortex-particle loop alone (profiling aid): case creation, 3 steps, `steps` timed steps."""
    import torch

    from cpanel_gb300 import vp, wing
    spec = wing.WingSpec(m=0.04, p=0.4, t=0.12, root_chord=1.0, span=6 * (1 + 0.6) / 2, taper=0.6, sweep_deg=0.0,
                         n_chord=80, n_span=26, wake_len=30.0, wake_dir=(1.0, 0.0, 0.0))
    nodes, tris, ids, info = wing.make_wing(spec)
    keep = ids < 1000
    S = vp.VPCase(nodes, tris[keep], ids[keep], V=1.0, alpha=8.0, dt=0.05, accelerate=True, Sref=info["area"],
                  precision=precision)
    S.step(3)
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        t0 = time.perf_counter()
        S.step(1)
        ms.append((time.perf_counter() - t0) * 1e3)
    print(json.dumps({"vp_loop": precision, "ms_per_step": [round(t, 2) for t in ms], "info": S.info()}))


def batch_loop_only(n_wings=64, lockstep=True):
    """The uneven batch alone (profiling aid): n_wings seeded wings x 8 alphas through
    cpg_batch_solve, a warm-up call (kernels, work-shape tuning) and one timed call."""
    from cpanel_gb300 import batch, wing
    meshes = []
    for i in range(n_wings):
        spec = wing.config_random(20261203 + i)
        nodes, tris, ids, info = wing.make_wing(spec)
        rng = np.random.default_rng(20261203 + i)
        meshes.append(dict(nodes=nodes, tris=tris, ids=ids, flows=[(1.0, float(a), 0.0, MACH) for a in
                                                                   rng.uniform(-2, 10, 8)],
                           Sref=info["area"], bref=spec.span, cref=1.0, cg=(0.25, 0, 0)))
    batch.batch_solve(meshes, workers=8, lockstep=lockstep)
    t0 = time.perf_counter()
    _, st = batch.batch_solve(meshes, workers=8, lockstep=lockstep)
    wall = time.perf_counter() - t0
    print(json.dumps({"batch_loop": n_wings, "lockstep": lockstep, "solves_per_s": st["solves"] / wall,
                      "stats": st}))


REF_SOLVES = 2  # config-2 right-hand sides the reference arm solves to convergence

# DRAM bytes (read + write) of one factorization of the benchmark wing: the sum of dram__bytes_read.sum and
# dram__bytes_write.sum over the 945 kernels of each factorization in a one-pass ncu capture of
# `bench.py --steps 1 --warmup 1 --no-cpu --no-plain --no-serving --no-vp` (four factorizations: 31.8-32.1 GB)
LU_TRAFFIC = {"multi_rhs": 3.20e10}
LU_TRAFFIC_SOURCE = "ncu capture (dram__bytes_read.sum + dram__bytes_write.sum over every kernel of one factorization)"


def cpu_model():
    """(model name, nproc) of the host."""
    name = ""
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    name = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not name:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for ln in out.splitlines():
                if ln.startswith("Model name"):
                    name = ln.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return name or platform.machine(), os.cpu_count() or 1


def run_reference(args):
    """The reference's CPU path, timed: the oracle restatement (the reference itself needs Eigen,
    Boost and GTest, absent here) on all host threads, on the benchmark's own workload.  The
    matrices are assembled once (timed), then REF_SOLVES angles of attack are solved to the
    reference's BiCGSTAB tolerance with post-processing, each timed.  One step = one solve plus
    its 1/17 share of the topology and assembly, so solves/s = 1000 / ms_per_step (the 17-alpha
    sweep extrapolated from the measured assembly and per-solve times).  Beside it, the full
    small case (NACA 0012, 3,896 panels, one alpha) end to end on all threads and on one."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import build as oracle_build
    oracle_build.build()
    from oracle import pyoracle as po
    from cpanel_gb300 import wing
    spec, nodes, tris, ids, info, refs = workload()
    nthreads = os.cpu_count() or 1
    k = len(ALPHAS)
    t_run = time.perf_counter()
    t0 = time.perf_counter()
    m = po.Mesh(nodes, tris, ids)
    t_topo = time.perf_counter() - t0
    t0 = time.perf_counter()
    A, B = m.set_inf_coeff(nthreads=nthreads)
    t_asm = time.perf_counter() - t0
    solves = []
    for i in range(max(1, min(args.steps, REF_SOLVES))):
        t0 = time.perf_counter()
        r = m.case(A, B, V=1.0, alpha=ALPHAS[i], mach=MACH, nthreads=nthreads, **refs)
        solves.append({"alpha": ALPHAS[i], "s": time.perf_counter() - t0, "iters": int(r["iters"]),
                       "converged": bool(r["converged"]), "CL": float(r["CL"])})
    del A, B, m
    t_solve = sum(q["s"] for q in solves) / len(solves)
    ms_step = ((t_topo + t_asm) / k + t_solve) * 1e3
    value = 1e3 / ms_step
    # the small steady case end to end (topology, assembly, BiCGSTAB, post)
    s1 = wing.config_small_steady()
    n1, t1, i1, inf1 = wing.make_wing(s1)
    refs1 = dict(Sref=inf1["area"], bref=s1.span, cref=1.0, cg=(0.25, 0.0, 0.0))
    small = {}
    for nt in (nthreads, 1):
        t0 = time.perf_counter()
        m1 = po.Mesh(n1, t1, i1)
        A1, B1 = m1.set_inf_coeff(nthreads=nt)
        r1 = m1.case(A1, B1, V=1.0, alpha=5.0, mach=MACH, nthreads=nt, **refs1)
        dt = time.perf_counter() - t0
        small["threads_%d" % nt] = {"solves_per_s": 1.0 / dt, "wall_s": dt, "iters": int(r1["iters"]),
                                   "CL": float(r1["CL"])}
        del m1, A1, B1
    model, nproc = cpu_model()
    sample = ("oracle on %d threads: topology and FP64 assembly of the %d-panel wing once (%.1f s), %d of the %d "
              "alphas solved to convergence (BiCGSTAB, Eigen semantics) with post-processing (%.1f s each); a step "
              "is one solve plus 1/%d of the assembly" % (nthreads, info["n_body"], t_topo + t_asm, len(solves), k,
                                                          t_solve, k))
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": len(solves),
            "warmup": 0, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded NACA wing)", "config": config_dict(info), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference": {"cpu": model, "nproc": nproc, "threads": nthreads, "ms_topology": t_topo * 1e3,
                          "ms_assembly": t_asm * 1e3, "solves": solves,
                          "sweep_17_alpha_s_extrapolated": t_topo + t_asm + k * t_solve,
                          "small_case_end_to_end": small, "wall_s": time.perf_counter() - t_run}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--workload", default="multi_rhs", choices=["multi_rhs", "mid"])
    ap.add_argument("--no-serving", action="store_true", help="skip the uneven-batch and served-stream runs")
    ap.add_argument("--no-vp", action="store_true", help="skip the vortex-particle sample")
    ap.add_argument("--batch-loop", type=int, default=0, metavar="N",
                    help="only the uneven batch of N seeded wings (lockstep), warm-up and one timed call")
    ap.add_argument("--vp-loop", choices=["plain", "mixed"],
                    help="only the vortex-particle loop in this precision: 3 steps, then --steps timed "
                         "steps (one JSON line; for profiling)")
    ap.add_argument("--vp-scale", action="store_true",
                    help="only the unsteady workload at its stated scale (300 mixed steps; one JSON line)")
    args = ap.parse_args()
    if args.vp_scale:
        import __graft_entry__
        __graft_entry__.build()
        print(json.dumps({"config4_300_steps": vp_config4_at_scale()}), flush=True)
        return
    if args.impl == "reference":
        return run_reference(args)
    if args.vp_loop:
        return vp_loop_only(args.vp_loop, args.steps)
    if args.batch_loop:
        return batch_loop_only(args.batch_loop)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if dist:
        dist.barrier()
    import cpanel_gb300 as cg

    spec, nodes, tris, ids, info, refs = workload(args.workload)
    flows = [(1.0, a, 0.0, MACH) for a in ALPHAS]
    k = len(flows)
    ctx = cg.Context(local)
    stream = torch.cuda.current_stream()
    ctx.check(ctx.L.cpg_set_stream(ctx.h, stream.cuda_stream), "set_stream")
    g = cg.Geometry(nodes, tris, ids, ctx=ctx)
    n = g.n

    # ---- accuracy vs the plain FP64 GPU path (untimed) and its throughput
    acc = {}
    plain = None
    if not args.no_plain:
        # the plain FP64 GPU path, timed over PLAIN_RUNS full sweeps (FP64 assembly, BiCGSTAB per
        # column, post-processing), the same step as the timed mixed one
        times = []
        for _ in range(PLAIN_RUNS):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g.setInfCoeff("fp64")
            rp = cg.solve_cases(g, flows, precision="fp64", want=("cp",), **refs)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        st = rp["stats"]
        t_plain = sum(times) / len(times)
        plain = {"value": k / t_plain, "unit": "solves/s", "ms_per_step": t_plain * 1e3,
                 "ms_per_run": [round(t * 1e3, 1) for t in times], "iters_max": st["iters_max"],
                 "ms_assemble": st["ms_assemble"], "ms_solve": st["ms_solve"], "ms_post": st["ms_post"],
                 "steps": len(times)}
        rm = cg.solve_cases(g, flows, precision="mixed", want=("cp",), **refs)
        acc = {"cp_err_max": float(np.abs(rm["cp"] - rp["cp"]).max()),
               "cl_relerr_max": float(np.max(np.abs(rm["CL"] - rp["CL"]) / np.abs(rp["CL"]))),
               "cdi_relerr_max": float(np.max(np.abs(rm["CDi"] - rp["CDi"]) / np.maximum(np.abs(rp["CDi"]), 1e-12)))}
        g.ctx.check(0)
        del rp, rm

    # ---- timed: mixed path, mesh resident
    def step():
        g.setInfCoeff("mixed")
        return cg.solve_cases(g, flows, precision="mixed", want=(), **refs)

    for _ in range(args.warmup):
        step()
    ctx.prof_enable(True)
    lat = []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            ev[i][0].record(stream)
            r = step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    lat = [a.elapsed_time(b) for a, b in ev]
    prof = ctx.prof_read()
    ctx.prof_enable(False)
    t_dev = sum(lat) / 1e3
    t_max = max_over_ranks(t_dev, dist)
    value = world * k * args.steps / t_max
    stats = r["stats"]

    # ---- e2e through the C ABI from host arrays
    e2e_times = []
    h2d = d2h = 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ge = cg.Geometry(nodes, tris, ids, ctx=ctx)
        ge.setInfCoeff("mixed")
        re = cg.solve_cases(ge, flows, precision="mixed", want=("cp",), **refs)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
        h2d = ge.info["h2d_bytes"] + k * 8 * 20
        d2h = re["cp"].nbytes + 2 * k * 8 + 9 * k * 8
        del ge
    e2e_value = world * k * len(e2e_times) / sum(e2e_times)

    # ---- roofline of the dominant kernel class in the timed region
    hbm, peak_kind = read_peaks()
    fp64 = C_double()
    ctx.check(ctx.L.cpg_measure_fp64_peak(ctx.h, C.byref(fp64)), "fp64 peak")
    fp64_peak = fp64.value
    roofs = {}
    a_l, a_ms = prof["assembly"]
    if a_l:
        # near pairs in FP64: per pair 3 edges x (~101 flop + 5 sqrt + 2 div + atan2 + log) + 20
        # flop + sqrt + div; transcendentals counted as one op each
        fl = stats["n_near"] * (3 * (101 + 5 + 2 + 2) + 22)
        ach = fl / (a_ms / a_l * 1e-3) / 1e12
        roofs["assembly"] = {"bound": "fp64", "kernel": "k_assemble_mixed (FP64 near field, df32 far field)",
                             "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                             "traffic": None, "peak_source": "measured in this run (FP64 FMA probe)",
                             "algorithmic_flops_per_launch": fl, "avg_launch_ms": a_ms / a_l, "launches": a_l}
    g_l, g_ms = prof["lu_factor"]
    tc_burst, tc_sust, tc_src = read_tensor_peak()
    if g_l:
        # 2/3 n^3 FP32-equivalent flop per factorization; its rank-1024 updates take three FP16
        # products per FP32-equivalent product (hi hi + hi lo + lo hi), so the tensor-pipe
        # denominator is the 16-bit peak / 3 (sustained: the factorization runs inside a long step)
        fl = 2.0 / 3.0 * n ** 3
        ach = fl / (g_ms / g_l * 1e-3) / 1e12
        pk = tc_sust / 3
        roofs["lu_factor"] = {"bound": "tensor", "kernel": "two-level blocked LU: k_lu_diag (128 x 128 blocks), "
                              "k_tc_gemm rank-1024 updates (tcgen05, FP16 hi/lo split), panel products",
                              "achieved": ach, "unit": "TFLOP/s (FP32-equivalent)", "peak": pk, "frac": ach / pk,
                              "peak_source": "%s bf16 sustained / 3 FP16 products (of %s)" % (tc_src, tc_src),
                              "traffic": LU_TRAFFIC.get(args.workload), "traffic_source": LU_TRAFFIC_SOURCE,
                              "avg_launch_ms": g_ms / g_l, "launches": g_l}
    t_l, t_ms = prof["tc_gemm"]
    if t_l and g_l:
        # the tensor-core GEMM launches inside the factorizations: 2 (n - KE)^2 1024 flop per
        # 1,024-column panel, summed over the panels
        ob = 1024
        fl_tc = sum(2.0 * (n - ke) * (n - ke) * ob for ke in range(ob, n, ob)) * 3  # FP16 flop
        ach = fl_tc / (t_ms / g_l * 1e-3) / 1e12
        roofs["tc_gemm"] = {"bound": "tensor", "kernel": "k_tc_gemm (rank-1024 updates of one factorization)",
                            "achieved": ach, "unit": "TFLOP/s (FP16 tensor)", "peak": tc_sust,
                            "frac": ach / tc_sust, "peak_source": "%s bf16 sustained" % tc_src, "traffic": None,
                            "ms_per_factorization": t_ms / g_l, "launches_per_factorization": t_l / g_l}
    s_l, s_ms = prof["lu_solve"]
    if s_l:
        bytes_s = 4.0 * n * n + 2 * 4.0 * k * n  # L and U read once per solve
        ach = bytes_s / (s_ms / s_l * 1e-3) / 1e9
        roofs["lu_solve"] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                             "peak_source": peak_kind, "traffic": None}
    r_l, r_ms = prof["residual"]
    if r_l:
        bytes_r = 8.0 * n * n + 8.0 * 3 * k * n
        ach = bytes_r / (r_ms / r_l * 1e-3) / 1e9
        roofs["residual"] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                             "peak_source": peak_kind, "traffic": None}
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    roof = roofs.get(dom[0])
    breakdown = {name: {"launches": int(l), "ms": round(ms, 3)} for name, (l, ms) in prof.items() if l}

    extra = {}
    if rank == 0 and world == 1 and not args.no_serving:
        extra = batched_and_served()
    if rank == 0 and world == 1 and not args.no_vp:
        extra.update(vortex_particles())

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, sample = cpu_cost_model(nodes, tris, ids, refs, os.cpu_count() or 1)
        cpu = {"value": v, "unit": "solves/s", "cores": os.cpu_count() or 1, "kind": "port", "sample": sample}

    if rank == 0:
        lat_sorted = sorted(lat)
        p50 = float(np.percentile(lat_sorted, 50))
        p99 = float(np.percentile(lat_sorted, 99))
        launches = int(sum(l for l, _ in prof.values()))
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+df32+f64", "data": "synthetic (seeded NACA wing)",
                "config": config_dict(info, args.workload),
                "latency_ms": {"p50": p50, "p99": p99, "what": "one 17-alpha sweep request (device time)"},
                "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "roofline": roof, "roofline_all": roofs, "dominant_kernel_class": {"name": dom[0], "ms": dom[1][1], "launches": dom[1][0]},
                "kernel_breakdown_ms": breakdown, "gpu_launches": launches,
                "solver": {"iters_max": stats["iters_max"], "refinements": stats["refinements"],
                           "residual_max": stats["residual_max"], "near_pairs": stats["n_near"]},
                "cpu_baseline": cpu, "clocks": clk.summary(), "wall_s": wall}
        line.update(extra)
        # the metric's accuracy claims last, where a truncated view of the line keeps them
        line["plain_fp64"] = plain
        line["accuracy_vs_plain_fp64"] = acc
        if plain:
            line["speedup_vs_plain_fp64"] = value / plain["value"]
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
