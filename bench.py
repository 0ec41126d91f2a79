#!/usr/bin/env python3
"""Benchmark: 3D Newton field FMM particles/s on GB300.

One step = one complete solve (Morton keys, sort, tree, interaction lists,
P2M, M2M, M2L, L2L, L2P, P2P, scatter) of the workload, inputs resident in
HBM (``value``) or in pinned host memory with the copies inside the timed
region (``e2e``, through the same C ABI call a user makes).

Workload (default ``plummer4m``): N = 4,000,000 particles from a Plummer
sphere (a = 0.05, radial cut 1.0, box [-1,1]^3), charges U[0,1], p = 12,
leaf capacity 64, potential + field, rotate flavour, mixed precision (FP32
bulk, FP64 tables/centres/final sums).  The same line reports the plain FP64
GPU path on the same input (``fp64``), the error of the mixed path against
it and against an FP64 direct sum on a target subset.

The same line carries the clustered configuration at the other two orders
(``orders``: p = 8 and 16, mixed and FP64, with their errors), the served
request stream (tolerance-driven plans, p50/p99 over an arrival-rate sweep,
per-request errors), the batched systems and the CPU baseline.

``--impl reference`` times the reference algorithm on the host cores: the
C restatement of LibAran's solver in oracle/ (the reference itself needs
glib and libvsg, which are not available), full solves of the same
4M-particle workload with the per-node and per-leaf work spread over every
host thread.

Multi-GPU: one process per GPU (torchrun); each rank solves its own
replica (the path does not shard: independent solves, no collective on the
data path); ``value`` = particles of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3D FMM particles/s at rel-err≤1e-6 vs plain FP64 GPU path; served p50/p99 latency"
UNIT = "particles/s"

WORKLOADS = {
    # name: (generator, n, order, maxbox, lb, ub, description)
    "plummer4m": ("plummer", 4_000_000, 12, 64, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0),
                  "N=4,000,000 Plummer (a=0.05, r<=1), q~U[0,1], p=12, leaf 64, field"),
    "uniform1m": ("uniform", 1_000_000, 12, 64, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0),
                  "N=1,000,000 uniform in [0,1]^3, q~U[-1,1], p=12, leaf 64, field"),
    # small case for full-set kernel captures (a few hundred MB on the device)
    "plummer400k": ("plummer", 400_000, 12, 64, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0),
                    "N=400,000 Plummer (a=0.05, r<=1), q~U[0,1], p=12, leaf 64, field"),
}


def m2l_flops_rotate(p: int) -> int:
    """Algorithmic flops of one rotate-flavour M2L by the operator's own
    definition: 4 [A(p-1) + B(p) + A(p)], A(L) = (L+1)(L+2)(4L+3)/6 the
    multiply-adds of a real Wigner-d block applied to complex coefficients
    (aransphericalseriesd-rotate.c:34-80), B(p) = p(p+1)(p+2)/3 those of the
    vertical translation (aransphericalseriesd-translate.c:647-675); 13,988 at
    p = 12."""
    a = lambda L: (L + 1) * (L + 2) * (4 * L + 3) // 6
    return 4 * (a(p - 1) + p * (p + 1) * (p + 2) // 3 + a(p))


def m2m_flops_rotate(p: int) -> int:
    """Algorithmic flops of one rotate M2M: 8 A(p-1) + 4 sum_{l<p} (l+1)(l+2)/2
    (two real-d rotations of the tri(p) multipole and the vertical shift)."""
    a = lambda L: (L + 1) * (L + 2) * (4 * L + 3) // 6
    return 8 * a(p - 1) + 4 * sum((l + 1) * (l + 2) // 2 for l in range(p))


def l2l_flops_rotate(p: int) -> int:
    """Algorithmic flops of one rotate L2L: 8 A(p) + 4 sum_{l<=p} sum_{m<=l}
    (p - l + 1) (two rotations of the tri(p+1) local and the vertical shift)."""
    a = lambda L: (L + 1) * (L + 2) * (4 * L + 3) // 6
    return 8 * a(p) + 4 * sum((p - l + 1) * (l + 1) for l in range(p + 1))


def p2m_flops(p: int) -> int:
    """Algorithmic flops of P2M per particle: 16 tri(p)."""
    return 16 * p * (p + 1) // 2


def l2p_flops(p: int) -> int:
    """Algorithmic flops of L2P with the gradient per particle: 32 tri(p+1)."""
    return 32 * (p + 1) * (p + 2) // 2


def stage_rooflines(stage_ms: dict, stats: dict, info: dict, n: int, p: int, fp32_tflops: float,
                    hbm_gbs: float) -> dict:
    """Ideal time of every stage against its bound (FP32 CUDA-core peak for
    the expansion and near-field stages, HBM for sort/tree/lists) from the
    algorithmic work: P2P 20 flops per directed pair (2 x the pair counter),
    M2L F(p) per translation, M2M/L2L by their rotate definitions per
    translation, P2M 16 tri(p) and L2P 32 tri(p+1) per particle, tree 80 B per
    particle (32 B read, 32 B sorted copy, 16 B key and permutation); the
    fraction is ideal / measured, and the sum of ideal times over the step's
    measured time is the step's roofline fraction."""
    peak = fp32_tflops * 1e12
    work = {
        "p2p": (20.0 * 2 * stats["p2p"], "flop"),
        "m2l": (float(info["far"]) * m2l_flops_rotate(p), "flop"),
        "m2m": (float(stats["m2m"]) * m2m_flops_rotate(p), "flop"),
        "l2l": (float(stats["l2l"]) * l2l_flops_rotate(p), "flop"),
        "p2m": (float(n) * p2m_flops(p), "flop"),
        "l2p": (float(n) * l2p_flops(p), "flop"),
        "sort+tree+lists": (80.0 * n, "byte"),
    }
    out, ideal_total = {}, 0.0
    for k, (w, unit) in work.items():
        meas = (sum(stage_ms[x] for x in ("sort", "tree", "lists")) if k == "sort+tree+lists"
                else stage_ms[k])
        ideal = 1e3 * (w / peak if unit == "flop" else w / (hbm_gbs * 1e9))
        ideal_total += ideal
        out[k] = {"work": w, "unit": unit, "ideal_ms": round(ideal, 4),
                  "measured_ms": round(meas, 4), "frac": round(ideal / meas, 4) if meas else None}
    out["sum_ideal_over_step"] = round(ideal_total / stage_ms["total"], 4)
    return out


def m2l_kernel_name(precision: str, p: int, choice: str) -> str:
    """The M2L kernel a solve runs: choice is ARAN_M2L_KERNEL ("lanes",
    "sibling", "tc" or empty); a kernel that does not serve the order or the
    precision hands over to the next in tc, lanes, sibling."""
    if precision != "mixed" or p not in (4, 8, 12) or choice == "sibling":
        return "k_m2l_sibling (rotate M2L, all levels, one launch)"
    if choice == "tc" and p in (8, 12):
        return (f"k_m2l_tc<{p}> (rotate M2L as dense TF32 hi/lo products on tcgen05, "
                "all levels, one launch)")
    return f"k_m2l_lanes<{p}> (rotate M2L, FP32 lane pairs, all levels, one launch)"


def m2l_flops(p: int) -> int:
    """Algorithmic flops of one rotate-flavour M2L as the GPU applies it:
    2 flops per multiply-add of
      * the z-phase of the tri(p) source and tri(p+1) local coefficients
        (4 multiply-adds per complex product),
      * the forward rotation, sum_{l<p} (l+1)^2 real factors on each of the
        real and imaginary parts (even/odd Wigner blocks),
      * the translation along z, p(p+1)(p+2)/3 real factors on both parts,
      * the backward rotation, sum_{l<=p} (l+1)^2 on both parts."""
    sq = lambda L: L * (L + 1) * (2 * L + 1) // 6          # sum_{l<L} (l+1)^2
    tri = lambda L: L * (L + 1) // 2
    macs = 4 * (tri(p) + tri(p + 1)) + 2 * (sq(p) + p * (p + 1) * (p + 2) // 3 + sq(p + 1))
    return 2 * macs


def make_workload(name: str, seed_offset: int = 0):
    from aran_gb300 import workloads as W
    gen, n, p, maxbox, lb, ub, desc = WORKLOADS[name]
    seed = (3 if gen == "plummer" else 2) + 1000 * seed_offset
    x, q = getattr(W, gen)(n, seed)
    return x, q


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region (200 ms period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------------ serving
TOLERANCES = (1e-4, 1e-6, 1e-9)


def serving_stream(nreq: int, rate: float, seed: int = 5):
    """Poisson arrivals of 3D potential+field solves: N log-uniform in
    [1e3, 2e6], a requested relative potential error drawn from 1e-4 / 1e-6
    / 1e-9 (the request loop picks order and precision for it), half uniform
    in [0,1]^3, half Plummer in [-1,1]^3, leaf 64."""
    import numpy as np
    from aran_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    reqs = []
    for i in range(nreq):
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(2e6))))
        tol = TOLERANCES[int(rng.integers(0, 3))]
        if rng.uniform() < 0.5:
            x, q = W.uniform(n, 1000 + i)
            lb, ub = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
        else:
            x, q = W.plummer(n, 1000 + i)
            lb, ub = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)
        reqs.append(dict(arrival=float(arrivals[i]), x=x, q=q, tol=tol,
                         kw=dict(lbound=lb, ubound=ub, maxbox=64, field=True)))
    return reqs


def run_serving(reqs, rate_scale: float = 1.0, plain_fp64: bool = False, nslots: int = 4,
                budget: float = 150e9, keep: bool = False) -> dict:
    """Replays the stream (arrival times / rate_scale; 0 = all at once).
    Default: every request carries its tolerance and the request loop plans
    order and precision.  plain_fp64: the same orders, every request FP64."""
    import numpy as np
    import aran_gb300 as A
    plans = {tol: A.plan_for_tolerance(tol) for tol in TOLERANCES}

    def args_of(r):
        order, prec, _ = plans[r["tol"]]
        if plain_fp64:
            return dict(order=order, precision="fp64", tolerance=0.0, **r["kw"])
        return dict(order=0, tolerance=r["tol"], **r["kw"])

    with A.Server(nslots=nslots, hbm_budget_bytes=budget) as sv:
        # one warm request per configuration so table builds stay out of the stream
        seen = set()
        for r in reqs:
            a = args_of(r)
            key = (plans[r["tol"]][:2], r["kw"]["lbound"])
            if key not in seen:
                seen.add(key)
                sv.wait(sv.submit(r["x"][:2000], r["q"][:2000], **a))
        t0 = time.perf_counter()
        tickets = []
        for r in reqs:
            if rate_scale > 0:
                dt = r["arrival"] / rate_scale - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
            tickets.append(sv.submit(r["x"], r["q"], **args_of(r)))
        outs = [sv.wait(t) for t in tickets]
    infos = [o[2] for o in outs]
    lat = np.array([i["end_s"] - i["submit_s"] for i in infos])
    span = max(i["end_s"] for i in infos) - min(i["submit_s"] for i in infos)
    npart = sum(len(r["q"]) for r in reqs)
    res = {"mode": "plain FP64" if plain_fp64 else "tolerance plan", "requests": len(reqs),
           "p50_ms": float(np.percentile(lat, 50) * 1e3),
           "p99_ms": float(np.percentile(lat, 99) * 1e3),
           "throughput": npart / span, "unit": UNIT,
           "mean_queue_ms": float(np.mean([i["start_s"] - i["submit_s"] for i in infos]) * 1e3)}
    if keep:
        res["_outs"] = outs
    return res


def serving_errors(reqs, outs, targets: int = 200) -> dict:
    """Per request: relative L2 and largest per-particle relative error
    |phi - phi_ref| / max(|phi|, |phi_ref|) (tests/newtonpot3.c:678-715) of
    the potential on a target sample against the FP64 direct sum, grouped by
    requested tolerance."""
    import numpy as np
    import oracle
    by = {}
    for r, (pot, fld, info) in zip(reqs, outs):
        n = len(r["q"])
        tgt = np.random.default_rng(n).choice(n, min(n, targets), replace=False)
        rp, _ = oracle.direct(r["x"], r["q"], targets=tgt)
        l2 = float(np.linalg.norm(pot[tgt] - rp) / np.linalg.norm(rp))
        mx = float((np.abs(pot[tgt] - rp) / np.maximum(np.abs(pot[tgt]), np.abs(rp))).max())
        d = by.setdefault(f"{r['tol']:g}", {"requests": 0, "met": 0, "worst_rel_l2": 0.0,
                                            "worst_max_rel": 0.0, "plans": set()})
        d["requests"] += 1
        d["met"] += int(l2 <= r["tol"])
        d["worst_rel_l2"] = max(d["worst_rel_l2"], l2)
        d["worst_max_rel"] = max(d["worst_max_rel"], mx)
        d["plans"].add(f"p={info['order']} {info['precision']}")
    for d in by.values():
        d["plans"] = sorted(d["plans"])
    return by


def run_serving_suite(nreq: int, rate: float) -> dict:
    """The served stream at the base rate (tolerance plans, with per-request
    errors, and plain FP64 at the same orders), then the planned stream at
    rates x4, x16 and all at once (saturation)."""
    import aran_gb300 as A
    reqs = serving_stream(nreq, rate)
    base = run_serving(reqs, keep=True)
    outs = base.pop("_outs")
    out = {"stream": (f"{nreq} Poisson arrivals, N log-uniform [1e3, 2e6], requested relative "
                      "potential error 1e-4 / 1e-6 / 1e-9, half uniform / half Plummer, leaf 64, "
                      "potential + field, 4 slots, 150 GB HBM admission budget"),
           "plans": {f"{t:g}": {"order": o, "precision": pr, "table_error": e}
                     for t, (o, pr, e) in ((t, A.plan_for_tolerance(t)) for t in TOLERANCES)},
           "base_rate_per_s": rate, "planned": base,
           "errors": serving_errors(reqs, outs)}
    del outs
    out["plain_fp64"] = run_serving(reqs, plain_fp64=True)
    sweep = []
    for k in (4.0, 16.0, 0.0):
        r = run_serving(reqs, rate_scale=k)
        r["rate_per_s"] = rate * k if k > 0 else "all at once"
        sweep.append(r)
    out["rate_sweep"] = sweep
    return out


# ------------------------------------------------------------------ batched
def _cpu_job2d(args):
    xy, q, order, maxbox = args
    import oracle
    t0 = time.perf_counter()
    oracle.solve2d(xy, q, [0, len(q)], [[-1.0, -1.0, 1.0, 1.0]], maxbox, order)
    return len(q), time.perf_counter() - t0


def run_batched_2d(nsys: int, steps: int, order: int = 20, maxbox: int = 32) -> dict:
    """Config 4, 2D part: one forest solve of nsys systems per step, in FP64
    and in mixed precision (FP32 scaled expansions and near-field arithmetic
    on FP64 differences, FP64 sums); the headline keys are the mixed run's."""
    import numpy as np
    import torch
    import aran_gb300 as A
    import oracle
    from aran_gb300 import workloads as W
    xy, q, offs, boxes = W.batch2d(nsys)
    n = len(q)
    dxy = torch.from_numpy(xy).cuda()
    dq = torch.from_numpy(q).cuda()
    dacc = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(9)
    check = [(int(offs[i]), int(offs[i + 1])) for i in rng.choice(nsys, 2, replace=False)]
    refs = []
    for a, b in check:
        tgt = rng.choice(b - a, min(500, b - a), replace=False).astype(np.int32)
        refs.append((a, b, tgt, oracle.direct2d(xy[a:b], q[a:b], tgt)))
    runs = {}
    for prec in ("fp64", "mixed"):
        r = {}
        with A.Solver2d(maxbox=maxbox, order=order, precision=prec) as s:
            for _ in range(2):
                s.solve_device(n, dxy.data_ptr(), dq.data_ptr(), dacc.data_ptr(), offs, boxes)
            dev_ms, stages = 0.0, []
            for _ in range(steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                s.solve_device(n, dxy.data_ptr(), dq.data_ptr(), dacc.data_ptr(), offs, boxes)
                st = s.timings()
                stages.append(st)
                dev_ms += st["total"]
            r["value"] = n * steps / (dev_ms * 1e-3)
            r["unit"] = UNIT
            r["ms_per_step"] = dev_ms / steps
            r["stage_ms"] = {k: round(statistics.mean(d[k] for d in stages), 3) for k in stages[0]}
            r["tree"] = s.tree_info()
            r["gpu_launches_per_step"] = s.launches()
            # end to end from pageable host arrays through the public call
            e2e_ms = 0.0
            for _ in range(steps):
                acc = s.solve(xy, q, offs, boxes)
                e2e_ms += s.timings()["total"]
            r["e2e"] = {"value": n * steps / (e2e_ms * 1e-3), "unit": UNIT,
                        "h2d_bytes_per_step": n * 24, "d2h_bytes_per_step": n * 16}
        worst, rl2 = 0.0, 0.0
        for a, b, tgt, ref in refs:
            got = acc[a:b][tgt]
            worst = max(worst, float((np.abs(got - ref) / np.maximum(np.abs(got), np.abs(ref))).max()))
            rl2 = max(rl2, float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
        r["accuracy"] = {"max_rel_vs_direct": worst, "rel_l2_vs_direct": rl2,
                         "systems": len(refs), "targets_each": 500}
        runs[prec] = r
    out = {"systems": nsys, "particles": n, "order": order, "maxbox": maxbox,
           "description": "N log-uniform in [1e3, 1e5], uniform in [-1,1]^2, q~U[-1,1], "
                          "sum_j q_j/(z_i - z_j) (tests/dummypot.c kernel)",
           "precision": "mixed"}
    out.update(runs["mixed"])
    out["fp64"] = runs["fp64"]
    out["speedup_vs_fp64_gpu"] = runs["fp64"]["ms_per_step"] / runs["mixed"]["ms_per_step"]
    # CPU: the oracle port on a sample of the systems, one process per core
    sample = [(xy[offs[i]:offs[i + 1]], q[offs[i]:offs[i + 1]], order, maxbox)
              for i in range(0, nsys, max(1, nsys // 32))][:32]
    procs = min(len(sample), os.cpu_count() or 1)
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(procs) as pool:
        done = sum(k for k, _ in pool.map(_cpu_job2d, sample))
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": done / el, "unit": UNIT, "cores": procs, "kind": "port",
                           "sample": f"{len(sample)} of the systems ({done} particles), one "
                                     f"single-threaded process each; {el:.1f} s wall"}
    return out


def run_batched_3d(nsys: int, check_systems: int = 8, steps: int = 3) -> dict:
    """Config 4, 3D part: the systems grouped by order, each group one
    forest solve (one octree per system, every level's kernels over the
    nodes of all systems of the group), the three groups on three solvers
    (streams) at once from host threads.  Host arrays in and out (pinned),
    copies inside the timed region; throughput = particles / wall time of
    all three; a sample of systems checked against the FP64 direct sum."""
    import threading

    import numpy as np
    import torch

    import aran_gb300 as A
    import oracle
    from aran_gb300 import workloads as W
    systems = W.batch3d(nsys)
    groups = {}
    for i, (x, q, p) in enumerate(systems):
        groups.setdefault(p, []).append(i)
    npart = sum(len(s[1]) for s in systems)
    data = {}
    for p, idx in groups.items():
        n = sum(len(systems[i][1]) for i in idx)
        hx = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
        hq = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
        hp = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
        hf = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
        offs = np.zeros(len(idx) + 1, np.int64)
        for k, i in enumerate(idx):
            x, q, _ = systems[i]
            offs[k + 1] = offs[k] + len(q)
            hx[offs[k]:offs[k + 1]] = x
            hq[offs[k]:offs[k + 1]] = q
        boxes = np.tile(np.array([0.0, 0.0, 0.0, 1.0, 1.0, 1.0]), (len(idx), 1))
        data[p] = (idx, offs, boxes, hx, hq, hp, hf)
    solvers = {p: A.Solver3d((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), maxbox=64, order=p, field=True,
                             precision="mixed") for p in groups}
    L = A.load()

    def solve(p):
        idx, offs, boxes, hx, hq, hp, hf = data[p]
        A._check(L.aran_gpu_solver3d_solve_forest(
            solvers[p]._h, len(idx), offs.ctypes.data_as(A.C.POINTER(A.C.c_int64)),
            boxes.ctypes.data_as(A.C.POINTER(A.C.c_double)), A.C.c_void_p(hx.ctypes.data),
            A.C.c_void_p(hq.ctypes.data), A.C.c_void_p(hp.ctypes.data),
            A.C.c_void_p(hf.ctypes.data), A.MEM_HOST))

    def all_at_once():
        ths = [threading.Thread(target=solve, args=(p,)) for p in sorted(groups)]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        return time.perf_counter() - t0

    all_at_once()                      # buffers sized, tables resident
    walls = [all_at_once() for _ in range(steps)]
    per_order = {}
    for p in sorted(groups):
        t0 = time.perf_counter()
        solve(p)
        w = time.perf_counter() - t0
        tm = solvers[p].timings()
        idx = data[p][0]
        per_order[str(p)] = {"systems": len(idx), "particles": int(data[p][1][-1]),
                             "wall_s_alone": w, "device_ms": tm["total"],
                             "stage_ms": {k: round(v, 3) for k, v in tm.items()},
                             "tree": solvers[p].tree_info()}
    worst = {}
    for i in np.random.default_rng(4).choice(nsys, check_systems, replace=False):
        x, q, p = systems[i]
        idx, offs, _, _, _, hp, _ = data[p]
        k = idx.index(i)
        pot = hp[offs[k]:offs[k + 1]]
        tgt = np.random.default_rng(i).choice(len(q), min(len(q), 300), replace=False)
        rp, _ = oracle.direct(x, q, targets=tgt)
        e = float(np.linalg.norm(pot[tgt] - rp) / np.linalg.norm(rp))
        worst[f"p={p}"] = max(worst.get(f"p={p}", 0.0), e)
    for sv in solvers.values():
        sv.close()
    wall = statistics.median(walls)
    return {"systems": nsys, "particles": npart, "precision": "mixed",
            "method": ("one forest solve per order (p=4, 8, 12), the three on their own "
                       "solvers and streams at once"),
            "description": (f"{nsys} systems of the config-4 3D stream: N log-uniform in "
                            "[1e3, 2e5], uniform in [0,1]^3 or 1-8 Gaussian blobs, p in "
                            "{4, 8, 12}, leaf 64, potential + field, pinned host arrays in and "
                            "out (copies timed)"),
            "value": npart / wall, "unit": UNIT, "wall_s": wall, "walls_s": walls,
            "systems_per_s": nsys / wall, "per_order": per_order,
            "accuracy": {"checked_systems": check_systems, "targets_each": 300,
                         "worst_rel_l2_vs_direct_by_order": worst}}


# ------------------------------------------------------------- CPU baseline
def run_flavours(steps: int, direct_targets: int) -> dict:
    """The uniform1m configuration (N=1M uniform, p=12, leaf 64, field) with
    both M2L flavours (rotate: point-and-shoot, kkylin: the reference's
    aransphericalseriesd-kkylin.c), mixed and FP64, each against the FP64
    direct sum on the same target sample."""
    import numpy as np
    import torch

    import aran_gb300 as A
    import oracle

    gen, n, p, maxbox, lb, ub, desc = WORKLOADS["uniform1m"]
    x, q = make_workload("uniform1m")
    dev = torch.device("cuda", torch.cuda.current_device())
    dx = torch.from_numpy(x).to(dev)
    dq = torch.from_numpy(q).to(dev)
    pot = torch.empty(n, dtype=torch.float64, device=dev)
    fld = torch.empty((n, 3), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    tgt = np.random.default_rng(5).choice(n, direct_targets, replace=False)
    rp, rf = oracle.direct(x, q, targets=tgt)

    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    out = {"workload": "uniform1m", "description": desc, "targets": direct_targets}
    for flavour in ("rotate", "kkylin"):
        for precision in ("mixed", "fp64"):
            k = steps if precision == "mixed" else 1
            with A.Solver3d(lb, ub, maxbox=maxbox, order=p, flavour=flavour, field=True,
                            precision=precision) as s:
                for _ in range(2):
                    s.solve_device(n, dx.data_ptr(), dq.data_ptr(), pot.data_ptr(),
                                   fld.data_ptr())
                ms = []
                for _ in range(k):
                    flush.fill_(1.0)
                    torch.cuda.synchronize()
                    s.solve_device(n, dx.data_ptr(), dq.data_ptr(), pot.data_ptr(),
                                   fld.data_ptr())
                    ms.append(s.timings())
                pm, fm = pot.cpu().numpy(), fld.cpu().numpy()
            tot = statistics.mean(d["total"] for d in ms)
            out[f"{flavour}_{precision}"] = {
                "value": n / (tot * 1e-3), "unit": UNIT, "ms_per_step": tot,
                "m2l_ms": statistics.mean(d["m2l"] for d in ms),
                "pot_vs_direct": rl2(pm[tgt], rp), "field_vs_direct": rl2(fm[tgt], rf)}
    return out


def run_c1(reps: int = 20) -> dict:
    """Config 1: N=10,000 uniform in [0,1]^3, q~U[-1,1], p=8, leaf 20, rotate,
    potential only (tests/newtonpot3.c's kernel).  GPU mixed and FP64 solves
    (device time and end to end from host arrays), the oracle's
    single-threaded solve on the host, errors against the FP64 direct sum on
    every particle."""
    import numpy as np

    import aran_gb300 as A
    import oracle
    from aran_gb300 import workloads as W

    x, q = W.uniform(10_000, 1)
    n = len(q)
    rp, _ = oracle.direct(x, q)

    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    out = {"workload": "c1", "description": "N=10,000 uniform in [0,1]^3, q~U[-1,1], p=8, "
                                            "leaf 20, rotate, potential"}
    for prec in ("mixed", "fp64"):
        with A.Solver3d(maxbox=20, order=8, field=False, precision=prec) as s:
            for _ in range(3):
                pot, _ = s.solve(x, q)
            dev, wall = [], []
            for _ in range(reps):
                t0 = time.perf_counter()
                pot, _ = s.solve(x, q)
                wall.append(time.perf_counter() - t0)
                dev.append(s.timings()["total"])
        out[prec] = {"value": n / (statistics.median(dev) * 1e-3), "unit": UNIT,
                     "device_ms": statistics.median(dev),
                     "e2e_ms": 1e3 * statistics.median(wall),
                     "pot_vs_direct": rl2(pot, rp)}
    t0 = time.perf_counter()
    opot, _ = oracle.solve(x, q, order=8, maxbox=20, field=False, nthreads=1)
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": n / el, "unit": UNIT, "cores": 1, "kind": "port",
                           "seconds": el, "pot_vs_direct": rl2(opot, rp),
                           "sample": "the whole workload, one solve, one thread"}
    return out


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline(x, q, name: str, max_solves: int = 1, budget_s: float = 0.0) -> dict:
    """Times the oracle port of the reference solver on the whole workload
    (same particles, order, leaf size, flavour, field): full solves with the
    per-node and per-leaf work spread over every host thread, max_solves of
    them or as many as fit in budget_s (at least one).  Also reports the
    particles per CPU-second (the one-core equivalent)."""
    import oracle
    oracle.build()
    gen, n, p, maxbox, lb, ub, desc = WORKLOADS[name]
    threads = os.cpu_count() or 1
    walls, cpus = [], []
    while len(walls) < max(1, max_solves):
        c0, t0 = time.process_time(), time.perf_counter()
        oracle.solve(x, q, order=p, maxbox=maxbox, flavour="rotate", field=True, lb=lb, ub=ub,
                     nthreads=threads)
        walls.append(time.perf_counter() - t0)
        cpus.append(time.process_time() - c0)
        if budget_s > 0 and sum(walls) + walls[-1] > budget_s:
            break
    wall = sum(walls)
    return {"value": len(walls) * len(q) / wall, "unit": UNIT, "cores": threads, "kind": "port",
            "solves": len(walls), "s_per_solve": wall / len(walls),
            "per_core_value": len(walls) * len(q) / sum(cpus),
            "cpu_model": cpu_model(),
            "sample": (f"the whole workload ({len(q)} particles, same p, leaf size, flavour, "
                       f"field): {len(walls)} full solve(s) by the C restatement of the "
                       f"reference solver, per-node/per-leaf work over {threads} host threads "
                       f"({wall / len(walls):.1f} s wall, {sum(cpus) / len(cpus):.0f} CPU-s "
                       "per solve); per_core_value = particles per CPU-second")}


# ----------------------------------------------------------------- GPU arm
# DRAM bytes of one k_m2l_lanes<12> launch on plummer4m (233,161 nodes,
# 38,977,626 M2L): ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum
# on one launch of that workload (-k regex:k_m2l_lanes -s 1 -c 1,
# --clock-control none): 154,687,232 B read + 128,904,192 B written
M2L_DRAM_BYTES_PLUMMER4M = 154_687_232 + 128_904_192


def run_gpu(args):
    import numpy as np
    import torch

    import aran_gb300 as A

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    gen, n, p, maxbox, lb, ub, desc = WORKLOADS[args.workload]
    x, q = make_workload(args.workload, seed_offset=rank)
    dev = torch.device("cuda", local)
    dx = torch.from_numpy(x).to(dev).contiguous()
    dq = torch.from_numpy(q).to(dev).contiguous()
    pot = torch.empty(n, dtype=torch.float64, device=dev)
    fld = torch.empty((n, 3), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def solve_dev(s):
        s.solve_device(n, dx.data_ptr(), dq.data_ptr(), pot.data_ptr(), fld.data_ptr())

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(s, fn, steps, label):
        """Device time of `steps` solves: the sum of the per-solve CUDA-event
        totals the library records on its launching stream (first to last
        operation of the solve, host-side tree-level syncs included), max over
        ranks.  The L2 flush between steps is outside those events.  The
        host wall clock around the loop is returned beside it."""
        barrier()
        t0 = time.perf_counter()
        stage = []
        launches = 0
        dev_ms = 0.0
        torch.cuda.nvtx.range_push(label)  # lets ncu select the timed launches
        for _ in range(steps):
            flush.fill_(1.0)           # evict L2 between steps (256 MB > 129 MB L2)
            torch.cuda.synchronize()
            fn(s)
            st = s.timings()
            stage.append(st)
            dev_ms += st["total"]
            launches += s.launches()
        torch.cuda.nvtx.range_pop()
        barrier()
        wall = time.perf_counter() - t0
        el = dev_ms * 1e-3
        if dist is not None:
            t = torch.tensor([el, wall], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el, wall = float(t[0].item()), float(t[1].item())
        stage[0]["_wall_s"] = wall
        return el, stage, launches

    def mean_stages(stages):
        return {k: round(statistics.mean(d[k] for d in stages), 4) for k in stages[0]
                if not k.startswith("_")}

    def run_order(order, precision, steps, warmup):
        """(seconds per step, stage ms, potential, field) of one configuration."""
        with A.Solver3d(lb, ub, maxbox=maxbox, order=order, flavour="rotate", field=True,
                        precision=precision) as s_:
            for _ in range(warmup):
                solve_dev(s_)
            el_, st_, _ = timed(s_, solve_dev, steps, f"order{order}_{precision}")
            return (el_ / steps, mean_stages(st_), pot.cpu().numpy().copy(),
                    fld.cpu().numpy().copy())

    # plain FP64 path on the same input (reference point of the metric)
    fp64_s, fp64_stages, pot64, fld64 = run_order(p, "fp64", max(1, args.fp64_steps),
                                                  max(1, min(args.warmup, 2)))

    s = A.Solver3d(lb, ub, maxbox=maxbox, order=p, flavour="rotate", field=True,
                   precision=args.precision)
    for _ in range(args.warmup):
        solve_dev(s)
    clocks = ClockSampler(local)
    clocks.start()
    el, stages, launches = timed(s, solve_dev, args.steps, "timed_device")
    clk = clocks.stop()
    potm = pot.cpu().numpy().copy()
    fldm = fld.cpu().numpy().copy()
    info = s.tree_info()
    stats = s.get_stats()

    # end to end through the host-pointer call: pinned host buffers, H2D and
    # D2H inside the timed region
    hx = torch.from_numpy(x).pin_memory()
    hq = torch.from_numpy(q).pin_memory()
    hpot = torch.empty(n, dtype=torch.float64).pin_memory()
    hfld = torch.empty((n, 3), dtype=torch.float64).pin_memory()

    def solve_host(s_):
        A._check(A.load().aran_gpu_solver3d_solve(
            s_._h, n, A.C.c_void_p(hx.data_ptr()), A.C.c_void_p(hq.data_ptr()),
            A.C.c_void_p(hpot.data_ptr()), A.C.c_void_p(hfld.data_ptr()), A.MEM_HOST))

    for _ in range(2):
        solve_host(s)
    el_e2e, st_e2e, _ = timed(s, solve_host, args.steps, "timed_e2e")
    wall_e2e = st_e2e[0].pop("_wall_s")
    s.close()

    # the clustered configuration at its other orders (mixed and FP64)
    orders = {}
    if rank == 0 and args.orders:
        for po in [int(v) for v in args.orders.split(",") if v]:
            ms_, stm_, pm_, fm_ = run_order(po, "mixed", max(1, min(args.steps, 5)), 2)
            m64_, st64_, p64_, f64_ = run_order(po, "fp64", 1, 1)
            orders[po] = {"mixed": {"value": n / ms_, "unit": UNIT, "ms_per_step": 1e3 * ms_,
                                    "stage_ms": stm_},
                          "fp64": {"value": n / m64_, "unit": UNIT, "ms_per_step": 1e3 * m64_},
                          "speedup_vs_fp64_gpu": m64_ / ms_,
                          "_arrays": (pm_, fm_, p64_, f64_)}

    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return

    # accuracy: mixed vs FP64 GPU path, both vs FP64 direct sum on a subset
    # of targets (the same subset for every order)
    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    acc = {"pot_vs_fp64_gpu": rl2(potm, pot64), "field_vs_fp64_gpu": rl2(fldm, fld64)}
    rp = rf = tgt = None
    if args.direct_targets > 0:
        import oracle
        tgt = np.random.default_rng(5).choice(n, args.direct_targets, replace=False)
        rp, rf = oracle.direct(x, q, targets=tgt)
        acc.update({"targets": args.direct_targets,
                    "pot_vs_direct": rl2(potm[tgt], rp), "field_vs_direct": rl2(fldm[tgt], rf),
                    "fp64_pot_vs_direct": rl2(pot64[tgt], rp),
                    "fp64_field_vs_direct": rl2(fld64[tgt], rf)})
    for po, d in orders.items():
        pm_, fm_, p64_, f64_ = d.pop("_arrays")
        a = {"pot_vs_fp64_gpu": rl2(pm_, p64_), "field_vs_fp64_gpu": rl2(fm_, f64_)}
        if tgt is not None:
            a.update({"pot_vs_direct": rl2(pm_[tgt], rp), "field_vs_direct": rl2(fm_[tgt], rf),
                      "fp64_pot_vs_direct": rl2(p64_[tgt], rp),
                      "fp64_field_vs_direct": rl2(f64_[tgt], rf)})
        d["accuracy"] = a
    orders[p] = {"mixed": {"value": n * args.steps / el, "unit": UNIT,
                           "ms_per_step": 1e3 * el / args.steps},
                 "fp64": {"value": n / fp64_s, "unit": UNIT, "ms_per_step": 1e3 * fp64_s},
                 "speedup_vs_fp64_gpu": fp64_s / (el / args.steps),
                 "accuracy": "see accuracy"}

    ms_step = 1e3 * el / args.steps
    value = world * n * args.steps / el
    wall_s = stages[0].pop("_wall_s")
    stage_ms = mean_stages(stages)
    # roofline of the dominant kernel (M2L): algorithmic flops per launch (the
    # operator's definition, F(p) per directed M2L) over its CUDA-event
    # duration recorded on the launching stream by the library
    m2l_s = stage_ms["m2l"] * 1e-3
    flops = info["far"] * m2l_flops_rotate(p)
    flops_applied = info["far"] * m2l_flops(p)
    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    smax = clk.get("sm_max_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * smax * 1e6 / 1e12
    achieved = flops / m2l_s / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    # algorithmic bytes of the launch: every node's multipole read and local
    # written once (FP32 complex), x2 as counted for expansions
    real = 4 if args.precision == "mixed" else 8
    alg_bytes = info["nodes"] * (p * (p + 1) // 2 + (p + 1) * (p + 2) // 2) * 2 * real * 2
    # the M2L kernel the library ran
    m2l_kernel = m2l_kernel_name(args.precision, p, os.environ.get("ARAN_M2L_KERNEL", ""))
    traffic = args.m2l_traffic
    if (traffic is None and args.workload == "plummer4m" and p == 12
            and m2l_kernel.startswith("k_m2l_lanes")):
        traffic = M2L_DRAM_BYTES_PLUMMER4M
    roof = {
        "kernel": m2l_kernel,
        "bound": "fp32",
        "achieved": round(achieved, 3), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
        "frac": round(achieved / fp32_peak, 4),
        "traffic": traffic,
        "peak_source": (f"FP32 CUDA-core peak: {sms} SMs (device property) x 128 FP32 lanes x 2 "
                        f"flop x {smax:.0f} MHz (max SM clock sampled by nvidia-smi); "
                        "MEASURED_PEAKS.json holds only HBM and bf16-tensor peaks and this "
                        "kernel runs on the FP32 pipes"),
        "flops_per_m2l": m2l_flops_rotate(p), "m2l_per_launch": info["far"],
        "flops_per_launch": flops,
        "as_applied": {"flops_per_m2l": m2l_flops(p), "flops_per_launch": flops_applied,
                       "achieved": round(flops_applied / m2l_s / 1e12, 3),
                       "frac": round(flops_applied / m2l_s / 1e12 / fp32_peak, 4)},
        "algorithmic_bytes": {"bytes_per_launch": alg_bytes,
                              "definition": "nodes x (multipole + local coefficients) x 8 B "
                                            "(FP32 complex) x 2",
                              "achieved_gbs": round(alg_bytes / m2l_s / 1e9, 1),
                              "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on "
                           "this workload" if traffic is not None else "not captured"),
        "stages": stage_rooflines(stage_ms, stats, info, n, p, fp32_peak,
                                  peaks.get("hbm_gbs") or 6800.0),
        "bf16_tensor_peak_tflops": peaks.get("bf16_tflops"),
        "tensor_frac": (round(achieved / peaks["bf16_tflops"], 4)
                        if peaks.get("bf16_tflops") else None),
    }
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded Plummer/uniform draws, no dataset)",
        "config": {"workload": args.workload, "description": desc, "n_per_gpu": n, "order": p,
                   "maxbox": maxbox, "flavour": "rotate", "precision": args.precision,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "flushed between steps by a 256 MB device write (outside the timed events)",
                   "timing": ("CUDA events on the solver's launching stream around each solve, "
                              "summed over the timed steps; max over ranks"),
                   "wall_ms_per_step": 1e3 * wall_s / args.steps},
        "fp64": {"value": world * n / fp64_s, "unit": UNIT, "ms_per_step": 1e3 * fp64_s,
                 "stage_ms": fp64_stages},
        "speedup_vs_fp64_gpu": fp64_s / (el / args.steps),
        "accuracy": acc,
        "orders": {str(k): orders[k] for k in sorted(orders)},
        "stage_ms": stage_ms,
        "tree": info, "stats": stats,
        "roofline": roof,
        "clocks": clk,
        "e2e": {"value": world * n * args.steps / el_e2e, "unit": UNIT,
                "ms_per_step": 1e3 * el_e2e / args.steps,
                "wall_ms_per_step": 1e3 * wall_e2e / args.steps,
                "h2d_bytes_per_step": n * 3 * 8 + n * 8,
                "d2h_bytes_per_step": n * 8 + n * 3 * 8},
        "gpu_launches": launches,
    }
    line["c1"] = run_c1()
    if args.flavours:
        line["flavours"] = run_flavours(max(1, min(args.steps, 5)), args.direct_targets or 10000)
    if args.serving_requests > 0:
        line["serving"] = run_serving_suite(args.serving_requests, args.serving_rate)
    if args.batched_2d_systems > 0 or args.batched_3d_systems > 0:
        line["batched"] = {}
        if args.batched_2d_systems > 0:
            line["batched"]["2d"] = run_batched_2d(args.batched_2d_systems, max(3, args.steps // 2))
        if args.batched_3d_systems > 0:
            line["batched"]["3d"] = run_batched_3d(args.batched_3d_systems)
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(x, q, args.workload, max_solves=1)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    gen, n, p, maxbox, lb, ub, desc = WORKLOADS[args.workload]
    x, q = make_workload(args.workload)
    res = cpu_baseline(x, q, args.workload, max_solves=args.steps, budget_s=args.ref_budget_s)
    line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": res["solves"],
            "warmup": 0, "ms_per_step": 1e3 * res["s_per_solve"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "n_per_gpu": n,
                       "order": p, "maxbox": maxbox, "flavour": "rotate",
                       "precision": "fp64 (reference algorithm)",
                       "steps_requested": args.steps,
                       "steps_note": ("full solves of the whole workload until --steps of them "
                                      f"or {args.ref_budget_s:.0f} s of wall time")},
            "cpu_baseline": res,
            "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plummer4m", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--orders", default="8,16",
                    help="other orders of the workload to run (mixed and FP64), comma-separated")
    ap.add_argument("--direct-targets", type=int, default=10000)
    ap.add_argument("--flavours", type=int, default=1,
                    help="also time uniform1m at p=12 with the rotate and kkylin M2L")
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--ref-budget-s", type=float, default=150.0,
                    help="--impl reference: wall-time budget for full CPU solves")
    ap.add_argument("--serving-requests", type=int, default=48)
    ap.add_argument("--serving-rate", type=float, default=16.0)
    ap.add_argument("--batched-2d-systems", type=int, default=512)
    ap.add_argument("--batched-3d-systems", type=int, default=2048)
    ap.add_argument("--m2l-traffic", type=float, default=None,
                    help="DRAM bytes of one M2L launch from an ncu capture of this workload")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
