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

``--impl reference`` times the reference algorithm on the host cores: the
C restatement of LibAran's solver in oracle/ (the reference itself needs
glib and libvsg, which are not available), one independent process per core
on bounded samples of the same workload.

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
}


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
def serving_stream(nreq: int, rate: float, seed: int = 5):
    """Poisson arrivals of 3D potential+field solves: N log-uniform in
    [1e3, 2e6], requested tolerance 1e-4/1e-6/1e-9 -> p = 6/10/16, half
    uniform in [0,1]^3, half Plummer in [-1,1]^3."""
    import numpy as np
    from aran_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    reqs = []
    for i in range(nreq):
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(2e6))))
        p = (6, 10, 16)[int(rng.integers(0, 3))]
        if rng.uniform() < 0.5:
            x, q = W.uniform(n, 1000 + i)
            lb, ub = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
        else:
            x, q = W.plummer(n, 1000 + i)
            lb, ub = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)
        reqs.append((float(arrivals[i]), x, q, dict(lbound=lb, ubound=ub, maxbox=64, order=p,
                                                     field=True)))
    return reqs


def run_serving(reqs, precision: str, nslots: int = 4, budget: float = 150e9) -> dict:
    import numpy as np
    import aran_gb300 as A
    with A.Server(nslots=nslots, hbm_budget_bytes=budget) as sv:
        # one warm request per configuration so table builds stay out of the stream
        seen = set()
        for _, x, q, kw in reqs:
            key = (kw["order"], kw["lbound"])
            if key not in seen:
                seen.add(key)
                sv.wait(sv.submit(x[:2000], q[:2000], precision=precision, **kw))
        t0 = time.perf_counter()
        tickets = []
        for arr, x, q, kw in reqs:
            dt = arr - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets.append(sv.submit(x, q, precision=precision, **kw))
        infos = [sv.wait(t)[2] for t in tickets]
    lat = np.array([i["end_s"] - i["submit_s"] for i in infos])
    span = max(i["end_s"] for i in infos) - min(i["submit_s"] for i in infos)
    npart = sum(len(r[2]) for r in reqs)
    return {"precision": precision, "requests": len(reqs),
            "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "throughput": npart / span, "unit": UNIT,
            "mean_queue_ms": float(np.mean([i["start_s"] - i["submit_s"] for i in infos]) * 1e3)}


# ------------------------------------------------------------------ batched
def _cpu_job2d(args):
    xy, q, order, maxbox = args
    import oracle
    t0 = time.perf_counter()
    oracle.solve2d(xy, q, [0, len(q)], [[-1.0, -1.0, 1.0, 1.0]], maxbox, order)
    return len(q), time.perf_counter() - t0


def run_batched_2d(nsys: int, steps: int, order: int = 20, maxbox: int = 32) -> dict:
    """Config 4, 2D part: one forest solve of nsys systems per step."""
    import numpy as np
    import torch
    import aran_gb300 as A
    from aran_gb300 import workloads as W
    xy, q, offs, boxes = W.batch2d(nsys)
    n = len(q)
    dxy = torch.from_numpy(xy).cuda()
    dq = torch.from_numpy(q).cuda()
    dacc = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {"systems": nsys, "particles": n, "order": order, "maxbox": maxbox,
           "description": "N log-uniform in [1e3, 1e5], uniform in [-1,1]^2, q~U[-1,1], "
                          "sum_j q_j/(z_i - z_j) (tests/dummypot.c kernel), FP64"}
    with A.Solver2d(maxbox=maxbox, order=order) as s:
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
        out["value"] = n * steps / (dev_ms * 1e-3)
        out["unit"] = UNIT
        out["ms_per_step"] = dev_ms / steps
        out["stage_ms"] = {k: round(statistics.mean(d[k] for d in stages), 3) for k in stages[0]}
        out["tree"] = s.tree_info()
        out["gpu_launches_per_step"] = s.launches()
        # end to end from pageable host arrays through the public call
        e2e_ms = 0.0
        for _ in range(steps):
            acc = s.solve(xy, q, offs, boxes)
            e2e_ms += s.timings()["total"]
        out["e2e"] = {"value": n * steps / (e2e_ms * 1e-3), "unit": UNIT,
                      "h2d_bytes_per_step": n * 24, "d2h_bytes_per_step": n * 16}
    # accuracy on two systems against the FP64 direct sum (500 targets each)
    import oracle
    rng = np.random.default_rng(9)
    worst, rl2 = 0.0, 0.0
    for i in rng.choice(nsys, 2, replace=False):
        a, b = int(offs[i]), int(offs[i + 1])
        tgt = rng.choice(b - a, min(500, b - a), replace=False).astype(np.int32)
        ref = oracle.direct2d(xy[a:b], q[a:b], tgt)
        got = acc[a:b][tgt]
        worst = max(worst, float((np.abs(got - ref) / np.maximum(np.abs(got), np.abs(ref))).max()))
        rl2 = max(rl2, float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    out["accuracy"] = {"max_rel_vs_direct": worst, "rel_l2_vs_direct": rl2}
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


def run_batched_3d(nsys: int, precision: str = "mixed", nslots: int = 4) -> dict:
    """Config 4, 3D part: every system a request of the request loop, all
    submitted at once; throughput = particles / (last end - first submit)."""
    import numpy as np
    import aran_gb300 as A
    from aran_gb300 import workloads as W
    systems = W.batch3d(nsys)
    kw = dict(lbound=(0.0, 0.0, 0.0), ubound=(1.0, 1.0, 1.0), maxbox=64, field=True,
              precision=precision)
    with A.Server(nslots=nslots, hbm_budget_bytes=150e9) as sv:
        for p in (4, 8, 12):   # resident solvers per order in every slot
            for t in [sv.submit(systems[0][0][:2000], systems[0][1][:2000], order=p, **kw)
                      for _ in range(nslots)]:
                sv.wait(t)
        tickets = [sv.submit(x, q, order=p, **kw) for x, q, p in systems]
        infos = [sv.wait(t)[2] for t in tickets]
    span = max(i["end_s"] for i in infos) - min(i["submit_s"] for i in infos)
    npart = sum(len(s[1]) for s in systems)
    return {"systems": nsys, "particles": npart, "precision": precision, "slots": nslots,
            "description": (f"the first {nsys} draws of the config-4 3D stream (2,048 "
                            "systems): N log-uniform in [1e3, 2e5], uniform in [0,1]^3 or 1-8 "
                            "Gaussian blobs, p in {4, 8, 12}, leaf 64, potential + field, "
                            "host arrays in and out"),
            "value": npart / span, "unit": UNIT, "wall_s": span}


# ------------------------------------------------------------- CPU baseline
def _cpu_job(args):
    name, n_sample, seed = args
    import numpy as np
    import oracle
    from aran_gb300 import workloads as W
    gen, n, p, maxbox, lb, ub, desc = WORKLOADS[name]
    x, q = getattr(W, gen)(n_sample, 100 + seed)
    t0 = time.perf_counter()
    oracle.solve(x, q, order=p, maxbox=maxbox, flavour="rotate", field=True, lb=lb, ub=ub)
    return n_sample, time.perf_counter() - t0


def cpu_baseline(name: str, n_sample: int, procs: int, rounds: int = 1) -> dict:
    """Times the oracle port of the reference solver: `procs` independent
    single-threaded processes (the reference has no threading), each solving
    its own n_sample-particle draw of the workload distribution."""
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    total_n, t0 = 0, time.perf_counter()
    with ctx.Pool(procs) as pool:
        for r in range(rounds):
            for n_done, _ in pool.map(_cpu_job, [(name, n_sample, r * procs + i) for i in range(procs)]):
                total_n += n_done
    el = time.perf_counter() - t0
    return {"value": total_n / el, "unit": UNIT, "cores": procs, "kind": "port",
            "sample": f"{procs} processes x {rounds} round(s), each a full solve of its own "
                      f"{n_sample}-particle draw of the workload distribution "
                      f"(same p, leaf size, flavour, field); {el:.1f} s wall"}


# ----------------------------------------------------------------- GPU arm
# DRAM bytes of the FP32 M2L launch per tree node: ncu capture of
# k_m2l_lanes<12> on uniform1m (37449 nodes), dram__bytes_read.sum +
# dram__bytes_write.sum = 26.004224 MB + 0.010496 MB
# (profiles/m2l_lanes_uniform1m_p12_mixed.md)
M2L_DRAM_BYTES_PER_NODE = (26.004224e6 + 0.010496e6) / 37449


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

    results = {}
    # plain FP64 path on the same input (reference point of the metric)
    with A.Solver3d(lb, ub, maxbox=maxbox, order=p, flavour="rotate", field=True,
                    precision="fp64") as s64:
        for _ in range(max(1, min(args.warmup, 2))):
            solve_dev(s64)
        el64, st64, _ = timed(s64, solve_dev, max(1, args.fp64_steps), "timed_fp64")
        pot64 = pot.cpu().numpy().copy()
        fld64 = fld.cpu().numpy().copy()
        results["fp64_s_per_step"] = el64 / max(1, args.fp64_steps)
        st64[0].pop("_wall_s")
        results["fp64_stage_ms"] = {k: round(statistics.mean(d[k] for d in st64), 3) for k in st64[0]}

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

    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return

    # accuracy: mixed vs FP64 GPU path, both vs FP64 direct sum on a subset
    def rl2(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    acc = {"pot_vs_fp64_gpu": rl2(potm, pot64), "field_vs_fp64_gpu": rl2(fldm, fld64)}
    if args.direct_targets > 0:
        import oracle
        tgt = np.random.default_rng(5).choice(n, args.direct_targets, replace=False)
        rp, rf = oracle.direct(x, q, targets=tgt)
        acc.update({"targets": args.direct_targets,
                    "pot_vs_direct": rl2(potm[tgt], rp), "field_vs_direct": rl2(fldm[tgt], rf),
                    "fp64_pot_vs_direct": rl2(pot64[tgt], rp),
                    "fp64_field_vs_direct": rl2(fld64[tgt], rf)})

    ms_step = 1e3 * el / args.steps
    value = world * n * args.steps / el
    wall_s = stages[0].pop("_wall_s")
    stage_ms = {k: round(statistics.mean(d[k] for d in stages), 4) for k in stages[0]}
    # roofline of the dominant kernel (M2L): algorithmic flops per launch over
    # its CUDA-event duration (recorded on the launching stream by the library)
    flops = info["far"] * m2l_flops(p)
    m2l_s = stage_ms["m2l"] * 1e-3
    smax = clk.get("sm_max_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * smax * 1e6 / 1e12
    achieved = flops / m2l_s / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    # algorithmic bytes of the M2L launch: every far source multipole and every
    # written local once (FP32 complex), at the HBM roofline
    alg_bytes = (info["far"] * (p * (p + 1) // 2) + info["nodes"] * ((p + 1) * (p + 2) // 2)) * 8
    roof = {
        "kernel": ("k_m2l_sibling<float> (rotate M2L, all levels, one launch)"
                   if os.environ.get("ARAN_M2L_KERNEL") == "sibling" or p not in (8, 12)
                   or args.precision != "mixed" else
                   f"k_m2l_lanes<{p}> (rotate M2L, FP32 lane pairs, all levels, one launch)"),
        "bound": "fp32",
        "achieved": round(achieved, 3), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
        "frac": round(achieved / fp32_peak, 4),
        "peak_source": ("FP32 CUDA-core peak 152 SMs x 128 lanes x 2 flop x max SM clock; "
                        "MEASURED_PEAKS.json holds only HBM and bf16-tensor peaks, and this "
                        "kernel runs on the FP32 pipes"),
        "flops_per_launch": flops, "m2l_per_launch": info["far"],
        "flops_per_m2l": m2l_flops(p),
        "hbm_view": {"bytes_per_launch": alg_bytes,
                     "achieved_gbs": round(alg_bytes / m2l_s / 1e9, 1),
                     "peak_gbs": peaks.get("hbm_gbs", 6803.8),
                     "frac": round(alg_bytes / m2l_s / 1e9 / peaks.get("hbm_gbs", 6803.8), 4)},
        # DRAM bytes per launch: ncu capture of this kernel on uniform1m,
        # 694 B per tree node, scaled by this tree's node count
        "traffic": (args.m2l_traffic if args.m2l_traffic is not None
                    else round(M2L_DRAM_BYTES_PER_NODE * info["nodes"])),
        "traffic_source": ("--m2l-traffic" if args.m2l_traffic is not None else
                           "ncu dram__bytes_read.sum+write.sum of the uniform1m launch, "
                           "scaled by node count"),
        "bf16_tensor_peak_tflops": peaks.get("bf16_tflops"),
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
        "fp64": {"value": world * n / results["fp64_s_per_step"], "unit": UNIT,
                 "ms_per_step": 1e3 * results["fp64_s_per_step"],
                 "stage_ms": results["fp64_stage_ms"]},
        "speedup_vs_fp64_gpu": (value / world) / (n / results["fp64_s_per_step"]),
        "accuracy": acc,
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
    if args.serving_requests > 0:
        reqs = serving_stream(args.serving_requests, args.serving_rate)
        line["serving"] = {
            "stream": (f"{args.serving_requests} Poisson arrivals at {args.serving_rate}/s, N "
                       "log-uniform [1e3, 2e6], p in {6,10,16}, half uniform / half Plummer, "
                       "4 slots, 150 GB HBM admission budget"),
            "mixed": run_serving(reqs, "mixed"),
            "fp64": run_serving(reqs, "fp64"),
        }
    if args.batched_2d_systems > 0 or args.batched_3d_systems > 0:
        line["batched"] = {}
        if args.batched_2d_systems > 0:
            line["batched"]["2d"] = run_batched_2d(args.batched_2d_systems, max(3, args.steps // 2))
        if args.batched_3d_systems > 0:
            line["batched"]["3d"] = run_batched_3d(args.batched_3d_systems)
    if args.cpu_baseline:
        procs = args.cpu_procs or os.cpu_count() or 1
        line["cpu_baseline"] = cpu_baseline(args.workload, args.cpu_sample, procs)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    gen, n, p, maxbox, lb, ub, desc = WORKLOADS[args.workload]
    procs = args.cpu_procs or os.cpu_count() or 1
    for _ in range(args.warmup if args.ref_warmup else 0):
        cpu_baseline(args.workload, max(2000, args.cpu_sample // 10), procs)
    res = cpu_baseline(args.workload, args.cpu_sample, procs, rounds=args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "order": p,
                       "maxbox": maxbox, "flavour": "rotate", "precision": "fp64 (reference)"},
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
    ap.add_argument("--direct-targets", type=int, default=1000)
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--cpu-sample", type=int, default=20000)
    ap.add_argument("--cpu-procs", type=int, default=0)
    ap.add_argument("--ref-warmup", type=int, default=0)
    ap.add_argument("--serving-requests", type=int, default=48)
    ap.add_argument("--serving-rate", type=float, default=16.0)
    ap.add_argument("--batched-2d-systems", type=int, default=512)
    ap.add_argument("--batched-3d-systems", type=int, default=512)
    ap.add_argument("--m2l-traffic", type=float, default=None,
                    help="dram bytes per M2L launch from an ncu capture (profiles/)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
