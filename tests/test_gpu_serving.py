"""The request loop (continuous batching of independent solves).

* every result is the same alone and in the mix: a burst of requests of
  different sizes, orders, distributions and precisions, served concurrently,
  matches each request solved alone (rel-L2 1e-10; the only difference is the
  order of FP64 atomic additions in the chunked near field);
* admission respects the HBM budget: requests whose footprints do not fit
  together never run at the same time; a request larger than the budget is
  refused at submission;
* a queued request can be cancelled; the others complete;
* every request that gives a tolerance instead of an order meets it: the
  server picks order and precision from its error table, and each result's
  potential is within the requested relative L2 error of the FP64 direct sum
  on a target sample (the reference checks each solve against the direct
  sum the same way, tests/newtonpot3.c:678-715).
"""
import numpy as np
import pytest

from aran_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def requests():
    rng = np.random.default_rng(77)
    out = []
    for i in range(10):
        n = int(np.exp(rng.uniform(np.log(2000), np.log(150000))))
        p = [6, 10, 16][i % 3]
        if i % 2:
            x, q = W.plummer(n, 200 + i)
            lb, ub = (-1, -1, -1), (1, 1, 1)
        else:
            x, q = W.uniform(n, 200 + i)
            lb, ub = (0, 0, 0), (1, 1, 1)
        prec = "mixed" if i % 4 else "fp64"
        out.append((x, q, dict(lbound=lb, ubound=ub, maxbox=32, order=p, field=True,
                               precision=prec)))
    return out


def test_same_alone_and_in_the_mix(aran):
    reqs = requests()
    alone = []
    for x, q, kw in reqs:
        kw2 = dict(kw)
        lb, ub = kw2.pop("lbound"), kw2.pop("ubound")
        with aran.Solver3d(lb, ub, **kw2) as s:
            alone.append(s.solve(x, q))
    with aran.Server(nslots=4, hbm_budget_bytes=100e9) as sv:
        tickets = [sv.submit(x, q, **kw) for x, q, kw in reqs]
        mixed = [sv.wait(t) for t in tickets]
    overlaps = 0
    infos = [m[2] for m in mixed]
    for i, a in enumerate(infos):
        for b in infos[i + 1:]:
            overlaps += a["start_s"] < b["end_s"] and b["start_s"] < a["end_s"]
    assert overlaps > 0, "requests should run concurrently"
    for (pa, fa), (pm, fm, info) in zip(alone, mixed):
        assert info["status"] == 0
        assert rel_l2(pm, pa) < TOL
        assert rel_l2(fm, fa) < TOL


def test_admission_budget(aran):
    n = 200_000
    fp = aran.footprint_bytes(n, maxbox=32, order=10, precision="mixed")
    with aran.Server(nslots=4, hbm_budget_bytes=1.5 * fp) as sv:
        tickets = []
        for i in range(3):
            x, q = W.uniform(n, 300 + i)
            tickets.append(sv.submit(x, q, maxbox=32, order=10, precision="mixed"))
        infos = [sv.wait(t)[2] for t in tickets]
        for i, a in enumerate(infos):
            for b in infos[i + 1:]:
                assert not (a["start_s"] < b["end_s"] and b["start_s"] < a["end_s"])
        x, q = W.uniform(2 * n, 9)
        with pytest.raises(aran.AranError) as ei:
            sv.submit(x, q, maxbox=32, order=10, precision="mixed")
        assert ei.value.code == -4


def test_cancel_queued_request(aran):
    with aran.Server(nslots=1, hbm_budget_bytes=100e9) as sv:
        big = W.uniform(400_000, 11)
        t0 = sv.submit(*big, maxbox=64, order=12, precision="fp64")
        small = [W.uniform(5000, 12 + i) for i in range(3)]
        ts = [sv.submit(*s, maxbox=32, order=6) for s in small]
        sv.cancel(ts[1])
        pot0, _, info0 = sv.wait(t0)
        assert info0["status"] == 0
        with pytest.raises(aran.AranError) as ei:
            sv.wait(ts[1])
        assert ei.value.code == -7
        for t in (ts[0], ts[2]):
            assert sv.wait(t)[2]["status"] == 0


TOLERANCES = (1e-4, 1e-6, 1e-9)


def test_served_results_meet_their_tolerance(aran, oracle):
    rng = np.random.default_rng(91)
    reqs = []
    for i in range(9):
        n = int(np.exp(rng.uniform(np.log(5000), np.log(60000))))
        if i % 2:
            x, q = W.plummer(n, 400 + i)
            lb, ub = (-1, -1, -1), (1, 1, 1)
        else:
            x, q = W.uniform(n, 400 + i)
            lb, ub = (0, 0, 0), (1, 1, 1)
        # order 0: the server picks order and precision from the tolerance
        reqs.append((x, q, TOLERANCES[i % 3],
                     dict(lbound=lb, ubound=ub, maxbox=32, order=0, field=True)))
    with aran.Server(nslots=4, hbm_budget_bytes=100e9) as sv:
        tickets = [sv.submit(x, q, tolerance=tol, **kw) for x, q, tol, kw in reqs]
        served = [sv.wait(t) for t in tickets]
    for (x, q, tol, _), (pot, fld, info) in zip(reqs, served):
        assert info["status"] == 0
        order, prec, _ = aran.plan_for_tolerance(tol)
        assert (info["order"], info["precision"]) == (order, prec)
        tg = np.random.default_rng(len(q)).choice(len(q), size=2000, replace=False)
        rp, _ = oracle.direct(x, q, targets=tg)
        assert rel_l2(pot[tg], rp) <= tol, (tol, len(q), order, prec)


def test_concurrent_orders_share_kernels(aran):
    """Requests of different orders run at once on the request loop's slots
    and launch the same kernels with different shared-memory sizes (FP64 at
    order 26 needs more than 128 KB in the M2M); each result equals the same
    solve alone."""
    reqs = []
    for i, p in enumerate((26, 8, 20, 12, 24, 6)):
        x, q = W.uniform(20000 + 1000 * i, 600 + i)
        reqs.append((x, q, p))
    alone = []
    for x, q, p in reqs:
        with aran.Solver3d(maxbox=32, order=p, field=True, precision="fp64") as s:
            alone.append(s.solve(x, q))
    with aran.Server(nslots=4, hbm_budget_bytes=100e9) as sv:
        tickets = [sv.submit(x, q, maxbox=32, order=p, field=True, precision="fp64")
                   for x, q, p in reqs]
        outs = [sv.wait(t) for t in tickets]
    for (pa, fa), (pm, fm, info) in zip(alone, outs):
        assert info["status"] == 0
        assert rel_l2(pm, pa) < TOL
        assert rel_l2(fm, fa) < TOL
