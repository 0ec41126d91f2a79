"""The allocation-free near-field entry point against the solver's.

aran_gpu_p2p_direct_noalloc serves callers that may not allocate device
memory during a call (a host that owns all device memory, or a loop that must
not meet cudaMalloc's implicit synchronisation); its scratch is a static
device array shared by every call.  Here it is called through the C ABI on
device buffers and compared with aran_gpu_solver3d_solve on the same
particles (FP64, one leaf holding every particle, so the solver's result is
its P2P) and with the oracle's FP64 direct sum, twice in a row with different
inputs so the second call proves the shared scratch is cleared.  After a
warm-up call the device's free memory is the same before and after a call.
This file is collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_noalloc(aran, x, q, field):
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    dx = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    dq = torch.from_numpy(np.ascontiguousarray(q)).to(dev)
    pot = torch.full((len(q),), float("nan"), dtype=torch.float64, device=dev)
    fld = torch.full((len(q), 3), float("nan"), dtype=torch.float64, device=dev) if field else None
    torch.cuda.synchronize()
    aran.p2p_direct_noalloc(len(q), dx.data_ptr(), dq.data_ptr(), pot.data_ptr(),
                            fld.data_ptr() if field else None)
    return pot.cpu().numpy(), (fld.cpu().numpy() if field else None)


def run_solver(aran, x, q, field):
    n = len(q)
    with aran.Solver3d((0, 0, 0), (1, 1, 1), maxbox=n, order=4, field=field,
                       precision="fp64") as s:
        return s.solve(x, q)


@pytest.mark.parametrize("field", [True, False])
def test_noalloc_matches_solver_twice(aran, oracle, field):
    rng = np.random.default_rng(123)
    for n in (3000, 1700):  # two calls in a row, the second smaller
        x = rng.uniform(0.0, 1.0, (n, 3))
        q = rng.uniform(-1.0, 1.0, n)
        pot, fld = run_noalloc(aran, x, q, field)
        rp, rf = run_solver(aran, x, q, field)
        assert np.all(np.isfinite(pot))
        assert rel_l2(pot, rp) < FP64_TOL
        if field:
            assert rel_l2(fld, rf) < FP64_TOL
        # the oracle's FP64 direct sum (no pair closer than 1e-5 here, so the
        # field guard removes nothing)
        op, of = oracle.direct(x, q)
        assert rel_l2(pot, op) < FP64_TOL
        if field:
            assert rel_l2(fld, of) < FP64_TOL


def test_noalloc_coincident_points(aran, oracle):
    """Copies of a particle are skipped like the particle itself (the
    potential-only rule of the solver and the oracle)."""
    rng = np.random.default_rng(7)
    x = rng.uniform(0.0, 1.0, (2000, 3))
    x[1990:] = x[:10]
    q = rng.uniform(-1.0, 1.0, 2000)
    pot, _ = run_noalloc(aran, x, q, False)
    op, _ = oracle.direct(x, q)
    assert np.all(np.isfinite(pot))
    assert rel_l2(pot, op) < FP64_TOL


def test_noalloc_allocates_nothing(aran):
    """After one warm-up call (which may load the library's device code on
    this device), a call leaves the device's free memory unchanged."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(5)
    n = 4096
    dx = torch.from_numpy(rng.uniform(0.0, 1.0, (n, 3))).to(dev)
    dq = torch.from_numpy(rng.uniform(-1.0, 1.0, n)).to(dev)
    pot = torch.empty(n, dtype=torch.float64, device=dev)
    fld = torch.empty((n, 3), dtype=torch.float64, device=dev)
    args = (n, dx.data_ptr(), dq.data_ptr(), pot.data_ptr(), fld.data_ptr())
    aran.p2p_direct_noalloc(*args)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    aran.p2p_direct_noalloc(*args)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0


def test_noalloc_rejects_oversize(aran):
    with pytest.raises(aran.AranError) as ei:
        aran.p2p_direct_noalloc(aran.NOALLOC_MAX + 1, 1, 1, 1, None)
    assert ei.value.code == -1
    assert "capacity" in str(ei.value)
