"""The allocation-free near-field entry point against the solver's.

aran_gpu_p2p_direct_noalloc serves callers that may not allocate device
memory during a call; its scratch is a static device array shared by every
call.  Here it is called through the C ABI on device buffers and compared with
aran_gpu_solver3d_solve on the same particles (FP64, one leaf holding every
particle, so the solver's result is its P2P), twice in a row with different
inputs so the second call proves the shared scratch is cleared.  This file is
collected last.
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
def test_noalloc_matches_solver_twice(aran, field):
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


def test_noalloc_rejects_oversize(aran):
    with pytest.raises(aran.AranError) as ei:
        aran.p2p_direct_noalloc(aran.NOALLOC_MAX + 1, 1, 1, 1, None)
    assert ei.value.code == -1
    assert "capacity" in str(ei.value)
