"""The autotuner: it times every leaf capacity and M2L kernel offered on a
sample, keeps the fastest in the profile database without disturbing the
file's other groups, and a solver created with maxbox=0 then runs the tuned
configuration (same results as a solver given that configuration)."""
import ctypes as C

import numpy as np
import pytest

from aran_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_autotune_roundtrip(aran, tmp_path, monkeypatch):
    x, q = W.plummer(60000, 41)
    kw = dict(lbound=(-1, -1, -1), ubound=(1, 1, 1), order=10, precision="mixed", field=True)
    db = tmp_path / "profiledb.ini"
    db.write_text("[aran-profile]\naran_development3d_p2m=1e-7;\n")
    res = aran.autotune(x, q, maxboxes=(16, 32, 64), reps=2, db_path=str(db), **kw)
    # 3 leaf sizes x (default sibling + 6 sibling configurations) at order 10
    assert res["candidates"] == 21
    assert res["maxbox"] in (16, 32, 64) and res["ms"] > 0
    text = db.read_text()
    assert "[aran-profile]" in text and "aran_development3d_p2m=1e-7;" in text
    # operator costs under the reference's names, read back by the profile DB
    L = aran.load()
    L.aran_profile_db_read_file.argtypes = [C.c_char_p, C.c_char_p]
    L.aran_profile_db_name_eval.argtypes = [C.c_char_p, C.c_double]
    L.aran_profile_db_name_eval.restype = C.c_double
    assert L.aran_profile_db_read_file(str(db).encode(), None)
    for name in ("aran_development3d_m2l_rotate", "aran_development3d_m2m_rotate",
                 "aran_development3d_l2l_rotate", "aran_development3d_p2m",
                 "aran_development3d_l2p"):
        cost = L.aran_profile_db_name_eval(name.encode(), 10.0)
        assert 0 < cost < 1e-3, (name, cost)
    # the polynomial stays for other orders; the sample wins at order 10
    assert L.aran_profile_db_name_eval(b"aran_development3d_p2m", 3.0) == pytest.approx(1e-7)
    assert "p10-mixed-rotate-field=" in text and "samples-p10-mixed-rotate-field=" in text
    samples = text.split("samples-p10-mixed-rotate-field=")[1].splitlines()[0].split(";")
    assert len(samples) == 21
    looked = aran.tune_lookup(str(db), **kw)
    assert looked["maxbox"] == res["maxbox"] and looked["m2l_kernel"] == res["m2l_kernel"]
    # a second run replaces the entry rather than adding one
    aran.autotune(x, q, maxboxes=(32,), reps=1, db_path=str(db), **kw)
    assert db.read_text().count("p10-mixed-rotate-field=") == 2   # key + samples- key
    assert aran.tune_lookup(str(db), **kw)["maxbox"] == 32
    # maxbox=0: the solver takes the tuned configuration
    monkeypatch.setenv("ARAN_PROFILE_DB", str(db))
    lb, ub = kw["lbound"], kw["ubound"]
    t = aran.tune_lookup(str(db), **kw)
    with aran.Solver3d(lb, ub, maxbox=0, order=10, precision="mixed") as s0:
        p0, f0 = s0.solve(x, q)
        i0 = s0.tree_info()
    with aran.Solver3d(lb, ub, maxbox=t["maxbox"], order=10, precision="mixed") as s1:
        s1.set_m2l_kernel(t["m2l_kernel"], t["m2l_nst"], t["m2l_g"])
        p1, f1 = s1.solve(x, q)
        i1 = s1.tree_info()
    assert i0 == i1
    assert np.array_equal(p0, p1) or np.linalg.norm(p0 - p1) / np.linalg.norm(p1) < 1e-12


def test_m2l_kernel_argument_checks(aran):
    with aran.Solver3d(maxbox=32, order=10, precision="mixed") as s:
        for bad in ((7, 0, 0), (2, 4, 1), (2, 1, 0), (2, 0, 3)):
            with pytest.raises(aran.AranError):
                aran._check(aran.load().aran_gpu_solver3d_set_m2l_kernel(s._h, *bad))
