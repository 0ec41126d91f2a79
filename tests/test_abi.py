"""The C-ABI library builds, loads and exports every symbol include/*.h declares.

No compute call is made here; without a GPU the solver constructor must fail
loudly (ARAN_ERR_NO_DEVICE) rather than fall back to the CPU.
"""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "**", "*.h"), recursive=True):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:aran|vsg)_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def lib_path():
    import aran_gb300
    aran_gb300.load()
    return aran_gb300.LIB_PATH


def test_headers_declare_functions():
    names = declared_functions()
    assert "aran_gpu_solver3d_solve" in names
    # the LibAran-compatible API (aran/aransolver3d.h and friends)
    for n in ("aran_solver3d_new", "aran_solver3d_solve", "aran_solver3d_insert_point",
              "aran_development3d_m2l_rotate", "aran_development3d_new", "vsg_prtree3d_new_full",
              "aran_init"):
        assert n in names, n
    assert len(names) >= 50


def test_library_exports_every_declared_symbol():
    path = lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_library_loads_with_ctypes():
    L = C.CDLL(lib_path())
    for n in declared_functions():
        assert hasattr(L, n), n


def test_python_mirror_lists_exports():
    import aran_gb300
    for n in aran_gb300.EXPORTS:
        assert n in declared_functions()


def test_no_device_fails_loudly():
    import aran_gb300
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(aran_gb300.AranError) as ei:
        aran_gb300.Solver3d()
    assert ei.value.code == -3


def test_invalid_configs_rejected_before_device_use():
    import aran_gb300
    # (3D maxbox 0 is valid: the tuned leaf capacity)
    bad = [dict(order=0), dict(order=99), dict(maxbox=-1), dict(max_depth=30),
           dict(precision=7)]
    for kw in bad:
        with pytest.raises(aran_gb300.AranError) as ei:
            aran_gb300.Solver3d(**kw)
        assert ei.value.code == -1, kw
    with pytest.raises(aran_gb300.AranError) as ei:
        aran_gb300.Solver3d((0, 0, 0), (0, 1, 1))
    assert ei.value.code == -1
    for kw in (dict(order=0), dict(order=65), dict(maxbox=0), dict(max_depth=22)):
        with pytest.raises(aran_gb300.AranError) as ei:
            aran_gb300.Solver2d(**kw)
        assert ei.value.code == -1, kw


def test_tolerance_plan():
    """The request loop's tolerance -> (order, precision) plan (host-only)."""
    import aran_gb300 as A
    plans = [A.plan_for_tolerance(t) for t in (1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9, 1e-10)]
    for tol, (order, prec, est) in zip((1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9), plans):
        assert est <= 0.5 * tol and prec in ("mixed", "fp64")
    # below the table's best error: the highest tabulated order in FP64
    assert plans[7][:2] == (30, "fp64") and plans[7][2] > 0.5e-10
    assert plans[1][:2] == (8, "mixed") and plans[3][:2] == (16, "mixed")
    assert plans[6][:2] == (26, "fp64")
    # mixed is preferred while its floor allows; tighter plans never lower the order
    assert [p[1] for p in plans[:4]] == ["mixed"] * 4 and plans[4][1] == "fp64"
    fp64_orders = [p[0] for p in plans if p[1] == "fp64"]
    assert fp64_orders == sorted(fp64_orders)
    # a given order only picks the precision
    assert A.plan_for_tolerance(1e-4, order=12)[:2] == (12, "mixed")
    assert A.plan_for_tolerance(1e-8, order=20)[:2] == (20, "fp64")
    with pytest.raises(A.AranError):
        A.plan_for_tolerance(0.0)


def test_tune_lookup(tmp_path):
    """The autotuner's entries are read from the profile database (host only):
    the key names order, precision, flavour and field; other groups of the
    file do not matter; a malformed entry is an error, a missing one None."""
    import aran_gb300 as A
    db = tmp_path / "profiledb.ini"
    db.write_text("[aran-profile]\naran_development3d_m2l_rotate=1e-6;2e-7;\n\n"
                  "[aran-gpu-tune]\n# tuned on a sample\n"
                  "p12-mixed-rotate-field=maxbox=48;m2l=1;nst=0;g=0;ms=24.5\n"
                  "p10-mixed-rotate-field=maxbox=32;m2l=2;nst=3;g=2;ms=40.0\n"
                  "p8-fp64-rotate-pot=maxbox=sixteen;m2l=0\n")
    r = A.tune_lookup(str(db), order=12, precision="mixed")
    assert r == {"maxbox": 48, "m2l_kernel": "lanes", "m2l_nst": 0, "m2l_g": 0, "ms": 24.5,
                 "candidates": 0}
    r = A.tune_lookup(str(db), order=10, precision="mixed")
    assert (r["maxbox"], r["m2l_kernel"], r["m2l_nst"], r["m2l_g"]) == (32, "sibling", 3, 2)
    assert A.tune_lookup(str(db), order=12, precision="fp64") is None
    assert A.tune_lookup(str(db), order=12, precision="mixed", field=False) is None
    with pytest.raises(A.AranError):
        A.tune_lookup(str(db), order=8, precision="fp64", field=False)
    assert A.tune_lookup(str(tmp_path / "absent.ini"), order=12) is None
