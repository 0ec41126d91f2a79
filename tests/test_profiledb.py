"""Operator cost database in LibAran's profiledb.ini format.

CPU: write/read round trip, lookup semantics (exact sample, else polynomial,
else NaN), groups and the ARAN_PROFILE_DB / ARAN_PROFILE_GROUP variables.
GPU: a database measured from the GPU kernels holds every operator at every
requested order with positive costs, and reads back.
"""
import math

import pytest

from aran_gb300 import profiledb as P


def test_round_trip_and_lookup(tmp_path, monkeypatch):
    prof = {"aran_development3d_m2l_rotate": {4: 1e-6, 8: 4e-6, 12: 9e-6},
            "p2p": {0: 2e-9}}
    path = tmp_path / "db.ini"
    P.write_ini(path, prof, degree=2)
    db = P.read_ini(str(path))
    assert db.eval("aran_development3d_m2l_rotate", 8) == pytest.approx(4e-6, rel=1e-5)
    # between samples: the polynomial (a quadratic through three points)
    assert 1e-6 < db.eval("aran_development3d_m2l_rotate", 6) < 4e-6
    assert db.eval("p2p", 0) == pytest.approx(2e-9, rel=1e-5)
    assert math.isnan(db.eval("missing", 3))
    # environment selects the file and the group
    monkeypatch.setenv("ARAN_PROFILE_DB", str(path))
    assert set(P.read_ini().names()) == set(prof)
    monkeypatch.setenv("ARAN_PROFILE_GROUP", "other")
    assert P.read_ini().names() == []


def test_reads_hand_written_groups(tmp_path):
    path = tmp_path / "h.ini"
    path.write_text("# comment\n[g1]\nf=1;2;\nsamples-f=1:10;2:20;\n[g2]\nf=5;\n")
    a = P.read_ini(str(path), "g1")
    assert a.eval("f", 1) == 10 and a.eval("f", 3) == 7
    assert P.read_ini(str(path), "g2").eval("f", 9) == 5


@pytest.mark.gpu
def test_measured_gpu_database(tmp_path):
    prof = P.measure_gpu(orders=(4, 8), n=50_000)
    for name in ("aran_development3d_m2l_rotate", "aran_development3d_m2m_kkylin",
                 "aran_development3d_l2l_rotate", "p2p", "p2m", "l2p"):
        assert set(prof[name]) == {4, 8}, name
        assert all(v > 0 for v in prof[name].values())
    path = tmp_path / "gpu.ini"
    P.write_ini(path, prof)
    db = P.read_ini(str(path))
    assert db.eval("aran_development3d_m2l_rotate", 8) == pytest.approx(
        prof["aran_development3d_m2l_rotate"][8], rel=1e-5)
