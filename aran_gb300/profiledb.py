"""Operator cost database in LibAran's ``profiledb.ini`` format.

LibAran keeps per-operator cost models in a GKeyFile (aran/aranprofiledb.c):
group ``[aran-profile]`` (or ``$ARAN_PROFILE_GROUP``), file
``$ARAN_PROFILE_DB``; for every operator symbol a key holding the ascending
coefficients of a polynomial in the order p (``name=c0;c1;...;``) and a key
``samples-name`` holding measured ``p:seconds`` pairs.  A lookup returns the
sample at exactly p when there is one, else the polynomial's value, else NaN
(aran_profile_db_name_eval, aranprofiledb.c:276-296).  The solver turns the
p2p/p2l/m2p costs into its semifar threshold (aransolver3d.c:687-740,
1090-1127).

``measure_gpu`` fills such a database from the GPU kernels: it times whole
solves at each order and divides each stage's CUDA-event time by the number
of operations the stage performed, giving the amortised cost of one
operator call on the GPU under the operator names of the reference, so
programs that read the file get the costs of the path that actually runs.
"""
from __future__ import annotations

import math
import os

import numpy as np

DEFAULT_GROUP = "aran-profile"
SAMPLES_PREFIX = "samples-"

# stage timing -> (operator key suffix, stats counter)
_STAGES = (("m2m", "m2m"), ("m2l", "m2l"), ("l2l", "l2l"))
_FLAVOUR_SUFFIX = {"normal": "", "kkylin": "_kkylin", "rotate": "_rotate"}


def _fmt(v: float) -> str:
    return repr(float(v))


def write_ini(path, profiles: dict, group: str = DEFAULT_GROUP, degree: int = 4) -> None:
    """profiles: name -> {order: seconds}.  Writes samples and a least-squares
    polynomial of the given degree (fewer coefficients when there are fewer
    samples), one comment line per operator with the fit's chi-square."""
    lines = ["# Aran profiling configuration file", "", f"[{group}]"]
    for name in sorted(profiles):
        samples = dict(sorted(profiles[name].items()))
        x = np.array(list(samples.keys()), np.float64)
        y = np.array(list(samples.values()), np.float64)
        deg = min(degree, len(x) - 1)
        coef = np.polynomial.polynomial.polyfit(x, y, deg) if len(x) else np.zeros(1)
        chisq = float(np.sum((np.polynomial.polynomial.polyval(x, coef) - y) ** 2)
                      / np.maximum(np.sum(y ** 2), 1e-300)) if len(x) else 0.0
        lines.append(f'# "{name}" function fitting: chisq={chisq:g}')
        lines.append(f"{name}=" + "".join(_fmt(c) + ";" for c in coef))
        lines.append(f"{SAMPLES_PREFIX}{name}="
                     + "".join(f"{int(k) if float(k).is_integer() else k}:{v:g};"
                               for k, v in samples.items()))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


class ProfileDB:
    """Polynomials and samples of one group of a profile database."""

    def __init__(self, poly: dict, samples: dict):
        self.poly = poly
        self.samples = samples

    def eval(self, name: str, x: float) -> float:
        s = self.samples.get(name)
        if s is not None and float(x) in s:
            return s[float(x)]
        c = self.poly.get(name)
        if c is None:
            return math.nan
        return float(np.polynomial.polynomial.polyval(float(x), np.asarray(c)))

    def names(self):
        return sorted(set(self.poly) | set(self.samples))


def read_ini(path: str | None = None, group: str | None = None) -> ProfileDB:
    """Reads ``path`` (default ``$ARAN_PROFILE_DB``) at ``group`` (default
    ``$ARAN_PROFILE_GROUP``, then ``aran-profile``)."""
    path = path or os.environ.get("ARAN_PROFILE_DB")
    if not path:
        raise FileNotFoundError("no profile database: pass a path or set ARAN_PROFILE_DB")
    group = group or os.environ.get("ARAN_PROFILE_GROUP") or DEFAULT_GROUP
    poly, samples = {}, {}
    cur = None
    with open(path) as fh:
        for raw in fh:
            line = raw.strip()
            if not line or line.startswith("#"):
                continue
            if line.startswith("[") and line.endswith("]"):
                cur = line[1:-1].strip()
                continue
            if cur != group or "=" not in line:
                continue
            key, val = (t.strip() for t in line.split("=", 1))
            items = [t for t in val.split(";") if t.strip()]
            if key.startswith(SAMPLES_PREFIX):
                d = {}
                for it in items:
                    k, _, v = it.partition(":")
                    try:
                        d[float(k)] = float(v)
                    except ValueError:
                        continue
                samples[key[len(SAMPLES_PREFIX):]] = d
            else:
                poly[key] = [float(t) for t in items]
    return ProfileDB(poly, samples)


def measure_gpu(orders=(4, 6, 8, 10, 12), n: int = 200_000, flavours=("rotate", "kkylin"),
                precision: str = "fp64", seed: int = 3) -> dict:
    """Amortised GPU cost per operator call, seconds, keyed by the
    reference's operator names (aran_development3d_m2l_rotate, ...) plus the
    Newton callbacks p2p (per pair), p2m and l2p (per point)."""
    import aran_gb300 as A
    from aran_gb300 import workloads as W
    x, q = W.uniform(n, seed)
    out: dict = {}
    for flavour in flavours:
        suffix = _FLAVOUR_SUFFIX[flavour]
        for p in orders:
            with A.Solver3d((0, 0, 0), (1, 1, 1), maxbox=64, order=p, flavour=flavour,
                            field=True, precision=precision) as s:
                s.solve(x, q)                      # tables and buffers
                s.solve(x, q)
                ms, st = s.timings(), s.get_stats()
            for stage, counter in _STAGES:
                if st[counter] > 0:
                    out.setdefault(f"aran_development3d_{stage}{suffix}", {})[p] = \
                        ms[stage] * 1e-3 / st[counter]
            if flavour == flavours[0]:
                for stage, counter in (("p2m", "p2m"), ("l2p", "l2p"), ("p2p", "p2p")):
                    if st[counter] > 0:
                        out.setdefault(stage, {})[p] = ms[stage] * 1e-3 / st[counter]
    return out
