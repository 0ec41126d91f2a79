"""TEST INFRASTRUCTURE: builds the reference's own operator layer.

The operator/math files of LibAran (aran/aransphericalseriesd*.c,
aranwigner*.c, aransphericalharmonic.c, aranlegendre.c, aranbinomial.c,
arandevelopment{2,3}d.c, aranlaurentseriesd.c) are compiled unmodified,
where they lie in the reference tree, against the glib/libvsg shims of
oracle/refshim/ into oracle/_ref/libaranref.so.  The two coefficient-buffer
sources the reference's build generates from templates
(aran/arancoefficientbuffer@t@.{c,h}, aran/aranbinomialbuffer@t@.{c,h};
aran/Makefile.am:83-93 with gencode/typegens.py) are made here for the
gdouble type by the same @name@ substitution, into oracle/_ref/gen/.

Only the oracle's pinning tests load the result; it is rebuilt when the
reference tree is present (oracle.build()) and absent otherwise.
"""
from __future__ import annotations

import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("ARAN_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
LIB = os.path.join(OUT, "libaranref.so")

SOURCES = ["aransphericalseriesd.c", "aransphericalseriesd-translate.c",
           "aransphericalseriesd-kkylin.c", "aransphericalseriesd-rotate.c", "aranwigner.c",
           "aranwignerrepo.c", "aransphericalharmonic.c", "aranlegendre.c", "aranbinomial.c",
           "arandevelopment3d.c", "aranlaurentseriesd.c", "arandevelopment2d.c"]
TEMPLATES = ["arancoefficientbuffer@t@.c", "arancoefficientbuffer@t@.h",
             "aranbinomialbuffer@t@.c", "aranbinomialbuffer@t@.h"]
# the gdouble entry of the reference's types.list
DOUBLE = {"type": "gdouble", "t": "d", "TYPE": "DOUBLE", "T": "D"}


def available() -> bool:
    return os.path.isdir(os.path.join(REF, "aran"))


def _substitute(text: str, table: dict) -> str:
    for k, v in table.items():
        text = re.sub("@%s@" % k, v, text)
    return text


def generate() -> list[str]:
    os.makedirs(GEN, exist_ok=True)
    out = []
    for t in TEMPLATES:
        src = os.path.join(REF, "aran", t)
        dst = os.path.join(GEN, _substitute(t, DOUBLE))
        text = _substitute(open(src).read(), DOUBLE)
        if not os.path.exists(dst) or open(dst).read() != text:
            with open(dst, "w") as fh:
                fh.write(text)
        out.append(dst)
    return [p for p in out if p.endswith(".c")]


def build(force: bool = False) -> str | None:
    """Compile into oracle/_ref/libaranref.so; None without the reference."""
    if not available():
        return None
    srcs = [os.path.join(REF, "aran", s) for s in SOURCES]
    shim = [os.path.join(HERE, "refshim", "shim.c")]
    deps = srcs + shim + [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(HERE, "refshim"))
                          for f in fs] + [os.path.abspath(__file__)]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    gen = generate()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu99", "-ffp-contract=off", "-w",
           "-I" + os.path.join(HERE, "refshim"), "-I" + GEN, "-I" + REF,
           "-I" + os.path.join(REF, "aran"), "-o", LIB + ".tmp"] + srcs + gen + shim + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference operator build failed:\n" + r.stderr[-4000:])
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
