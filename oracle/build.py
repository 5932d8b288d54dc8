"""Build the oracle's own C restatement (``fc3d_oracle.c``, ``colour_oracle.c``)
into ``oracle/_build/liboracle.so``.  Test infrastructure only.

``-ffp-contract=off`` keeps the arithmetic identical on x86-64 and aarch64 and
identical to the reference build in ``oracle/_ref``."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SOURCES = ["fc3d_oracle.c", "colour_oracle.c", "fc2d_oracle.c", "rfc3d_oracle.c"]


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = [HERE / s for s in SOURCES if (HERE / s).exists()]
    if not force and LIB.exists() and all(LIB.stat().st_mtime > s.stat().st_mtime for s in srcs):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
           *[str(s) for s in srcs], "-o", str(LIB), "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
