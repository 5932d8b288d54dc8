"""Build the oracle's own C restatement (``fc3d_oracle.c``, ``colour_oracle.c``,
``fc2d_oracle.c``, ``rfc3d_oracle.c``) into ``oracle/_build/liboracle.so``.
Test infrastructure only.

The library also carries the seeded sphere-lattice generator
(``siconos_gb300/csrc/fc3d_lattice.c``, the workload definition shared with
the solver's tests), so a CPU-only baseline can make its scenes without
loading the solver library.

``-O3 -ffp-contract=off``: optimised as a baseline should be, with the
arithmetic identical on x86-64 and aarch64 and identical to the reference
build in ``oracle/_ref`` (no contraction into FMA, no reassociation).  No
``-march=native``: the same source must give the same results on both
machines."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SOURCES = ["fc3d_oracle.c", "colour_oracle.c", "fc2d_oracle.c", "rfc3d_oracle.c", "gfc3d_oracle.c"]
ROOT = HERE.parent
GENERATOR = ROOT / "siconos_gb300" / "csrc" / "fc3d_lattice.c"


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = [HERE / s for s in SOURCES if (HERE / s).exists()] + [GENERATOR]
    deps = srcs + [HERE / "build.py", ROOT / "include" / "fc3dgpu_scene.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime > s.stat().st_mtime for s in deps):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", f"-I{ROOT / 'include'}",
           *[str(s) for s in srcs], "-o", str(LIB), "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
