"""Build recipe for ``oracle/_ref``: the reference's own Siconos numerics C
sources, compiled where they lie under the reference checkout, plus this
project's BLAS shim and a small runner, into one shared library.

Test infrastructure only: the library is the checker for the CPU restatement
in ``oracle/fc3d_oracle.c`` and the source of the committed golden fixtures.
Nothing in the product links or loads it.

Recipe (nothing is copied out of the reference tree):

1. compile every ``numerics/src/**/*.c`` except tests, optional linear-algebra
   back-ends, the OpenMP/PETSc/CUDA ``FrictionContact/parallel`` solvers and
   ``Unstable_or_deprecated`` with ``gcc -std=gnu11 -O3 -DCS_LONG -DNCOMPLEX``,
   against the reference's own headers plus the self-written stand-ins in
   ``oracle/include`` (cs.h, cblas.h, openblas_config.h, lapacke.h);
2. compile ``oracle/ref_shim.c`` (naive CBLAS loops) and
   ``oracle/ref_runner.c`` (array-in/array-out wrappers around the
   reference's ``fc3d_driver``);
3. link once, collect the symbols no object defines (CXSparse, LAPACKE,
   MUMPS ... none reached on the SBM NSGS path), generate an aborting stub for
   each, and link ``oracle/_ref/libsiconos_numerics_ref.so``.

4. compile the device code of the reference's 2D GPU solvers
   (``FrictionContact/parallel/gpu/fc2d_nsgs_graph_permut_cuda.cu`` and
   ``..._blocklegacy.cu``, their local-solve kernels) with ``nvcc -fatbin``
   for sm_103a into ``oracle/_ref/<file>.fatbin``, with the reference's
   Release flags (``-O3 -DNDEBUG -DSICONOS_CUDA``, default contraction): an
   image the measurement-only per-colour comparator loads to run the
   reference's own kernel (its host code needs PETSc's colouring and does not
   build here).

``-ffp-contract=off`` keeps x86-64 and aarch64 builds bit-identical (gcc
contracts a*b+c into FMA by default on aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libsiconos_numerics_ref.so"
# the reference checkout the library was built from (one line), for the
# tests that compile against its headers
SOURCE = OUT / "SOURCE"
ENV = "SICONOS_REFERENCE"


def source_dir() -> Path | None:
    """The reference checkout: ``$SICONOS_REFERENCE``, else the one
    ``oracle/_ref`` was built from; None when neither names a checkout."""
    for cand in (os.environ.get(ENV), SOURCE.read_text().strip() if SOURCE.exists() else None):
        if cand and (Path(cand) / "numerics" / "src").is_dir():
            return Path(cand)
    return None


def include_flags(ref: Path) -> list[str]:
    """The include path the reference's sources compile with here."""
    return _includes(Path(ref))

FC2D_CUDA_SOURCES = (Path("numerics/src/FrictionContact/parallel/gpu/fc2d_nsgs_graph_permut_cuda.cu"),
                     Path("numerics/src/FrictionContact/parallel/gpu/fc2d_nsgs_graph_permut_cuda_blocklegacy.cu"))
FC2D_CUDA_IMAGE = OUT / "fc2d_nsgs_graph_permut_cuda.fatbin"
FC2D_CUDA_IMAGE_BLOCKLEGACY = OUT / "fc2d_nsgs_graph_permut_cuda_blocklegacy.fatbin"

EXCLUDE_PARTS = ("/test/", "/test-utils/", "/linalg/optional/", "/FrictionContact/parallel/",
                 "/Unstable_or_deprecated/", "/tools/parallel/")
CFLAGS = ["-std=gnu11", "-O3", "-fPIC", "-DCS_LONG", "-DNCOMPLEX", "-ffp-contract=off", "-w"]


def _sources(ref: Path) -> list[Path]:
    src = ref / "numerics" / "src"
    out = []
    for p in sorted(src.rglob("*.c")):
        s = str(p)
        if any(x in s for x in EXCLUDE_PARTS):
            continue
        out.append(p)
    return out


def _includes(ref: Path) -> list[str]:
    src = ref / "numerics" / "src"
    dirs = [HERE / "include", src] + sorted(d for d in src.rglob("*") if d.is_dir())
    dirs += [ref / "externals" / "blas_lapack", ref / "externals" / "tools", ref / "externals" / "sort"]
    return [f"-I{d}" for d in dirs]


def _compile(args):
    src, obj, inc = args
    if obj.exists() and obj.stat().st_mtime > src.stat().st_mtime:
        return src, True, ""
    r = subprocess.run(["gcc", *CFLAGS, *inc, "-c", str(src), "-o", str(obj)],
                       capture_output=True, text=True)
    return src, r.returncode == 0, r.stderr[-400:]


def build(ref: str | os.PathLike, verbose: bool = False) -> Path:
    ref = Path(ref)
    if not (ref / "numerics" / "src").is_dir():
        raise FileNotFoundError(f"reference numerics sources not found under {ref}")
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = _includes(ref)
    jobs = []
    for s in _sources(ref):
        rel = s.relative_to(ref / "numerics" / "src")
        obj = objdir / (str(rel).replace("/", "__")[:-2] + ".o")
        jobs.append((s, obj, inc))
    for extra in ("ref_shim.c", "ref_runner.c"):
        jobs.append((HERE / extra, objdir / ("oracle__" + extra[:-2] + ".o"), inc))
    failed = []
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for src, ok, err in ex.map(_compile, jobs):
            if not ok:
                failed.append(src)
                if verbose:
                    print(f"[oracle/_ref] skip {src}: {err}", file=sys.stderr)
    for extra in ("ref_shim.c", "ref_runner.c"):
        if HERE / extra in failed:
            raise RuntimeError(f"failed to compile {extra}")
    objs = sorted(str(o) for s, o, _i in jobs if s not in failed and o.exists())
    # first link: find what nothing defines
    r = subprocess.run(["gcc", "-shared", "-o", str(LIB), *objs, "-Wl,--no-undefined", "-lm"],
                       capture_output=True, text=True)
    missing = sorted(set(re.findall(r"undefined reference to `([^']+)'", r.stderr)))
    stub_c = objdir / "stubs.c"
    with open(stub_c, "w") as f:
        f.write("/* generated by oracle/build_ref.py: symbols off the SBM NSGS path */\n")
        f.write("#include <stdio.h>\n#include <stdlib.h>\n")
        for m in missing:
            f.write(f'void {m}(void) {{ fprintf(stderr, "oracle stub reached: {m}\\n"); abort(); }}\n')
    stub_o = objdir / "oracle__stubs.o"
    subprocess.run(["gcc", "-O0", "-fPIC", "-w", "-c", str(stub_c), "-o", str(stub_o)], check=True)
    r = subprocess.run(["gcc", "-shared", "-o", str(LIB), *objs, str(stub_o), "-Wl,--no-undefined", "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle/_ref link failed:\n" + r.stderr[-3000:])
    SOURCE.write_text(str(ref.resolve()) + "\n")
    if verbose:
        print(f"[oracle/_ref] {len(objs)} objects, {len(failed)} skipped, {len(missing)} stubs -> {LIB}")
    build_cuda(ref, verbose)
    return LIB


def build_cuda(ref: str | os.PathLike, verbose: bool = False) -> list[Path]:
    """Step 4: the reference's two fc2d CUDA files as sm_103a fatbins (device
    code only; nvcc parses the host code against the reference's headers).
    Returns the images present; an image whose compile fails (or with no nvcc)
    is left out, keeping any earlier one."""
    ref = Path(ref)
    out = []
    for rel, img in zip(FC2D_CUDA_SOURCES, (FC2D_CUDA_IMAGE, FC2D_CUDA_IMAGE_BLOCKLEGACY)):
        src = ref / rel
        if not src.is_file():
            continue
        if img.exists() and img.stat().st_mtime > src.stat().st_mtime:
            out.append(img)
            continue
        OUT.mkdir(parents=True, exist_ok=True)
        tmp = img.with_suffix(".tmp")
        cmd = ["nvcc", "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-DNDEBUG", "-DSICONOS_CUDA",
               "-DCS_LONG", "-DNCOMPLEX", "-w", *_includes(ref), str(src), "-o", str(tmp)]
        try:
            r = subprocess.run(cmd, capture_output=True, text=True)
        except FileNotFoundError:
            return out
        if r.returncode != 0:
            if verbose:
                print(f"[oracle/_ref] {img.name} not built: {r.stderr[-400:]}", file=sys.stderr)
            continue
        os.replace(tmp, img)
        if verbose:
            print(f"[oracle/_ref] -> {img}")
        out.append(img)
    return out
