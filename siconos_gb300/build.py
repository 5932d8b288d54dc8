"""Build ``libfc3dgpu.so`` in-tree: the host C files with gcc and the CUDA
files with nvcc for sm_103a only, linked with the static CUDA runtime.

The FP64 sweep unit is compiled with ``--fmad=false`` so its arithmetic is
that of the CPU restatement; host C uses ``-ffp-contract=off`` for the same
reason on aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libfc3dgpu.so"
# measurement-only comparator (the reference's per-colour 2D GPU design with
# cuSPARSE): its own library, so the solver library links no cuSPARSE
COMPARATOR = OUT / "libfc2dpercolour.so"
COMPARATOR_SOURCE = "fc2dgpu_percolour.cu"
COMPARATOR_FLAGS = ["--fmad=false", "-Xcompiler", "-ffp-contract=off"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

C_SOURCES = ["fc3d_lattice.c", "fc3dgpu_nsgs.c", "fc3d_dat.c", "fc2dgpu_nsgs.c", "rfc3dgpu_nsgs.c", "fc3d_colour.c",
             "gfc3dgpu_nsgs.c"]
CU_SOURCES = {
    "fc3dgpu_ctx.cu": ["--fmad=false"],
    "fc3dgpu_sweep_f64.cu": ["--fmad=false"],
    # the same FP64 kernels with the fast one-contact arithmetic (opt-in)
    "fc3dgpu_sweep_f64fast.cu": ["--fmad=false"],
    "fc3dgpu_noalloc.cu": ["--fmad=false"],
    # host code computes determinants and norms the kernel reuses
    "fc2dgpu.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    # host code computes the rolling solver's rho (Jacobi eigenvalues)
    "rfc3dgpu.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    # the global problem: the reference's iterates bit for bit; host code
    # computes |q|
    "gfc3dgpu.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    # BF16 tensor-core MLP of the learned warm start
    "fc3dgpu_mlp.cu": [],
    # the FP32 sweeps are the accelerator whose result the FP64 polish
    # finishes: approximate division and square root, denormals flushed
    "fc3dgpu_sweep_f32.cu": ["--use_fast_math"],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def _deps_newer(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    nvcc = _nvcc()
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    jobs = []
    objs = []
    for s in C_SOURCES:
        src, obj = CSRC / s, OUT / (s + ".o")
        objs.append(obj)
        if force or _deps_newer(obj, src):
            jobs.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", *inc, "-c", str(src),
                         "-o", str(obj)])
    cmp_src, cmp_obj = CSRC / COMPARATOR_SOURCE, OUT / (COMPARATOR_SOURCE + ".o")
    if force or _deps_newer(cmp_obj, cmp_src):
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *COMPARATOR_FLAGS, *inc,
                     "-c", str(cmp_src), "-o", str(cmp_obj)])
    for s, extra in CU_SOURCES.items():
        src, obj = CSRC / s, OUT / (s + ".o")
        objs.append(obj)
        if force or _deps_newer(obj, src):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                         *extra, *inc, "-c", str(src), "-o", str(obj)])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 2))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if jobs or force or not LIB.exists():
        tmp = OUT / (LIB.name + ".tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for o in objs]])
        os.replace(tmp, LIB)
    if jobs or force or not COMPARATOR.exists():
        tmp = OUT / (COMPARATOR.name + ".tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), str(cmp_obj), f"-L{OUT}", "-lfc3dgpu", "-lcusparse",
              "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"])
        os.replace(tmp, COMPARATOR)
    if verbose:
        for l in logs:
            print(l)
    return LIB


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
