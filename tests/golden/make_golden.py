"""Generate the golden fixtures in tests/golden from the reference itself.

Run in a checkout that has the reference sources (the library in
``oracle/_ref`` is built from them by ``oracle/build_ref.py``):

    python tests/golden/make_golden.py /path/to/reference [--only=fixtures|fc2d|rfc3d|gfc3d|to_tolerance]

For each SBM/dense friction-contact fixture of the reference's own test data
(numerics/src/FrictionContact/test/data) and for the 5x5x6 lattice scene,
this stores the problem (block-CSR) and the reference fc3d_driver result
(SICONOS_FRICTION_3D_NSGS defaults, tol 1e-8, 10000 iterations; and a
20-iteration run) in one compressed .npz per case.  It also evaluates the
reference's computeAlartCurnierSTD on the 1000 samples of data/ACinputs.dat
(the known-answer set of fc3d_AlartCurnierFunctions_test.c), and records
checksums of generated lattice scenes so that other platforms can check the
generator reproduces them bit for bit.
"""
from __future__ import annotations

import hashlib
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

FIXTURES = [
    "FC3D_Example1_SBM.dat",
    "FrictionContact3D_1c.dat",
    "Confeti-ex13-4contact-Fc3D-SBM.dat",
    "Confeti-ex13-Fc3D-SBM.dat",
    "Confeti-ex03-Fc3D-SBM.dat",
    "KaplasTower-i1061-4.hdf5.dat",
    "Capsules-i122-1617.dat",
    "BoxesStack1-i100000-32.hdf5.dat",
    "RockPile_tob1.dat",
    "FC3D_Example1.dat",
    "Rover4396.dat",
    "NESpheres_10_1.dat",
    # the rest of the reference's fc3d test collection (data_collection_1.c)
    # and OneObject from data_collection_3.c
    "FrictionContact3D_RR_1c.dat",
    "Capsules-i100-1090.dat",
    "Capsules-i100-889.dat",
    "Capsules-i101-404.dat",
    "Capsules-i103-990.dat",
    "Rover1039.dat",
    "Rover1040.dat",
    "Rover1041.dat",
    "Rover11035.dat",
    "Rover11211.dat",
    "Rover3865.dat",
    "Rover4144.dat",
    "Rover4493.dat",
    "Rover4516.dat",
    "Rover4609.dat",
    "Rover4613.dat",
    "Rover4622.dat",
    "Rover9770.dat",
    "NESpheres_30_1.dat",
    "OneObject-i100000-499.hdf5.dat",
]


def checksum(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def save_case(name, P, res_full, res_20, extra=None):
    d = dict(nc=P.nc, rowptr=P.rowptr, colidx=P.colidx, blocks=P.blocks, q=P.q, mu=P.mu,
             info=res_full.info, iterations=res_full.iterations, error=res_full.error, r=res_full.r, u=res_full.u,
             trace=res_full.trace, info20=res_20.info, iterations20=res_20.iterations, error20=res_20.error,
             r20=res_20.r, u20=res_20.u, trace20=res_20.trace)
    if extra:
        d.update(extra)
    np.savez_compressed(HERE / f"{name}.npz", **d)


FC2D_FIXTURES = [
    # the reference's fc2d test collection (data_collection_fc2d_1.c)
    "FrictionContactProblem00374.dat",
    "FrictionContactProblem00394.dat",
    "FC2D_SliderCrankLagrangian00000.dat",
    "FC2D_SliderCrankLagrangian00001.dat",
    "FrictionContactProblem00727.dat",
    "FrictionContactProblem00031.dat",
    "FrictionContactProblem00071.dat",
    "FrictionContactProblem00237.dat",
    # CSparse storage: the reference built here cannot read it (its CSparse
    # sources are not compiled), so these hold the restatement's results
    "fc2d_granularflowonwall_00667_00000.dat",
    "fc2d_granularflowonwall_02020_00213.dat",
    "fc2d_granularflowonwall_07002_00801.dat",
]


def make_fc2d(data: Path):
    """2D problems with the reference's fc2d_nsgs results (tol 1e-5, 10000
    iterations, the reference's own fc2d test settings) and a 20-iteration
    run; problems the reference cannot read here get the restatement's."""
    import oracle as O
    import siconos_gb300.numerics as sn
    for f in FC2D_FIXTURES:
        storage = (data / f).read_text()[:64].split()[2]
        if storage != "2":
            P = O.read_dat(data / f)
            run, kind = O.fc2d_nsgs_ref, "reference"
        else:
            p = sn.read_dat(data / f)
            M = p._M
            P = O.Problem(M.nc, M.rowptr, M.colidx, M.blocks, p._q, p._mu, 2)
            run, kind = O.fc2d_nsgs_port, "oracle"
        assert P.dim == 2
        full = run(P, tol=1e-5, maxiter=10000)
        short = run(P, tol=1e-5, maxiter=20)
        name = "fc2d_" + f.replace(".dat", "").replace("-", "_")
        d = dict(nc=P.nc, rowptr=P.rowptr, colidx=P.colidx, blocks=P.blocks, q=P.q, mu=P.mu, dim=2,
                 info=full.info, iterations=full.iterations, error=full.error, r=full.r, u=full.u,
                 info20=short.info, iterations20=short.iterations, error20=short.error, r20=short.r, u20=short.u,
                 source=f, results=kind)
        np.savez_compressed(HERE / f"{name}.npz", **d)
        print(f"{f}: nc={P.nc} nnzb={P.nnzb} {kind} info={full.info} it={full.iterations} err={full.error:.3e}")


RFC3D_FIXTURES = [
    # the reference's rolling-friction test data (RollingFrictionContact/test/
    # data); the reference's rolling NSGS takes dense storage only, the
    # CSparse-stored files are left out
    "RFC3D_sphere_1.dat",
    "RFC3D_sphere_2.dat",
    "RFC3D_cube_1.dat",
    "rfc3d_sphere_from_grfc3d_dense.dat",
    "rockfall_14_25792.dat",
    "rockfall_21_54029.dat",
]


def make_rfc3d(data: Path):
    """Rolling-friction problems with the reference's rolling_friction_3d_nsgs
    results (its defaults, tol 1e-8, 10000 iterations; and a 20-iteration
    run), W as read by the reference (dense, every 5x5 block holding a
    nonzero kept, in column order)."""
    import oracle as O
    for f in RFC3D_FIXTURES:
        P = O.read_rfc3d_dat(data / f)
        full = O.rfc3d_nsgs_ref(P, tol=1e-8, maxiter=10000, trace_cap=10000)
        short = O.rfc3d_nsgs_ref(P, tol=1e-8, maxiter=20, trace_cap=20)
        name = "rfc3d_" + f.replace(".dat", "").replace("-", "_")
        d = dict(nc=P.nc, rowptr=P.rowptr, colidx=P.colidx, blocks=P.blocks, q=P.q, mu=P.mu, mur=P.mur,
                 info=full.info, iterations=full.iterations, error=full.error, r=full.r, u=full.u, trace=full.trace,
                 info20=short.info, iterations20=short.iterations, error20=short.error, r20=short.r, u20=short.u,
                 trace20=short.trace, source=f)
        np.savez_compressed(HERE / f"{name}.npz", **d)
        print(f"{f}: nc={P.nc} nnzb={P.nnzb} info={full.info} it={full.iterations} err={full.error:.3e}")


GFC3D_FIXTURES = [
    # the reference's global-problem test data (data_collection_gfc3d); the
    # reference built here reads M and H in dense and sparse-block storage
    # (GFC3D_TwoRods1-condensed.dat stores H in CSparse form, which it
    # cannot read)
    "GFC3D_Example0.dat",
    "GFC3D_Example00.dat",
    "GFC3D_Example00_badly_scaled.dat",
    "GFC3D_Example0_SBM.dat",
    "GFC3D_Example1.dat",
    "GFC3D_OneContact.dat",
    "GFC3D_TwoRods1.dat",
]


def make_gfc3d(data: Path):
    """Global problems with the reference's gfc3d_nsgs results through its
    gfc3d_driver on dense copies of M and H (the settings of its gfc3d test
    collection: tol 1e-8 with 1000 iterations, and the default tol 1e-4 with
    10000), a 20-iteration run, and the 5x5x6 sphere lattice in global form
    (bodies of mass 10, inertia 1)."""
    import oracle as O
    cases = [(f.replace(".dat", "").replace("-", "_"), O.read_gfc3d_dat(data / f)[0], f) for f in GFC3D_FIXTURES]
    cases.append(("lattice_5x5x6_s1", O.lattice_global(5, 5, 6, seed=1), "lattice 5x5x6 seed 1, mass scale 10"))
    for name, P, src in cases:
        d = dict(n=P.n, nc=P.nc, Mp=P.Mp, Mi=P.Mi, Mx=P.Mx, Hp=P.Hp, Hi=P.Hi, Hx=P.Hx, q=P.q, b=P.b, mu=P.mu,
                 source=src)
        for tag, tol, it in (("", 1e-8, 1000), ("_default", 1e-4, 10000), ("20", 0.0, 20)):
            res = O.gfc3d_nsgs_ref(P, tol=tol, maxiter=it)
            d.update({f"info{tag}": res.info, f"error{tag}": res.error, f"r{tag}": res.r, f"u{tag}": res.u,
                      f"v{tag}": res.v})
        np.savez_compressed(HERE / f"gfc3d_{name}.npz", **d)
        print(f"{src}: n={P.n} nc={P.nc} info={d['info']} err={d['error']:.3e} "
              f"default: info={d['info_default']} err={d['error_default']:.3e}")


def make_to_tolerance():
    """The reference's own fc3d_nsgs (oracle/_ref) on the 60x60x30 lattice
    (seed 1, mu 0.5) from r = 0 to 1e-3 and to 1e-4 (defaults, budget
    10000): info, sweeps, final error and the whole error trace.  Too slow
    for a test to recompute (about a minute per tolerance on one core); the
    benchmark reads the sweep counts as the reference's side of the time to
    tolerance."""
    import json

    import oracle as O
    P = O.lattice(60, 60, 30, seed=1, mu=0.5)
    out = {"scene": "lattice 60x60x30, seed 1, mu 0.5", "nc": P.nc, "nnzb": P.nnzb, "source": "oracle/_ref"}
    for tol in (1e-3, 1e-4):
        res = O.nsgs_ref(P, tol=tol, maxiter=10000, trace_cap=10000)
        out[f"{tol:g}"] = {"info": res.info, "iterations": res.iterations, "error": res.error,
                           "trace": [float(x) for x in res.trace[:res.iterations]]}
        print(f"to {tol:g}: info={res.info} it={res.iterations} err={res.error:.3e}")
    (HERE / "lattice_60x60x30_s1_to_tolerance.json").write_text(json.dumps(out) + "\n")


def main(ref_root: str, only: str | None = None):
    from oracle import build_ref
    import oracle as O

    build_ref.build(ref_root)
    data = Path(ref_root) / "numerics" / "src" / "FrictionContact" / "test" / "data"
    if only == "rfc3d":
        make_rfc3d(Path(ref_root) / "numerics" / "src" / "RollingFrictionContact" / "test" / "data")
        return
    if only == "gfc3d":
        make_gfc3d(data)
        return
    if only == "to_tolerance":
        make_to_tolerance()
        return
    if only == "fc2d":
        from siconos_gb300 import build as B
        B.build()
        make_fc2d(data)
        return
    for f in FIXTURES:
        name = "fixture_" + f.replace(".hdf5", "").replace(".dat", "").replace("-", "_")
        if only == "fixtures" and (HERE / f"{name}.npz").exists():
            continue  # --only=fixtures: the fixtures not yet generated
        P = O.read_dat(data / f)
        full = O.nsgs_ref(P, tol=1e-8, maxiter=10000, trace_cap=20000)
        short = O.nsgs_ref(P, tol=1e-8, maxiter=20, trace_cap=20)
        save_case(name, P, full, short, {"source": f})
        print(f"{f}: nc={P.nc} nnzb={P.nnzb} info={full.info} it={full.iterations} err={full.error:.3e}")
    if only == "fixtures":
        return

    # lattice scenes (generator in the product library)
    from siconos_gb300 import build as B
    B.build()
    from siconos_gb300 import scene
    sums = {}
    for dims, seed in [((5, 5, 6), 1), ((5, 5, 6), 2), ((3, 3, 2), 1)]:
        s = scene.lattice(*dims, seed=seed)
        P = O.Problem(s.nc, s.rowptr, s.colidx, s.blocks, s.q, s.mu)
        full = O.nsgs_ref(P, tol=1e-8, maxiter=10000, trace_cap=20000)
        short = O.nsgs_ref(P, tol=1e-8, maxiter=20, trace_cap=20)
        name = f"lattice_{dims[0]}x{dims[1]}x{dims[2]}_s{seed}"
        save_case(name, P, full, short, {"dims": np.array(dims), "seed": seed})
        print(f"{name}: nc={P.nc} info={full.info} it={full.iterations} err={full.error:.3e}")
    for dims, seed in [((5, 5, 6), 1), ((12, 9, 7), 3), ((60, 60, 30), 1)]:
        s = scene.lattice(*dims, seed=seed)
        sums[f"{dims[0]}x{dims[1]}x{dims[2]}_s{seed}"] = [s.nc, s.nnzb, checksum(s.rowptr, s.colidx, s.blocks, s.q)]
    with open(HERE / "lattice_checksums.txt", "w") as fh:
        for k, (nc, nnzb, h) in sums.items():
            fh.write(f"{k} {nc} {nnzb} {h}\n")

    # Alart-Curnier known answers
    vals = np.array([float(x) for x in (data / "ACinputs.dat").read_text().split()])
    n = int(vals[0])
    R = vals[1:1 + 3 * n].reshape(n, 3)
    V = vals[1 + 3 * n:1 + 6 * n].reshape(n, 3)
    MU = vals[1 + 6 * n:1 + 7 * n]
    RHO = vals[1 + 7 * n:1 + 10 * n].reshape(n, 3)
    lib = O.ref()
    F = np.zeros((n, 3))
    A = np.zeros((n, 9))
    Bm = np.zeros((n, 9))
    for k in range(n):
        f, a, b = np.zeros(3), np.zeros(9), np.zeros(9)
        lib.computeAlartCurnierSTD(np.ascontiguousarray(R[k]), np.ascontiguousarray(V[k]), MU[k],
                                   np.ascontiguousarray(RHO[k]), f, a.ctypes.data, b.ctypes.data)
        F[k], A[k], Bm[k] = f, a, b
    np.savez_compressed(HERE / "ac_known_answers.npz", R=R, V=V, mu=MU, rho=RHO, F=F, A=A, B=Bm)
    print("ACinputs:", n, "samples")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = next((a[7:] for a in sys.argv[1:] if a.startswith("--only=")), None)
    src = args[0] if args else os.environ.get("SICONOS_REFERENCE")
    if not src:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout> [--only=NAME]"
                 "  (or set SICONOS_REFERENCE)")
    main(src, only)
