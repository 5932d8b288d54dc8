"""Lattice generator: sizes from the definition and platform-independent
bit-exact output (checksums recorded by tests/golden/make_golden.py)."""
import hashlib

import numpy as np
import pytest

from conftest import GOLDEN


def _sum(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_counts_from_definition(built_lib):
    from siconos_gb300 import scene
    for (nx, ny, nz) in [(5, 5, 6), (3, 3, 2), (4, 7, 2)]:
        s = scene.lattice(nx, ny, nz, seed=5)
        nc = (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1) + nx * ny
        assert s.nc == nc
        deg = np.zeros(nx * ny * nz, int)
        for i in range(nx):
            for j in range(ny):
                for k in range(nz):
                    d = (i > 0) + (i < nx - 1) + (j > 0) + (j < ny - 1) + (k > 0) + (k < nz - 1) + (k == 0)
                    deg[i + nx * (j + ny * k)] = d
        assert s.nnzb == nc + int((deg * (deg - 1)).sum())
        W = s.problem().M().todense()
        assert np.allclose(W, W.T, atol=1e-12)
        assert np.all(np.linalg.eigvalsh(W) > -1e-10)


@pytest.mark.parametrize("line", (GOLDEN / "lattice_checksums.txt").read_text().split("\n")[:-1])
def test_generator_bit_exact(built_lib, line):
    from siconos_gb300 import scene
    key, nc, nnzb, h = line.split()
    dims, seed = key.split("_s")
    nx, ny, nz = (int(v) for v in dims.split("x"))
    s = scene.lattice(nx, ny, nz, seed=int(seed))
    assert s.nc == int(nc) and s.nnzb == int(nnzb)
    assert _sum(s.rowptr, s.colidx, s.blocks, s.q) == h


def test_golden_lattice_matches_generator(built_lib):
    from siconos_gb300 import scene
    z = np.load(GOLDEN / "lattice_5x5x6_s1.npz")
    s = scene.lattice(5, 5, 6, seed=1)
    assert np.array_equal(s.blocks, z["blocks"]) and np.array_equal(s.q, z["q"])


@pytest.mark.parametrize("dims, seed, mu", [((5, 5, 6), 1, 0.5), ((7, 3, 4), 11, 0.3), ((3, 3, 2), 2, 0.9)])
def test_oracle_generator_equals_package_generator(built_lib, dims, seed, mu):
    """The generator compiled into the oracle library (what the benchmark's
    reference arm uses, so that it loads no solver library) gives the arrays
    of siconos_gb300.scene.lattice bit for bit."""
    import oracle as O
    from siconos_gb300 import scene as sc
    P = O.lattice(*dims, seed=seed, mu=mu)
    s = sc.lattice(*dims, seed=seed, mu=mu)
    assert P.nc == s.nc
    for a, b in ((P.rowptr, s.rowptr), (P.colidx, s.colidx), (P.blocks, s.blocks), (P.q, s.q), (P.mu, s.mu)):
        assert np.array_equal(a, b)


def test_batch_specs_match_batch_scenes(built_lib):
    from siconos_gb300 import scene as sc
    specs = sc.batch_specs(count=6, seed=3)
    scenes = sc.batch_scenes(count=6, seed=3)
    for (d, seed, mu), s in zip(specs, scenes):
        t = sc.lattice(*d, seed=seed, mu=mu)
        assert t.nc == s.nc and np.array_equal(t.q, s.q) and float(s.mu[0]) == mu
