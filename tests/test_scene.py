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
