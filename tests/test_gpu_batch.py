"""Batched persistent solve (many independent scenes, one launch per
precision): each scene gets its solo colouring, so its FP64 iterates equal a
solo solve's bit for bit, and whole solves reach the reference tolerance
where the colour-ordered oracle does."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _scenes(n=12, seed=3):
    from siconos_gb300 import scene
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        d = [int(rng.integers(2, 7)), int(rng.integers(2, 7)), int(rng.integers(1, 4))]
        out.append(scene.lattice(*d, seed=100 + k, mu=float(rng.uniform(0.1, 0.9))))
    return out


def test_batch_fp64_equals_solo_bitwise(gpu):
    from siconos_gb300.device import DeviceSolver
    sc = _scenes()
    gpu.load_batch(sc)
    st = gpu.solve_batch(tol=1e-300, max_iter=15, precision=1)
    assert np.all(st["sweeps64"] == 15)
    rb, ub = gpu.get_batch()
    solo = DeviceSolver(0)
    for k, s in enumerate(sc):
        solo.load(s)
        solo.solve(tol=1e-300, max_iter=15, precision=1, lanes=1)
        r, u = solo.get()
        assert np.array_equal(rb[k], r), k
        # and the colour-ordered oracle
        col = solo.colours()
        order = np.lexsort((np.arange(s.nc), col)).astype(np.int32)
        P = O.Problem(s.nc, s.rowptr, s.colidx, s.blocks, s.q, s.mu)
        ref = O.nsgs_port(P, tol=1e-300, maxiter=15, order=order)
        assert np.array_equal(r, ref.r), k
    solo.close()


def test_batch_mixed_reaches_tolerance(gpu):
    sc = _scenes(16, seed=5)
    gpu.load_batch(sc)
    st = gpu.solve_batch(tol=1e-8, max_iter=5000)
    rb, ub = gpu.get_batch()
    for k, s in enumerate(sc):
        P = O.Problem(s.nc, s.rowptr, s.colidx, s.blocks, s.q, s.mu)
        e, u = O.compute_error_port(P, rb[k])
        assert abs(e - st["error"][k]) <= 1e-9 * max(e, 1e-300) + 1e-18
        assert np.allclose(ub[k], u, rtol=0, atol=1e-12 * (1 + np.abs(u).max()))
        col = np.zeros(s.nc, np.int32)
        O.port().oracle_colour_greedy(s.nc, s.rowptr, s.colidx, 0, col)
        ref = O.nsgs_port(P, tol=1e-8, maxiter=5000, order=np.lexsort((np.arange(s.nc), col)).astype(np.int32))
        if ref.info == 0:
            assert st["info"][k] == 0 and e <= 1e-8, (k, st["info"][k], e)
        else:
            assert st["info"][k] in (0, -20)


def test_batch_graph_replay(gpu):
    sc = _scenes(6, seed=9)
    gpu.load_batch(sc)
    a = gpu.solve_batch(tol=1e-8, max_iter=200)
    ra, _ = gpu.get_batch()
    gpu.set_r(np.zeros(3 * gpu.nc))
    b = gpu.solve_batch(tol=1e-8, max_iter=200)  # replays the recorded graph
    rb, _ = gpu.get_batch()
    assert np.array_equal(a["sweeps32"], b["sweeps32"]) and np.array_equal(a["info"], b["info"])
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y)
