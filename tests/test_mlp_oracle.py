"""The learned warm start's CPU oracle (numpy): BF16 rounding, its exact
gradient against finite differences, and the host feature layout."""
import numpy as np
import pytest

from oracle import mlp_oracle as M


def test_bf16_rounding_nearest_even():
    x = np.array([1.0, 1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, -2.5, 3.0e-3], np.float32)
    y = M.bf16(x)
    assert y[0] == 1.0
    assert y[1] == 1.0                      # halfway: ties to the even mantissa
    assert y[2] == np.float32(1 + 2.0 ** -6)  # halfway: rounds up to even
    assert y[3] == -2.5
    assert abs(y[4] - 3.0e-3) <= 3.0e-3 * 2.0 ** -8
    assert (M.bf16(y) == y).all()          # idempotent


def _problem(seed=0, n=96):
    from siconos_gb300.learned import init_params, make_stats
    g = np.random.default_rng(seed)
    X = g.standard_normal((n, M.NF)).astype(np.float32)
    T = np.stack([np.tanh(X[:, 0] + X[:, 3]), X[:, 5] * X[:, 6], np.abs(X[:, 9])], 1).astype(np.float32)
    p = init_params(seed)
    p[M.OFFS[0][1]:M.OFFS[0][1] + 128] = 0.05  # non-zero biases reach more ReLUs
    return p, make_stats(X, T), X, T


def test_exact_gradient_matches_finite_differences():
    p, st, X, T = _problem()
    p64 = p.astype(np.float64)
    st64 = st.astype(np.float64)
    _, g = M.loss_and_grad(p64, st64, X, T, exact=True)
    rng = np.random.default_rng(1)
    # parameters that matter: weights on real inputs/outputs and biases
    cand = [i for i in range(M.NPARAM) if abs(g[i]) > 1e-6]
    pick = rng.choice(cand, 40, replace=False)
    h = 1e-6
    for i in pick:
        a = p64.copy()
        b = p64.copy()
        a[i] += h
        b[i] -= h
        fd = (M.loss_only(a, st64, X, T) - M.loss_only(b, st64, X, T)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1e-3, abs(g[i])), (i, fd, g[i])


def test_rounded_gradient_close_to_exact():
    p, st, X, T = _problem(2)
    _, g64 = M.loss_and_grad(p.astype(np.float64), st.astype(np.float64), X, T, exact=True)
    _, g16 = M.loss_and_grad(p, st, X, T)
    assert np.linalg.norm(g16 - g64) <= 0.05 * np.linalg.norm(g64)


def test_host_features_layout():
    from conftest import load_case
    from siconos_gb300.learned import host_features
    P, _ = load_case("lattice_3x3x2_s1")
    r = np.arange(3 * P.nc, dtype=np.float64)
    gap = np.linspace(0, 1, P.nc)
    X = host_features(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu, r, gap)
    assert X.shape == (P.nc, 17)
    blocks = np.asarray(P.blocks).reshape(-1, 9)
    for i in (0, P.nc // 2, P.nc - 1):
        row = range(P.rowptr[i], P.rowptr[i + 1])
        d = [b for b in row if P.colidx[b] == i][0]
        assert (X[i, :9] == blocks[d].astype(np.float32)).all()
        assert (X[i, 9:12] == P.q[3 * i:3 * i + 3].astype(np.float32)).all()
        assert X[i, 12] == np.float32(P.mu[i])
        assert (X[i, 13:16] == r[3 * i:3 * i + 3].astype(np.float32)).all()
        assert X[i, 16] == np.float32(gap[i])
