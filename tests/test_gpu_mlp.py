"""The learned warm start on the GPU: the BF16 tensor-core training kernels'
gradients and the inference kernel against the CPU oracle, training that
lowers the loss, device features against host features, and the warm start's
fallback rule."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mlp(built_lib):
    from siconos_gb300.learned import WarmStartMLP
    try:
        m = WarmStartMLP(0)
    except RuntimeError as e:
        pytest.fail(f"no usable CUDA device for a -m gpu run: {e}")
    yield m
    m.close()


def _problem(seed, n):
    from siconos_gb300.learned import init_params, make_stats
    g = np.random.default_rng(seed)
    X = g.standard_normal((n, M.NF)).astype(np.float32) * 2 + 1
    T = np.stack([np.tanh(X[:, 0] + X[:, 3]), X[:, 5] * X[:, 6], np.abs(X[:, 9])], 1).astype(np.float32)
    p = init_params(seed)
    p[M.OFFS[0][1]:M.OFFS[0][1] + 128] = 0.05
    p[M.OFFS[1][1]:M.OFFS[1][1] + 128] = 0.02
    return p, make_stats(X, T), X, T


def _layers_close(g, ref, tol):
    for (k, n), (wo, bo) in zip(M.SHAPES, M.OFFS):
        for a, b in ((wo, wo + k * n), (bo, bo + n)):
            num = np.linalg.norm(g[a:b] - ref[a:b])
            den = np.linalg.norm(ref[a:b])
            assert num <= tol * max(den, 1e-12), (a, b, num, den)


@pytest.mark.parametrize("tc", [False, True], ids=["mma_sync", "tcgen05"])
@pytest.mark.parametrize("n", [64, 300, 1000])
def test_gradient_matches_oracle(mlp, n, tc):
    """Both tensor-core paths (tcgen05 with TMEM accumulators, and the
    mma.sync reference) against the CPU oracle's gradient."""
    p, st, X, T = _problem(n, n)
    mlp.set_params(p, st)
    mlp.set_data(X, T)
    idx = np.random.default_rng(5).permutation(n).astype(np.int32)
    prev = mlp.tensor_path(tc)
    try:
        g, loss = mlp.grad(idx)
    finally:
        mlp.tensor_path(prev)
    loss_o, g_o = M.loss_and_grad(p, st, X[idx], T[idx])
    assert abs(loss - loss_o) <= 1e-3 * loss_o
    # same rounding points, FP32 sums in another order: 1e-2 per layer
    _layers_close(g, g_o, 1e-2)
    # and the exact (float64, unrounded) gradient's direction
    _, g64 = M.loss_and_grad(p.astype(np.float64), st.astype(np.float64), X[idx], T[idx], exact=True)
    cos = g.astype(np.float64) @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64))
    assert cos > 0.999


@pytest.mark.parametrize("tc", [False, True], ids=["mma_sync", "tcgen05"])
def test_inference_matches_oracle(mlp, tc):
    p, st, X, T = _problem(7, 777)
    mlp.set_params(p, st)
    prev = mlp.tensor_path(tc)
    try:
        Y = mlp.infer(X)
    finally:
        mlp.tensor_path(prev)
    y, _ = M.forward(p, st, X)
    Yo = y * st[2 * M.NF + M.NO:] + st[2 * M.NF:2 * M.NF + M.NO]
    scale = np.abs(Yo).max(axis=0)
    assert (np.abs(Y - Yo).max(axis=0) <= 1e-2 * scale).all()


def _identity_net(s):
    """A network whose output is s * bf16(previous reaction) exactly:
    relu(x) - relu(-x) through the hidden layers."""
    W = [np.zeros(k * n, np.float32).reshape(k, n) for k, n in M.SHAPES]
    for c in range(3):
        W[0][13 + c, c] = 1.0
        W[0][13 + c, 3 + c] = -1.0
        W[3][c, c] = s
        W[3][3 + c, c] = -s
    for j in range(6):
        W[1][j, j] = 1.0
        W[2][j, j] = 1.0
    p = M.pack([(w, np.zeros(w.shape[1], np.float32)) for w in W])
    st = np.concatenate([np.zeros(M.NF), np.ones(M.NF), np.zeros(3), np.ones(3)]).astype(np.float32)
    return p, st


def test_identity_network_is_exact(mlp):
    p, st = _identity_net(0.5)
    mlp.set_params(p, st)
    X = np.random.default_rng(3).standard_normal((200, M.NF)).astype(np.float32)
    Y = mlp.infer(X)
    assert (Y == 0.5 * M.bf16(X[:, 13:16])).all()


def test_training_lowers_the_loss(mlp):
    p, st, X, T = _problem(11, 8192)
    mlp.set_params(p, st)
    mlp.set_data(X, T)
    val = np.arange(7168, 8192)
    l0 = mlp.loss(val)
    g = np.random.default_rng(0)
    for k in range(300):
        mlp.step(g.integers(0, 7168, 512), lr=3e-3, wd=0.0, want_loss=False)
    l1 = mlp.loss(val)
    assert l1 < 0.2 * l0, (l0, l1)


def _lattice_solver(r):
    from conftest import load_case
    from siconos_gb300.device import DeviceSolver
    P, ref = load_case("lattice_5x5x6_s1")
    d = DeviceSolver(0)
    d.set_W(P.nc, P.rowptr, P.colidx, P.blocks)
    d.set_q_mu(P.q, P.mu)
    d.set_r(r(P, ref))
    return d, P, ref


def test_device_features_match_host(built_lib):
    from siconos_gb300.learned import device_features, host_features
    rr = np.random.default_rng(2)
    d, P, _ = _lattice_solver(lambda P, ref: rr.standard_normal(3 * P.nc))
    try:
        r, _ = d.get()
        gap = np.linspace(-1e-3, 2e-3, P.nc)
        Xd = device_features(d, gap)
        Xh = host_features(P.nc, P.rowptr, P.colidx, P.blocks, P.q, P.mu, r, gap)
        assert (Xd == Xh).all()
        assert (device_features(d)[:, 16] == 0).all()
    finally:
        d.close()


def test_warm_start_takes_a_better_proposal(mlp):
    from siconos_gb300.learned import warm_start
    mlp.set_params(*_identity_net(0.5))
    # the context holds 2 r*: the proposal 0.5 * bf16(2 r*) is far better
    d, P, ref = _lattice_solver(lambda P, ref: 2.0 * ref["r"])
    try:
        out = warm_start(d, mlp)
        assert out["taken"] and out["error_proposal"] < out["error_fallback"]
        r, _ = d.get()
        np.testing.assert_allclose(r, ref["r"], rtol=1e-2, atol=1e-2 * np.abs(ref["r"]).max())
        assert abs(d.compute_error() - out["error_proposal"]) <= 1e-12
    finally:
        d.close()


def test_warm_start_keeps_a_better_fallback(mlp):
    from siconos_gb300.learned import warm_start
    mlp.set_params(*_identity_net(0.5))
    # the context holds r*: the proposal 0.5 r* is worse and is discarded
    d, P, ref = _lattice_solver(lambda P, ref: ref["r"])
    try:
        out = warm_start(d, mlp)
        assert not out["taken"] and out["error_proposal"] > out["error_fallback"]
        r, _ = d.get()
        assert (r == ref["r"]).all()
        assert d.compute_error() == out["error_fallback"]
        # the solve then starts from the kept reaction
        st = d.solve(tol=1e-300, max_iter=1, precision=1)
        assert st["sweeps64"] == 1
    finally:
        d.close()


def test_tensor_paths_agree(mlp):
    """tcgen05 and mma.sync compute the same products (same BF16 operands,
    FP32 sums in another order): proposals within 1e-3 of the output scale,
    gradients within 1e-2 per layer, on a batch that spans several tiles of
    either path (2,000 samples)."""
    p, st, X, T = _problem(11, 2000)
    mlp.set_params(p, st)
    mlp.set_data(X, T)
    idx = np.random.default_rng(3).permutation(2000).astype(np.int32)
    out = {}
    prev = mlp.tensor_path(False)
    try:
        for tc in (False, True):
            mlp.tensor_path(tc)
            out[tc] = (mlp.infer(X), *mlp.grad(idx))
    finally:
        mlp.tensor_path(prev)
    (y0, g0, l0), (y1, g1, l1) = out[False], out[True]
    scale = np.abs(y0).max(axis=0)
    assert (np.abs(y1 - y0).max(axis=0) <= 1e-3 * scale).all()
    assert abs(l1 - l0) <= 1e-4 * l0
    _layers_close(g1, g0, 1e-2)
