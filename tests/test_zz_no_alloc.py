"""fc3dgpu_compute_error_device: the error evaluation that allocates no
device memory (its scratch is a fixed array inside the library).  Compared
with fc3dgpu_compute_error, the context-based entry point, and directly with
the oracle's fc3d_compute_error (pinned to the reference's), on the same
inputs, over two calls in a row.  The 60x60x30 lattice (320,400 contacts,
1,252 chunks) is larger than four chunks per SM, so its blocks take several
chunks each.  Named to be collected last, so it also runs after every other
test has used the device."""
import ctypes as C

import numpy as np
import pytest

NUMERICS_ERR_INVALID_ARGUMENT = -2
MAX_CONTACTS = 4194304


def _call(lib, nc, nnz, d, norm_q, velocity, error, stream):
    return lib.fc3dgpu_compute_error_device(nc, nnz, d["rowptr"].data_ptr(), d["colidx"].data_ptr(),
                                            d["blocks"].data_ptr(), d["q"].data_ptr(), d["mu"].data_ptr(),
                                            d["r"].data_ptr(), norm_q, velocity.data_ptr() if velocity is not None
                                            else None, error.data_ptr(), stream)


def test_rejects_more_contacts_than_the_scratch_holds(built_lib):
    """Checked on the host before any device call (runs without a GPU)."""
    import siconos_gb300.numerics as sn
    rc = built_lib.fc3dgpu_compute_error_device(MAX_CONTACTS + 1, 0, None, None, None, None, None, None, 1.0,
                                                None, None, None)
    assert rc == NUMERICS_ERR_INVALID_ARGUMENT
    assert "exceed the limit" in sn.last_error()


def _reaction(nc, seed):
    g = np.random.default_rng(seed)
    r = np.empty((nc, 3))
    r[:, 0] = np.abs(g.standard_normal(nc))
    r[:, 1:] = 0.3 * g.standard_normal((nc, 2))
    return r.reshape(-1)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["fixture_FC3D_Example1_SBM", "lattice_5x5x6_s1", "lattice_40x40x20",
                                  "lattice_60x60x30"])
def test_matches_context_entry_point_twice(built_lib, case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device for a -m gpu run")
    import siconos_gb300.numerics as sn
    from siconos_gb300.scene import lattice
    if case in ("lattice_40x40x20", "lattice_60x60x30"):
        sc = lattice(*(int(x) for x in case[8:].split("x")), seed=3)
        nc, rowptr, colidx, blocks, q, mu = sc.nc, sc.rowptr, sc.colidx, sc.blocks.reshape(-1), sc.q, sc.mu
    else:
        from conftest import load_case
        P, _ = load_case(case)
        nc, rowptr, colidx, blocks, q, mu = P.nc, P.rowptr, P.colidx, P.blocks.reshape(-1), P.q, P.mu
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    colidx = np.ascontiguousarray(colidx, np.int64)
    blocks = np.ascontiguousarray(blocks, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    mu = np.ascontiguousarray(mu, np.float64)
    nnz = int(rowptr[-1])
    r = _reaction(nc, 11)
    norm_q = float(np.linalg.norm(q))

    # the context-based entry point (host buffers)
    W = sn.SparseBlockMatrix(nc, rowptr, colidx, blocks.reshape(nnz, 9))
    prob = sn.FrictionContactProblem(3, nc, W, q, mu)
    u_ref = np.zeros(3 * nc)
    info, err_ref = sn.fc3d_compute_error(prob, r.copy(), u_ref, 1e-300, norm_q)
    assert info in (0, 1)
    # and the oracle's (CPU, bit-exact with the reference's fc3d_compute_error)
    import oracle as O
    err_oracle, u_oracle = O.compute_error_port(O.Problem(nc, rowptr, colidx, blocks.reshape(nnz, 9), q, mu), r)

    dev = torch.device("cuda:0")
    d = {k: torch.from_numpy(v).to(dev) for k, v in
         dict(rowptr=rowptr, colidx=colidx, blocks=blocks, q=q, mu=mu, r=r).items()}
    velocity = torch.full((3 * nc,), float("nan"), dtype=torch.float64, device=dev)
    error = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize()

    rtol = 1e-12  # FP64 on both sides; only the order of the final sums differs
    for call in range(2):
        rc = _call(built_lib, nc, nnz, d, norm_q, velocity, error, stream)
        assert rc == 0, sn.last_error()
        torch.cuda.synchronize()
        e = float(error.item())
        u = velocity.cpu().numpy()
        assert abs(e - err_ref) <= rtol * abs(err_ref), (call, e, err_ref)
        assert abs(e - err_oracle) <= rtol * abs(err_oracle), (call, e, err_oracle)
        scale = max(1.0, float(np.abs(u_ref).max()))
        np.testing.assert_allclose(u, u_ref, rtol=rtol, atol=rtol * scale)
        np.testing.assert_allclose(u, u_oracle, rtol=rtol, atol=rtol * scale)
        velocity.fill_(float("nan"))
        error.fill_(float("nan"))
        torch.cuda.synchronize()
    # the set-up is done by now: calls change no device memory use.  The
    # free-memory figure is the whole device's, so another process could move
    # it: take the first of three rounds of ten calls in which it never drops.
    ok = False
    for _ in range(3):
        free0 = torch.cuda.mem_get_info(dev)[0]
        low = free0
        for _ in range(10):
            assert _call(built_lib, nc, nnz, d, norm_q, velocity, error, stream) == 0, sn.last_error()
            torch.cuda.synchronize()
            low = min(low, torch.cuda.mem_get_info(dev)[0])
        if low >= free0:
            ok = True
            break
    assert ok, "device free memory dropped during calls"


@pytest.mark.gpu
def test_bad_column_index_gives_nan_not_a_fault(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device for a -m gpu run")
    import siconos_gb300.numerics as sn
    dev = torch.device("cuda:0")
    nc = 2
    d = dict(rowptr=torch.tensor([0, 1, 2], dtype=torch.int64, device=dev),
             colidx=torch.tensor([0, 7], dtype=torch.int64, device=dev),
             blocks=torch.eye(3, dtype=torch.float64, device=dev).reshape(-1).repeat(2),
             q=torch.ones(6, dtype=torch.float64, device=dev), mu=torch.full((2,), 0.5, dtype=torch.float64,
                                                                            device=dev),
             r=torch.zeros(6, dtype=torch.float64, device=dev))
    error = torch.zeros(1, dtype=torch.float64, device=dev)
    rc = _call(built_lib, nc, 2, d, 1.0, None, error, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0, sn.last_error()
    torch.cuda.synchronize()
    assert np.isnan(error.item())
    # the next, valid call is unaffected
    d["colidx"] = torch.tensor([0, 1], dtype=torch.int64, device=dev)
    rc = _call(built_lib, nc, 2, d, 1.0, None, error, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0, sn.last_error()
    torch.cuda.synchronize()
    assert np.isfinite(error.item())


@pytest.mark.gpu
def test_host_memory_the_device_cannot_use_is_refused(built_lib):
    """Pageable host memory is refused on the host, before any device work."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device for a -m gpu run")
    import siconos_gb300.numerics as sn
    dev = torch.device("cuda:0")
    nc = 2
    d = dict(rowptr=torch.tensor([0, 1, 2], dtype=torch.int64, device=dev),
             colidx=torch.tensor([0, 1], dtype=torch.int64, device=dev),
             blocks=torch.eye(3, dtype=torch.float64, device=dev).reshape(-1).repeat(2),
             q=torch.ones(6, dtype=torch.float64, device=dev), mu=torch.full((2,), 0.5, dtype=torch.float64,
                                                                            device=dev),
             r=torch.zeros(6, dtype=torch.float64, device=dev))
    error = torch.zeros(1, dtype=torch.float64, device=dev)
    host_q = np.ones(6)
    rc = built_lib.fc3dgpu_compute_error_device(nc, 2, d["rowptr"].data_ptr(), d["colidx"].data_ptr(),
                                                d["blocks"].data_ptr(), host_q.ctypes.data, d["mu"].data_ptr(),
                                                d["r"].data_ptr(), 1.0, None, error.data_ptr(),
                                                torch.cuda.current_stream(dev).cuda_stream)
    assert rc == NUMERICS_ERR_INVALID_ARGUMENT
    assert "can access" in sn.last_error()


@pytest.mark.gpu
def test_another_devices_memory_is_refused(built_lib):
    """Memory of device 1 passed while device 0 is current is refused on the
    host (peer access may be off), not read by a kernel."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("one visible GPU")
    import siconos_gb300.numerics as sn
    d0, d1 = torch.device("cuda:0"), torch.device("cuda:1")
    nc = 2
    d = dict(rowptr=torch.tensor([0, 1, 2], dtype=torch.int64, device=d0),
             colidx=torch.tensor([0, 1], dtype=torch.int64, device=d0),
             blocks=torch.eye(3, dtype=torch.float64, device=d0).reshape(-1).repeat(2),
             q=torch.ones(6, dtype=torch.float64, device=d1), mu=torch.full((2,), 0.5, dtype=torch.float64,
                                                                           device=d0),
             r=torch.zeros(6, dtype=torch.float64, device=d0))
    error = torch.zeros(1, dtype=torch.float64, device=d0)
    torch.cuda.set_device(0)
    rc = _call(built_lib, nc, 2, d, 1.0, None, error, torch.cuda.current_stream(d0).cuda_stream)
    assert rc == NUMERICS_ERR_INVALID_ARGUMENT
    assert "can access" in sn.last_error()
