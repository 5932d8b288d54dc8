"""Device assembly of W = H M^-1 H^T and q = H (v + h g): bit-identical to the
scene generator's host assembly, and the device random walk."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(3, 3, 2), (5, 5, 6), (12, 10, 7)])
def test_device_W_and_q_equal_host(gpu, dims):
    from siconos_gb300.scene import lattice
    sc = lattice(*dims, seed=3, mu=0.4)
    geo = sc.contacts()
    gpu.set_contacts(geo)
    gpu.set_mu(sc.mu)
    gpu.set_velocities(geo["vel"], 1e-3)
    rp, ci, bl = gpu.get_W()
    assert (rp == sc.rowptr).all()
    assert (ci == sc.colidx).all()
    assert (bl == sc.blocks.reshape(-1, 9)).all()
    assert (gpu.get_q() == sc.q).all()
    # the assembled problem solves like the uploaded one
    gpu.zero_r()
    st1 = gpu.solve(tol=1e-300, max_iter=20, precision=1)
    r1, _ = gpu.get()
    gpu.load(sc)
    st2 = gpu.solve(tol=1e-300, max_iter=20, precision=1)
    r2, _ = gpu.get()
    assert (r1 == r2).all()
    # |q| is a fixed-order parallel sum on the device, a sequential one on the host
    assert abs(st1["error"] - st2["error"]) <= 1e-14 * st2["error"]


def test_random_walk(gpu):
    from siconos_gb300.scene import lattice
    sc = lattice(20, 20, 10, seed=4)
    geo = sc.contacts()
    gpu.set_contacts(geo)
    gpu.set_mu(sc.mu)
    gpu.set_velocities(geo["vel"], 1e-3)
    v0 = gpu.get_velocities()
    gpu.random_walk(77, 0.01)
    v1 = gpu.get_velocities()
    q1 = gpu.get_q()
    dv = v1 - v0
    assert abs(dv.mean()) < 5 * 0.01 / np.sqrt(dv.size)
    assert abs(dv.std() / 0.01 - 1) < 0.02
    # same seed from the same start: same velocities and q
    gpu.set_velocities(v0, 1e-3)
    gpu.random_walk(77, 0.01)
    assert (gpu.get_velocities() == v1).all() and (gpu.get_q() == q1).all()
    # q is H (v + h g) of the walked velocities, as the host generator forms it
    gpu.set_velocities(v1, 1e-3)
    assert (gpu.get_q() == q1).all()
