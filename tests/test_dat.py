"""The .dat text format of friction-contact problems: this library's reader
and writer against each other and against the reference's own reader and
writer (oracle/_ref, where it was built), on every golden problem."""
import numpy as np
import pytest

from conftest import FIXTURE_CASES, LATTICE_CASES, load_case

CASES = FIXTURE_CASES + LATTICE_CASES


def _ours(path):
    import siconos_gb300.numerics as sn
    p = sn.read_dat(path)
    M = p._M
    return M.rowptr, M.colidx, M.blocks, p._q, p._mu


def _same(a, P):
    rp, ci, bl, q, mu = a
    assert (rp == P.rowptr).all() and (ci == P.colidx).all()
    assert (bl.reshape(-1) == np.asarray(P.blocks).reshape(-1)).all()
    assert (q == P.q).all() and (mu == P.mu).all()


@pytest.mark.parametrize("case", CASES)
def test_write_then_read(built_lib, tmp_path, case):
    import siconos_gb300.numerics as sn
    P, _ = load_case(case)
    prob = sn.FrictionContactProblem(3, P.nc, sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks), P.q, P.mu)
    f = tmp_path / "p.dat"
    sn.write_dat(prob, f)
    _same(_ours(f), P)


def _need_ref():
    import oracle as O
    if O.ref() is None:
        pytest.skip("oracle/_ref (the reference built from its sources) is not here")
    return O


@pytest.mark.parametrize("case", CASES)
def test_reference_reads_our_file(built_lib, tmp_path, case):
    O = _need_ref()
    import siconos_gb300.numerics as sn
    P, _ = load_case(case)
    prob = sn.FrictionContactProblem(3, P.nc, sn.SparseBlockMatrix(P.nc, P.rowptr, P.colidx, P.blocks), P.q, P.mu)
    f = tmp_path / "p.dat"
    sn.write_dat(prob, f)
    R = O.read_dat(f)
    assert (R.rowptr == P.rowptr).all() and (R.colidx == P.colidx).all()
    assert (np.asarray(R.blocks).reshape(-1) == np.asarray(P.blocks).reshape(-1)).all()
    assert (R.q == P.q).all() and (R.mu == P.mu).all()


@pytest.mark.parametrize("dense", [False, True])
@pytest.mark.parametrize("case", CASES)
def test_we_read_the_reference_file(built_lib, tmp_path, case, dense):
    O = _need_ref()
    P, _ = load_case(case)
    if dense and P.nc > 600:
        pytest.skip("dense file too large for a quick test")
    f = tmp_path / "r.dat"
    O.write_dat_ref(P, f, dense=dense)
    rp, ci, bl, q, mu = _ours(f)
    if not dense:
        _same((rp, ci, bl, q, mu), P)
    else:
        # dense: blocks holding a nonzero (and the diagonal), as the oracle converts them
        R = O.read_dat(f)
        _same((rp, ci, bl, q, mu), R)


def test_bad_files_rejected(built_lib, tmp_path):
    import siconos_gb300.numerics as sn
    f = tmp_path / "bad.dat"
    f.write_text("4\n5\n")
    with pytest.raises(ValueError, match="dimension"):
        sn.read_dat(f)
    f.write_text("3\n2\n5\n6\n6\n")
    with pytest.raises(ValueError, match="storage type"):
        sn.read_dat(f)
    with pytest.raises(ValueError, match="cannot open"):
        sn.read_dat(tmp_path / "missing.dat")
