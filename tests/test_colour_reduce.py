"""Host Kempe-chain reduction of contact colourings (fc3dgpu_colour_reduce):
the result is a proper colouring of the conflict graph with no more colours
than the input, independent of the order of the adjacency lists, and on the
sphere lattices (bipartite body graphs of degree 6) it reaches the 6 colours
Konig's theorem allows, from the greedy colouring's 8."""
import numpy as np
import pytest

from conftest import FIXTURE_CASES, LATTICE_CASES, load_case

GREEDY = 4 << 8  # hash priority + 4 recolouring passes, no Kempe step


def conflict_graph(P, seed=None):
    """Symmetric CSR of the contact conflict graph (a W block between two
    contacts); with a seed, each adjacency list is shuffled."""
    rows = np.repeat(np.arange(P.nc), np.diff(P.rowptr))
    m = rows != P.colidx
    i = np.concatenate([rows[m], P.colidx[m]])
    j = np.concatenate([P.colidx[m], rows[m]])
    key = np.random.default_rng(seed).random(i.size) if seed is not None else j
    order = np.lexsort((key, i))
    gptr = np.zeros(P.nc + 1, np.int64)
    np.add.at(gptr, i + 1, 1)
    return np.cumsum(gptr).astype(np.int32), j[order].astype(np.int32)


def reduce(P, col, ncol, seed=None, cap=0):
    import siconos_gb300.numerics as sn
    gptr, adj = conflict_graph(P, seed)
    out = col.copy()
    n = sn.lib().fc3dgpu_colour_reduce(P.nc, gptr, adj, out, ncol, cap)
    return n, out


def greedy(P):
    import oracle as O
    col = np.zeros(P.nc, np.int32)
    n = O.port().oracle_colour_greedy(P.nc, P.rowptr, P.colidx, GREEDY, col)
    return n, col


@pytest.mark.parametrize("case", FIXTURE_CASES + LATTICE_CASES)
def test_reduction_is_proper_and_never_worse(built_lib, case):
    import oracle as O
    P, _ = load_case(case)
    n0, col = greedy(P)
    n1, out = reduce(P, col, n0)
    assert 1 <= n1 <= n0
    assert out.min() >= 0 and out.max() == n1 - 1
    assert O.port().oracle_colour_check(P.nc, P.rowptr, P.colidx, out) == 0
    # the same colouring whatever the order of the adjacency lists
    n2, out2 = reduce(P, col, n0, seed=7)
    assert n2 == n1 and np.array_equal(out, out2)


@pytest.mark.parametrize("dims", [(5, 5, 6), (20, 20, 10)])
def test_lattice_reaches_six_colours(built_lib, dims):
    import oracle as O
    from siconos_gb300 import scene
    s = scene.lattice(*dims, seed=1)
    P = O.Problem(s.nc, s.rowptr, s.colidx, s.blocks, s.q, s.mu)
    n0, col = greedy(P)
    assert n0 >= 7
    n1, out = reduce(P, col, n0)
    assert n1 == 6
    assert O.port().oracle_colour_check(P.nc, P.rowptr, P.colidx, out) == 0


def test_search_cap_keeps_the_colouring_proper(built_lib):
    """With Kempe searches capped at one vertex only direct recolouring is
    left: fewer colours or the same, always proper."""
    import oracle as O
    from siconos_gb300 import scene
    s = scene.lattice(12, 12, 6, seed=3)
    P = O.Problem(s.nc, s.rowptr, s.colidx, s.blocks, s.q, s.mu)
    n0, col = greedy(P)
    n1, out = reduce(P, col, n0, cap=1)
    assert 6 <= n1 <= n0
    assert O.port().oracle_colour_check(P.nc, P.rowptr, P.colidx, out) == 0


@pytest.mark.parametrize("threads", [1, 3, 16])
def test_batch_groups_reduce_as_alone(built_lib, threads):
    """fc3dgpu_colour_reduce_groups on a batch of independent lattices (their
    conflict graphs side by side): each group gets exactly the colouring
    fc3dgpu_colour_reduce gives it alone, whatever the number of threads, and
    the return value is the largest number of colours."""
    import oracle as O
    import siconos_gb300.numerics as sn
    from siconos_gb300 import scene
    dims = [(3, 3, 2), (7, 5, 3), (12, 12, 6), (4, 9, 2), (5, 5, 6), (2, 2, 2), (9, 3, 4)]
    gp_all, adj_all, col_all, off, alone, counts = [0], [], [], [0], [], []
    for k, d in enumerate(dims):
        s = scene.lattice(*d, seed=k + 1)
        P = O.Problem(s.nc, s.rowptr, s.colidx, s.blocks, s.q, s.mu)
        n0, col = greedy(P)
        gptr, adj = conflict_graph(P)
        gp_all.extend((gptr[1:] + gp_all[-1]).tolist())
        adj_all.append(adj + off[-1])
        col_all.append(col)
        n1, out = reduce(P, col, n0)
        alone.append(out)
        counts.append(n1)
        off.append(off[-1] + P.nc)
    gp = np.asarray(gp_all, np.int32)
    adj = np.concatenate(adj_all).astype(np.int32)
    col = np.concatenate(col_all).astype(np.int32)
    r = sn.lib().fc3dgpu_colour_reduce_groups(len(dims), np.asarray(off, np.int32), gp, adj, col, threads)
    assert r == max(counts)
    np.testing.assert_array_equal(col, np.concatenate(alone))
