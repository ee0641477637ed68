"""The subtree scheduler (LLJBASH_Gb300TreeSchedule, the reference's tree_schedule of
src/subtree.hpp restated on the host) against the reference build, bit for bit: worker
partitions, queue rows, task queue and the elimination-tree subtree sizes and weights,
for the L-DAG and the reverse U-DAG, several worker counts, queue granularities and
relax factors, on matrices whose elimination trees are long chains (grids in natural
order) and bushy (random patterns, randomly permuted grids)."""
import numpy as np
import pytest

import oracle
from conftest import ragged, rel_err
from par_ilu0_cpp_gb300 import api
from par_ilu0_cpp_gb300 import generators as g


@pytest.fixture(scope="module")
def ref():
    try:
        return oracle.Ref(oracle.REF_SO)
    except OSError as e:
        pytest.skip(f"reference build not loadable here: {e}")


def permuted(a, seed):
    perm = np.random.default_rng(seed).permutation(a.n)
    sp = a.to_scipy()[perm][:, perm].tocsr()
    sp.sort_indices()
    return g.Csr(a.n, sp.indptr, sp.indices, sp.data)


MATS = [
    ("laplace2d_20", lambda: g.laplace2d(20)),
    ("convdiff3d_8", lambda: g.convdiff3d(8)),
    ("ragged_600", lambda: ragged(600, 6, seed=3)),
    ("laplace2d_24_permuted", lambda: permuted(g.laplace2d(24), 1)),
    ("convdiff3d_7_permuted", lambda: permuted(g.convdiff3d(7), 2)),
    ("lognormal27_6_ilu1", lambda: api.iluk_symbolic(g.lognormal27(6, seed=1), 1)[0]),
]


@pytest.mark.parametrize("name,make", MATS, ids=[m[0] for m in MATS])
@pytest.mark.parametrize("upper", [False, True], ids=["L", "U"])
def test_tree_schedule_bit_exact(ref, name, make, upper):
    a = make()
    for nproc in (1, 2, 4, 8, 16):
        for granularity in (1, 8):
            for relax in (1.0, 0.7):
                mine = api.tree_schedule(a, upper, nproc, granularity, relax)
                theirs = ref.tree_schedule(a, upper, nproc, granularity, relax)
                for key in ("part_ptr", "partitions", "task_queue", "subtree_size", "subtree_weight"):
                    assert np.array_equal(mine[key], theirs[key]), (key, nproc, granularity, relax)


def test_tree_schedule_is_a_topological_order():
    """Workers' rows, interleaved, then the queue rows: every row after its dependencies."""
    a = permuted(g.laplace2d(30), 4)
    s = api.tree_schedule(a, False, 8, 1)
    order = s["partitions"]
    rank = np.empty(a.n, dtype=np.int64)
    rank[order] = np.arange(a.n)
    diag = api.analyze_pattern(a)["diag"]
    for r in range(a.n):
        deps = a.col_idx[a.row_ptr[r]:diag[r]]
        assert np.all(rank[deps] < rank[r])


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", MATS + [("convdiff3d_24_permuted", lambda: permuted(g.convdiff3d(24), 5))],
                         ids=[m[0] for m in MATS] + ["convdiff3d_24_permuted"])
def test_factorisation_in_subtree_schedule_order(name, make):
    """The factorisation kernel taking rows in the subtree scheduler's order gives the
    factors of the level order bit for bit."""
    f = make()
    out = []
    for order in (0, 1, 2):
        ilu = api.IluSolver()
        ilu.set_option(api.ILU_OPT_TICKET_ORDER, order)
        ilu.set_matrix(f)
        assert ilu.setup() == 0, api.last_error()
        assert ilu.factorize() == 0, api.last_error()
        out.append(ilu.values())
    assert np.array_equal(out[0], out[1])
    assert np.array_equal(out[0], out[2])


SUBTREE_MATS = [
    ("convdiff3d_32_nd", lambda: api.reorder(g.convdiff3d(32), "nd")),
    ("laplace2d_96_nd", lambda: api.reorder(g.laplace2d(96), "nd")),
    ("lognormal27_12_ilu1_nd", lambda: api.iluk_symbolic(api.reorder(g.lognormal27(12, seed=3), "nd"), 1)[0]),
    ("convdiff3d_24_amd", lambda: api.reorder(g.convdiff3d(24), "amd")),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,make", SUBTREE_MATS, ids=[m[0] for m in SUBTREE_MATS])
def test_subtree_partitions_one_cta_each(name, make):
    """Fill-reducing orders give the elimination tree wide independent subtrees: most rows
    are factorised by subtree CTAs without waiting on any other CTA, and the factors (and
    the substitution) are those of the level-ordered kernel bit for bit, 1e-12 against the
    oracle."""
    import oracle

    f = make()
    ref = api.IluSolver()
    ref.set_matrix(f)
    assert ref.setup() == 0 and ref.factorize() == 0, api.last_error()
    ilu = api.IluSolver()
    ilu.set_option(api.ILU_OPT_TICKET_ORDER, 2)
    ilu.set_matrix(f)
    assert ilu.setup() == 0, api.last_error()
    assert ilu.factorize() == 0, api.last_error()
    info = ilu.info()
    assert info.factor_subtree_parts > 1 and info.factor_subtree_rows > f.n // 2, (info.factor_subtree_parts,
                                                                                  info.factor_subtree_rows)
    assert np.array_equal(ilu.values(), ref.values())
    oracle.build_port()
    port = oracle.Port()
    lu, _ = port.factorize(f)
    assert rel_err(ilu.values(), lu, floor=1e-300) <= 1e-12
    b = np.random.default_rng(3).uniform(-1, 1, f.n)
    assert np.array_equal(ilu.substitute(b), ref.substitute(b))
