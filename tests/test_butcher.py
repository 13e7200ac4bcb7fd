"""The Runge-Kutta tables of the library (gbmv_butcher_table, CPU: no GPU needed): every table
satisfies the order conditions of its method order q and embedding order p (rooted trees up to
order 5), the additive pairs (2, 104) and (13, 112) the coupled IMEX conditions of their order,
the implicit tables are stiffly accurate ESDIRKs with L-stable stability functions, and the
library's copies of the DIRK tables equal the oracle's bit for bit."""
import itertools

import numpy as np
import pytest

import oracle_py as O

ERK = [0, 1, 2, 3, 6, 8, 13]
DIRK = [102, 104, 112]
PAIRS = [(2, 104), (13, 112)]


def _trees(order):
    """Rooted trees with `order` nodes, each a sorted tuple of child subtrees."""
    if order == 1:
        return [()]
    out = set()

    def parts(n, maxpart):  # multisets of subtree sizes summing to n
        if n == 0:
            yield []
            return
        for k in range(min(n, maxpart), 0, -1):
            for rest in parts(n - k, k):
                yield [k] + rest

    for sizes in parts(order - 1, order - 1):
        for combo in itertools.product(*[_trees(k) for k in sizes]):
            out.add(tuple(sorted(combo)))
    return sorted(out)


def _gamma(t):
    n, g = 1, 1
    for ch in t:
        n += _size(ch)
        g *= _gamma(ch)
    return n * g


def _size(t):
    return 1 + sum(_size(ch) for ch in t)


def _phi(t, mats, colors):
    """Stage vector of tree t with each child edge's matrix from `colors` (an iterator)."""
    v = np.ones(mats[0].shape[0])
    for ch in t:
        A = mats[next(colors)]
        v = v * (A @ _phi(ch, mats, colors))
    return v


def _edges(t):
    return sum(1 + _edges(ch) for ch in t)


def _max_defect(b, mats, order):
    worst = 0.0
    for q in range(1, order + 1):
        for t in _trees(q):
            for col in itertools.product(range(len(mats)), repeat=_edges(t)):
                d = abs(b @ _phi(t, mats, iter(col)) - 1.0 / _gamma(t))
                worst = max(worst, d)
    return worst


def _table(i):
    import gbmv
    return gbmv.butcher_table(i)


def test_tree_enumeration():
    assert [len(_trees(q)) for q in range(1, 6)] == [1, 1, 2, 4, 9]


@pytest.mark.parametrize("tid", ERK + DIRK)
def test_order_conditions(tid):
    T = _table(tid)
    A, b, bh, c = (np.array(T[k]) for k in ("A", "b", "bhat", "c"))
    assert np.allclose(A.sum(axis=1), c, atol=1e-15, rtol=0)
    assert _max_defect(b, [A], T["q"]) < 1e-14, T["name"]
    assert _max_defect(bh, [A], T["p"]) < 1e-14, T["name"]
    # the method is not of a higher order than claimed (the tables are not mislabelled)
    assert _max_defect(b, [A], T["q"] + 1) > 1e-6, T["name"]
    if tid in ERK:
        assert np.all(np.triu(A) == 0.0)


@pytest.mark.parametrize("ei", PAIRS)
def test_additive_pairs(ei):
    E, I = _table(ei[0]), _table(ei[1])
    assert E["c"] == I["c"] and E["b"] == I["b"] and E["bhat"] == I["bhat"]
    AE, AI, b, bh = (np.array(x) for x in (E["A"], I["A"], E["b"], E["bhat"]))
    assert _max_defect(b, [AE, AI], E["q"]) < 1e-14
    assert _max_defect(bh, [AE, AI], E["p"]) < 1e-14


@pytest.mark.parametrize("tid", DIRK)
def test_dirk_tables_are_stiffly_accurate_l_stable_esdirks(tid):
    T = _table(tid)
    A, b = np.array(T["A"]), np.array(T["b"])
    s = T["s"]
    assert A[0, 0] == 0.0 and np.all(np.triu(A, 1) == 0.0)
    assert np.all(np.diag(A)[1:] == A[1, 1])
    assert np.array_equal(A[-1], b)
    # stability function R(z) = 1 + z b^T (I - z A)^{-1} 1 -> 0 as z -> -inf, |R| <= 1 on
    # the negative real axis and the imaginary axis
    for z in [-1e8, -1e4, -10.0, -1.0] + [1j * w for w in (0.1, 1.0, 10.0, 1e3)]:
        R = 1.0 + z * b @ np.linalg.solve(np.eye(s) - z * A, np.ones(s))
        assert abs(R) <= 1.0 + 1e-12, (tid, z, R)
    R = 1.0 - 1e6 * b @ np.linalg.solve(np.eye(s) + 1e6 * A, np.ones(s))
    assert abs(R) < 1e-4  # R(z) = O(1/z): L-stable


@pytest.mark.parametrize("tid", [112, 102])
def test_library_dirk_tables_equal_the_oracle_copy(tid):
    T, R = _table(tid), O.DIRK_TABLES[tid]
    assert T["s"] == R["s"] and T["p"] == R["p"]
    for k in ("A", "b", "bhat", "c"):
        assert np.array_equal(np.array(T[k]), np.array(R[k])), k


def test_erk_default_tables_and_refusals():
    import gbmv
    assert [gbmv.erk_default_table(q) for q in (2, 3, 4, 5, 6)] == [0, 1, 3, 6, -1]
    with pytest.raises(gbmv.GbmvError):
        gbmv.butcher_table(5)
