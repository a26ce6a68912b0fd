"""Host logic of contract_network without a GPU: the C++ greedy order equals the oracle's
greedy order (so GPU and oracle contract in the same sequence), left-associative steps,
argument checks."""
import numpy as np
import pytest

from oracle import contract_oracle as C
from itn_gb300 import graphs as G


def test_greedy_order_matches_oracle(lib_built):
    from itn_gb300.contract import contraction_order, norm_network_tensors
    for L, D in ((4, 2), (3, 3)):
        g = G.square_lattice(L, L, D, periodic=False, phys=2)
        t = G.random_tensors(g, np.random.default_rng(0), np.float64)
        ts, ls = norm_network_tensors(g, t)
        assert contraction_order([a.shape for a in ts], ls) == C.contraction_order_greedy([a.shape for a in ts], ls)


def test_left_associative_steps(lib_built):
    from itn_gb300.contract import contraction_order
    shapes = [(2, 3), (3, 4), (4, 5), (5, 2)]
    labels = [["a", "b"], ["b", "c"], ["c", "d"], ["d", "a"]]
    # working list after (0, 1): [t2, t3, acc]; then acc (position 2) with t2, then with t3
    assert contraction_order(shapes, labels, "left") == [(0, 1), (2, 0), (1, 0)]


def test_order_rejects_hyperedges(lib_built):
    from itn_gb300 import ItnArgumentError
    from itn_gb300.contract import contraction_order
    with pytest.raises(ItnArgumentError):
        contraction_order([(2,), (2,), (2,)], [["x"], ["x"], ["x"]])


def _order_cost(shapes, labels, steps):
    """Multiply-adds of a working-list order: per step the product of every index dimension
    of the two operands."""
    dim = {x: d for s, l in zip(shapes, labels) for d, x in zip(s, l)}
    work = [list(l) for l in labels]
    total = 0.0
    for i, j in steps:
        a, b = work[i], work[j]
        total += float(np.prod([dim[x] for x in a + [y for y in b if y not in a]], dtype=np.float64))
        lo = [x for x in a if x not in b] + [x for x in b if x not in a]
        work = [work[k] for k in range(len(work)) if k not in (i, j)] + [lo]
    assert len(work) == 1
    return total


def test_sweep_order_is_never_worse_than_greedy(lib_built):
    """order_alg "sweep" (itn_contraction_order alg 3) returns a valid working-list order whose
    multiply-adds are at most the greedy order's, and on lattice norm networks finds the
    boundary-sweep orders: the 6x6 D=3 PEPS norm network (72 tensors) drops from 3.3e11
    multiply-adds (greedy) to 2.2e9."""
    from itn_gb300.contract import contraction_order, norm_network_tensors, plain_network_tensors
    rng = np.random.default_rng(11)
    cases = []
    for L, D, per in ((6, 3, False), (4, 2, False), (5, 4, True), (3, 3, True)):
        g = G.square_lattice(L, L, D, periodic=per, phys=2)
        t = G.random_tensors(g, rng, np.float64)
        for f in (norm_network_tensors, plain_network_tensors):
            ts, ls = f(g, t)
            cases.append(([a.shape for a in ts], ls))
    for _ in range(30):  # small random networks, some disconnected, some with open indices
        n, nl = int(rng.integers(2, 10)), int(rng.integers(1, 16))
        held, labels = {}, []
        for t_ in range(n):
            ls_ = []
            for x in rng.integers(0, nl, size=int(rng.integers(0, 4))).tolist():
                if x not in ls_ and len(held.get(x, [])) < 2:
                    ls_.append(x)
                    held.setdefault(x, []).append(t_)
            labels.append(ls_)
        dims = {x: int(rng.integers(1, 5)) for x in range(nl)}
        cases.append(([tuple(dims[x] for x in l) for l in labels], labels))
    for shapes, labels in cases:
        sw = contraction_order(shapes, labels, "sweep")
        gr = contraction_order(shapes, labels, "greedy")
        assert len(sw) == len(shapes) - 1
        assert _order_cost(shapes, labels, sw) <= _order_cost(shapes, labels, gr)
    shapes, labels = cases[0]
    assert _order_cost(shapes, labels, contraction_order(shapes, labels, "greedy")) > 3e11
    assert _order_cost(shapes, labels, contraction_order(shapes, labels, "sweep")) < 2.5e9
