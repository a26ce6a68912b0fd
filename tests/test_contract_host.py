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
