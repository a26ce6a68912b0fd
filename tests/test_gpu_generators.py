"""Partition-function networks on the GPU (ITensorNetworkGenerators: ising_network,
delta_network), the known answers of test/test_itensornetworkgenerators.jl:

* 1D Ising, 4 sites, beta = 0.4, open and periodic: exact contraction gives the analytic
  free energy (test/utils.jl:12-39), and BP with one tree sweep is exact on the open chain;
* 2D Ising, 4x4 torus at beta_c: the exact free energy is within 10 % of Onsager's
  infinite-lattice value (:55-75), and the GPU agrees with the oracle to 1e-12;
* delta network on a 3x3 grid (:13-27): the contraction counts the global configurations
  (all indices equal), 2 for link dimension 2;
* BP on the 2D Ising network (single layer, field h = 0.1) agrees with the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import contract_oracle as C
from oracle import oracle as O
from itn_gb300 import BPEngine
from itn_gb300 import generators as GEN
from itn_gb300 import graphs as G
from itn_gb300.contract import contract_plain_network

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


@pytest.mark.parametrize("periodic", [False, True])
def test_ising_1d_free_energy(periodic):
    beta = 0.4
    edges = G.cycle_edges(4) if periodic else G.path_edges(4)
    g = G.from_edges(4, edges, 2, phys=1, layers=1)
    t = GEN.ising_network(g, beta)
    z = contract_plain_network(g, t)
    f = -np.log(z) / (beta * 4)
    assert np.isclose(f, GEN.f_1d_ising(beta, 4, periodic=periodic), rtol=1e-12)
    if not periodic:
        # one sweep over the tree edge sequence makes BP exact on the open chain
        with BPEngine(g) as e:
            e.set_tensors(t)
            e.set_messages(G.ones_messages(g))
            e.run(schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=1)
            assert np.isclose(np.exp(e.bethe_free_energy()), z, rtol=1e-12)


def test_ising_2d_onsager():
    beta = GEN.beta_c_2d_ising()
    g = G.square_lattice(4, 4, 2, periodic=True, phys=1, layers=1)
    t = GEN.ising_network(g, beta)
    z = contract_plain_network(g, t)
    ref, _ = C.contract_plain(g, t)
    assert abs(z - ref) <= 1e-12 * abs(ref)
    f = -np.log(z) / (beta * 16)
    assert np.isclose(f, GEN.f_2d_ising(beta), rtol=0.1)


def test_delta_network_counts_configurations():
    g = G.square_lattice(3, 3, 2, periodic=False, phys=1, layers=1)
    t = GEN.delta_tensors(g)
    assert np.isclose(contract_plain_network(g, t), 2.0, rtol=1e-14)


@pytest.mark.parametrize("beta", [0.2, 0.35])
def test_ising_2d_bp_matches_oracle(beta):
    # a field and perturbed messages, so that the all-ones start is not already the
    # fixed point (it is for h = 0)
    g = G.square_lattice(6, 6, 2, periodic=True, phys=1, layers=1)
    t = GEN.ising_network(g, beta, h=0.1)
    rng = np.random.default_rng(5)
    m0 = G.ones_messages(g) + 0.5 * rng.random(int(g.moff[-1]))
    ref, it, delta, at = O.bp_run(g, t, m0, maxiter=200, tol=1e-13)
    assert it > 10
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        r = e.run(maxiter=200, tol=1e-13)
        assert abs(r.iterations - it) <= 1
        got = e.bethe_free_energy()
    want = O.bethe_free_energy(g, t, ref)
    assert abs(got - want) <= 1e-10 * abs(want)
    # below the critical coupling BP is close to the exact free energy
    z = contract_plain_network(g, t)
    assert abs(got - np.log(z)) < 0.05 * abs(np.log(z))
