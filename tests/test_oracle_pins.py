"""Pins of the CPU oracle against the reference's own known-answer tests.

The reference (Julia) cannot run here, so the oracle is pinned by the analytic and
exactness checks its test suite holds for this path:
* BP is exact on trees: chain (2,1) and comb (4,3) with all-ones messages, one sweep
  (test/test_beliefpropagation.jl:157-202), for Float32/Float64/ComplexF64;
* spin ice on an n x n torus: exp(bethe_free_energy) = 1.5^(n^2)
  (test/test_beliefpropagation.jl:204-225);
* iterate_diff of identical caches is 0 within 10 eps (test_beliefpropagation.jl:134-150);
* incoming_messages excludes the reverse edge (test_beliefpropagation.jl:104-114);
* <psi|psi> = |psi|^2 for a norm network (test/test_normnetwork.jl:148-166);
* contraction order independence (test/test_contract_network.jl:26-45);
* 1D Ising free energy, open and periodic (test/test_itensornetworkgenerators.jl:29-54)
  and 2D Ising at beta_c vs Onsager within 10 % (:55-75).
"""
import numpy as np
import pytest

from oracle import contract_oracle as C
from oracle import oracle as O
from itn_gb300 import generators as GEN
from itn_gb300 import graphs as G


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
@pytest.mark.parametrize("case", ["chain", "comb"])
def test_tree_exactness(dtype, case):
    rng = np.random.default_rng(123)
    if case == "chain":
        g = G.from_edges(2, G.path_edges(2), 2, phys=1, layers=1)
    else:
        g = G.from_edges(12, G.comb_tree_edges(4, 3), 3, phys=1, layers=1)
    t = G.random_tensors(g, rng, dtype)
    m0 = G.ones_messages(g, dtype)
    m, it, _, _ = O.bp_run(g, t, m0, schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=1)
    assert it == 1
    z_bp = np.exp(O.bethe_free_energy(g, t, m))
    z_ex, lo = C.contract_plain(g, t.astype(np.complex128 if np.iscomplexobj(t) else np.float64))
    rtol = np.finfo(np.dtype(dtype).type(0).real.dtype).eps ** (1 / 3)
    assert abs(z_bp - z_ex) <= rtol * abs(z_ex)


def test_norm_network_tree_exactness():
    rng = np.random.default_rng(7)
    g = G.from_edges(12, G.comb_tree_edges(4, 3), 3, phys=2, layers=2)
    t = G.random_tensors(g, rng, np.complex128)
    m0 = G.identity_messages(g, np.complex128)
    m, *_ = O.bp_run(g, t, m0, schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=1)
    z_bp = np.exp(O.bethe_free_energy(g, t, m))
    z_ex = C.contract_norm(g, t)
    assert abs(z_bp - z_ex) <= 1e-10 * abs(z_ex)
    # the parallel schedule reaches the same fixed point after enough sweeps
    m, *_ = O.bp_run(g, t, m0, schedule="parallel", maxiter=12)
    assert abs(np.exp(O.bethe_free_energy(g, t, m)) - z_ex) <= 1e-10 * abs(z_ex)


@pytest.mark.parametrize("n", [3, 4, 5])
def test_spin_ice(n):
    rng = np.random.default_rng(123)
    g = G.square_lattice(n, n, 2, periodic=True, phys=1, layers=1)
    t = GEN.spin_ice_tensors(g)
    m0 = G.random_messages(g, rng)
    m, it, delta, _ = O.bp_run(g, t, m0, schedule="sequential", edges=G.tree_edge_sequence(g),
                               maxiter=10, tol=1e-10)
    z = np.exp(O.bethe_free_energy(g, t, m))
    assert abs(z / 1.5 ** (n * n) - 1) < 1e-6


def test_iterate_diff_identical():
    rng = np.random.default_rng(1)
    g = G.square_lattice(3, 3, 2, phys=2)
    m = G.random_messages(g, rng)
    assert abs(O.iterate_diff(g.moff, m, m.copy())) <= 10 * np.finfo(float).eps


def test_incoming_excludes_reverse():
    """Path 1-2-3 (0-based 0-1-2): the update of 1->2 reads only 0->1; 0->1 reads none."""
    g = G.from_edges(3, G.path_edges(3), 2, phys=1, layers=1)
    t = np.arange(1, int(g.toff[-1]) + 1, dtype=np.float64)
    m = G.ones_messages(g)
    s01, s12, s21 = g.slot(0, 1), g.slot(1, 2), g.slot(2, 1)
    # an update of 0->1 does not depend on any message (vertex 0 has one leg)
    m2 = m.copy()
    m2[g.moff[g.slot(1, 0)]:g.moff[g.slot(1, 0) + 1]] = 123.0
    a = O.message_update(g, t, m.copy(), s01)
    b = O.message_update(g, t, m2.copy(), s01)
    assert np.array_equal(a[g.moff[s01]:g.moff[s01 + 1]], b[g.moff[s01]:g.moff[s01 + 1]])
    # the update of 1->2 ignores the reverse message 2->1
    m3 = m.copy()
    m3[g.moff[s21]:g.moff[s21 + 1]] = 5.0
    a = O.message_update(g, t, m.copy(), s12)
    b = O.message_update(g, t, m3.copy(), s12)
    assert np.array_equal(a[g.moff[s12]:g.moff[s12 + 1]], b[g.moff[s12]:g.moff[s12 + 1]])


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_norm_equals_state_norm(dtype):
    rng = np.random.default_rng(5)
    g = G.square_lattice(2, 2, 2, phys=2)
    t = G.random_tensors(g, rng, dtype)
    ts, ls = C.plain_network(g, t)
    psi, _ = C.contract_network(ts, ls)
    z = C.contract_norm(g, t)
    ref = np.vdot(psi, psi)
    assert abs(z - ref) <= 1e-12 * abs(ref)
    assert abs(np.imag(z)) <= 1e-12 * abs(z)
    assert np.real(z) > 0


def test_contraction_order_independence():
    rng = np.random.default_rng(3)
    g = G.square_lattice(4, 4, 2, phys=1, layers=1)
    t = G.random_tensors(g, rng, np.float64)
    z1, _ = C.contract_plain(g, t, "left")
    z2, _ = C.contract_plain(g, t, "greedy")
    assert abs(z1 - z2) / abs(z1) <= 1e3 * np.finfo(float).eps


@pytest.mark.parametrize("periodic", [False, True])
def test_ising_1d(periodic):
    beta = 0.4
    edges = G.cycle_edges(4) if periodic else G.path_edges(4)
    g = G.from_edges(4, edges, 2, phys=1, layers=1)
    t = GEN.ising_network(g, beta)
    z, _ = C.contract_plain(g, t)
    f = -np.log(z) / (beta * 4)
    assert np.isclose(f, GEN.f_1d_ising(beta, 4, periodic=periodic), rtol=1e-12)
    if not periodic:  # BP is exact on the open chain
        m, *_ = O.bp_run(g, t, G.ones_messages(g), schedule="sequential",
                         edges=G.tree_edge_sequence(g), maxiter=1)
        assert np.isclose(np.exp(O.bethe_free_energy(g, t, m)), z, rtol=1e-12)


def test_ising_2d_onsager():
    beta = GEN.beta_c_2d_ising()
    g = G.square_lattice(4, 4, 2, periodic=True, phys=1, layers=1)
    t = GEN.ising_network(g, beta)
    z, _ = C.contract_plain(g, t)
    f = -np.log(z) / (beta * 16)
    assert np.isclose(f, GEN.f_2d_ising(beta), rtol=0.1)


def test_stopping_criterion_semantics():
    """StopWhenConverged skips iteration 0 and fires at the first delta < tol; maxiter
    caps the outer loop (AlgorithmsInterfaceExtensions.jl:84-118)."""
    rng = np.random.default_rng(11)
    g = G.square_lattice(4, 4, 2, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g)
    _, it, delta, at = O.bp_run(g, t, m0, maxiter=3)
    assert it == 3 and at == -1 and delta == np.inf
    _, it, delta, at = O.bp_run(g, t, m0, tol=1e-8)
    assert it == at and delta < 1e-8
    _, it0, *_ = O.bp_run(g, t, m0, maxiter=0)
    assert it0 == 0
    with pytest.raises(ValueError):
        O.bp_run(g, t, m0)
