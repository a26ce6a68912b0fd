"""Edge cases of the BP engine against the oracle: empty networks, isolated vertices,
degree-one and high-degree vertices, bond dimensions outside the compiled set (runtime
loop bounds), and vertices too large for shared memory (global-memory scratch buffers).
FP64 bound 1e-10 relative, as in test_gpu_bp.py."""
import numpy as np
import pytest

from oracle import oracle as O
from itn_gb300 import BPEngine, ItnArgumentError
from itn_gb300 import graphs as G
from helpers import msg_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _compare(g, t, m0, sweeps, tol=1e-10):
    ref, *_ = O.bp_run(g, t, m0, maxiter=sweeps)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        r = e.run(maxiter=sweeps)
        assert r.iterations == sweeps
        assert msg_rel(g, e.messages(), ref) < tol
        rr = O.logscalars(g, t, ref)
        got = e.logscalars()
        assert abs(got["totals"][0][0] - rr["total"][0]) < tol * max(1.0, abs(rr["total"][0]))


def test_runtime_bond_dimension_path():
    """D = 10 is not among the compiled bond dimensions: runtime-bound loops."""
    rng = np.random.default_rng(10)
    g = G.square_lattice(3, 3, 10, periodic=True, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    _compare(g, t, G.identity_messages(g), 3)


def test_global_scratch_path():
    """D = 12, z = 4, FP64: one vertex buffer is 332 KB, beyond shared memory, so the
    contraction buffers live in per-CTA global scratch."""
    rng = np.random.default_rng(12)
    g = G.square_lattice(3, 3, 12, periodic=True, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    _compare(g, t, G.identity_messages(g), 2)


def test_star_graph_mixed_degrees():
    """A hub of degree 8 with leaves of degree 1, uneven bonds {2, 3}."""
    rng = np.random.default_rng(8)
    edges = [(0, k) for k in range(1, 9)]
    bonds = [2, 3, 2, 3, 2, 3, 2, 3]
    g = G.from_edges(9, edges, bonds, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    _compare(g, t, G.identity_messages(g), 4)


def test_isolated_vertices_and_empty_network():
    rng = np.random.default_rng(1)
    # two isolated vertices: Z_v = sum |A|^2, no edge scalars
    g = G.from_edges(2, [], [], phys=3)
    t = G.random_tensors(g, rng, np.float64)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        r = e.run(maxiter=3)
        assert r.iterations == 3
        with pytest.raises(ItnArgumentError):
            e.run(tol=1e-8)
        got = e.logscalars()
    ref = np.log([np.sum(t[:3] ** 2), np.sum(t[3:] ** 2)]).sum()
    assert abs(got["totals"][0][0] - ref) < 1e-12 * abs(ref)
    # a network with no vertices
    g0 = G.from_edges(0, [], [], phys=2)
    with BPEngine(g0) as e:
        e.set_tensors(np.zeros(0))
        e.init_messages()
        assert e.run(maxiter=2).iterations == 2
        assert e.logscalars()["totals"][0][0] == 0.0


def test_mixed_component_with_isolated_vertex():
    """A 3x3 lattice plus one isolated vertex in the same network."""
    rng = np.random.default_rng(5)
    base = G.square_lattice_edges(3, 3)
    g = G.from_edges(10, base, 3, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    _compare(g, t, G.identity_messages(g), 5)
