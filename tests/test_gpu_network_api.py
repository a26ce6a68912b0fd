"""The reference's test cases, through the mirrored named-tensor API on the GPU
(test/test_beliefpropagation.jl, test/test_normnetwork.jl, test/test_contract_network.jl)."""
import itertools

import numpy as np
import pytest

from itn_gb300 import network as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _grid_links(nx, ny, D, periodic=False):
    """Edges of an nx x ny grid with one Index per edge; vertex (x, y)."""
    links = {}
    for x in range(nx):
        for y in range(ny):
            for dx, dy in ((1, 0), (0, 1)):
                if (x + dx < nx and y + dy < ny) or periodic:
                    w = ((x + dx) % nx, (y + dy) % ny)
                    if w != (x, y):
                        links[((x, y), w)] = N.Index(D)
    return links


def _incident(links, v):
    return [i for (a, b), i in links.items() if v in (a, b)]


def _comb_links(nx, ny, D):
    links = {}
    for x in range(nx):
        if x + 1 < nx:
            links[((x, 0), (x + 1, 0))] = N.Index(D)
        for y in range(ny - 1):
            links[((x, y), (x, y + 1))] = N.Index(D)
    return links


def _random_tn(links, vertices, dtype, rng, site=None):
    ts = {}
    for v in vertices:
        inds = ([site[v]] if site else []) + _incident(links, v)
        shape = tuple(i.dim for i in inds)
        data = rng.standard_normal(shape)
        if np.dtype(dtype).kind == "c":
            data = data + 1j * rng.standard_normal(shape)
        ts[v] = N.ITensor(data.astype(dtype), inds)
    return N.ITensorNetwork(ts)


def _ones_messages(tn, dtype):
    return N.messagecache(lambda e: N.ITensor(np.ones(tuple(tn[e[0]].inds[tn[e[0]].dimnames.index(n)].dim
                                                          for n in tn.linknames(*e)), dtype=dtype),
                                               [N.Index(tn[e[0]].inds[tn[e[0]].dimnames.index(n)].dim, n)
                                                for n in tn.linknames(*e)]),
                          [x for u, v in tn.edges() for x in ((u, v), (v, u))])


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_tree_exactness(dtype):
    """test_beliefpropagation.jl:157-202: chain (2,1) D=2 and comb (4,3) D=3, all-ones
    messages, one sweep: exp(bethe_free_energy) = exact contraction."""
    rng = np.random.default_rng(123)
    for links, verts in ((_grid_links(2, 1, 2), [(0, 0), (1, 0)]),
                         (_comb_links(4, 3, 3), [(x, y) for x in range(4) for y in range(3)])):
        tn = _random_tn(links, verts, dtype, rng)
        cache = N.beliefpropagation(tn, _ones_messages(tn, dtype), stopping_criterion={"maxiter": 1})
        z_bp = np.exp(N.bethe_free_energy(tn, cache))
        z_exact = N.contract_network(tn)[()]
        rtol = np.finfo(np.dtype(dtype).type(0).real.dtype).eps ** (1 / 3)
        assert abs(z_bp - z_exact) <= rtol * abs(z_exact)


@pytest.mark.parametrize("n", [3, 4, 5])
def test_spin_ice(n):
    """test_beliefpropagation.jl:204-225: BP partition function 1.5^(n^2) on an n x n torus."""
    rng = np.random.default_rng(123)
    links = _grid_links(n, n, 2, periodic=True)
    verts = [(x, y) for x in range(n) for y in range(n)]
    ts = {}
    for v in verts:
        inds = _incident(links, v)
        T = np.zeros((2,) * len(inds))
        for idx in itertools.product(*[range(2)] * len(inds)):
            if sum(idx) == 2:
                T[idx] = 1
        ts[v] = N.ITensor(T, inds)
    tn = N.ITensorNetwork(ts)
    msgs = N.messagecache(
        lambda e: N.ITensor(rng.random(2), [N.Index(2, tn.linknames(*e)[0])]),
        [x for u, v in tn.edges() for x in ((u, v), (v, u))])
    cache = N.beliefpropagation(tn, msgs, stopping_criterion={"maxiter": 10, "tol": 1e-10})
    z = np.exp(N.bethe_free_energy(tn, cache))
    assert abs(z / 1.5 ** (n * n) - 1) < 1e-6


def test_vertex_region_scalars():
    """test_beliefpropagation.jl:83-115: path of 3, ComplexF32 tensors, ones messages."""
    rng = np.random.default_rng(1)
    links = {((0,), (1,)): N.Index(2), ((1,), (2,)): N.Index(2)}
    tn = _random_tn(links, [(0,), (1,), (2,)], np.complex64, rng)
    cache = _ones_messages(tn, np.complex64)
    v = N.vertex_scalar(tn, cache, (1,))
    assert np.iscomplexobj(v)
    assert np.isclose(N.region_scalar(tn, cache, [(0,)]), N.vertex_scalar(tn, cache, (0,)))
    assert np.isclose(N.region_scalar(tn, cache, [(1,), (2,)]),
                      np.prod(N.vertex_scalars(tn, cache, [(1,), (2,)])), rtol=1e-6)
    assert np.isclose(N.edge_scalar(cache, ((0,), (1,))), 2.0)
    assert abs(N.iterate_diff(cache, cache.copy())) <= 10 * np.finfo(float).eps


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_norm_network_contraction(dtype):
    """test_normnetwork.jl:148-166: <psi|psi> = |prod(tn)|^2, real, rescaling gives 1, and
    independence of the bra name map."""
    rng = np.random.default_rng(7)
    links = _grid_links(2, 2, 2)
    verts = [(x, y) for x in range(2) for y in range(2)]
    site = {v: N.Index(2) for v in verts}
    tn = _random_tn(links, verts, dtype, rng, site)
    z = N.contract_network(N.NormNetwork(tn))[()]
    psi = N.contract_network(tn).data
    assert abs(z - np.vdot(psi, psi)) <= 1e-12 * abs(z)
    assert abs(np.imag(z)) <= 1e-12 * abs(z) and np.real(z) > 0
    v0 = verts[0]
    tn[v0] = N.ITensor(tn[v0].data / np.sqrt(np.real(z)), tn[v0].inds)
    assert np.isclose(N.contract_network(N.NormNetwork(tn))[()], 1.0)
    custom = {n: ("custom", k) for k, n in enumerate(tn.dimname_vertices)}
    assert np.isclose(N.contract_network(N.normnetwork(tn, custom))[()],
                      N.contract_network(N.NormNetwork(tn))[()])


def test_single_normalized_tensor_contracts_to_one():
    """test_normnetwork.jl:137-146: <psi|psi> of one normalised site tensor is 1."""
    rng = np.random.default_rng(8)
    s = N.Index(3)
    v = rng.standard_normal(3)
    tn = N.ITensorNetwork({1: N.ITensor(v / np.linalg.norm(v), [s])})
    assert np.isclose(N.contract_network(N.NormNetwork(tn))[()], 1.0, rtol=1e-14)


def test_bp_on_norm_network_matches_exact_on_tree():
    """BP on a NormNetwork (the path used by apply_operator's environment,
    test_apply_operator.jl:70-74) is exact on a tree."""
    rng = np.random.default_rng(9)
    links = _comb_links(3, 3, 2)
    verts = [(x, y) for x in range(3) for y in range(3)]
    site = {v: N.Index(2) for v in verts}
    tn = _random_tn(links, verts, np.float64, rng, site)
    nn = N.normnetwork(tn)
    env = N.beliefpropagation(nn, N.message_environment("ones", nn),
                              stopping_criterion={"maxiter": 100, "tol": 1e-13})
    z_bp = np.exp(N.bethe_free_energy(nn, env))
    z = N.contract_network(nn)[()]
    assert abs(z_bp - z) <= 1e-10 * abs(z)
    # the GPU parallel schedule reaches the same fixed point
    env2 = N.beliefpropagation(nn, N.message_environment("ones", nn),
                               stopping_criterion={"maxiter": 100, "tol": 1e-13},
                               message_update_algorithm=N.GPUMessageUpdate(schedule="parallel"))
    assert abs(np.exp(N.bethe_free_energy(nn, env2)) - z) <= 1e-10 * abs(z)


def test_message_update_single_edge():
    rng = np.random.default_rng(11)
    links = _grid_links(2, 2, 2)
    verts = [(x, y) for x in range(2) for y in range(2)]
    site = {v: N.Index(2) for v in verts}
    tn = _random_tn(links, verts, np.float64, rng, site)
    nn = N.normnetwork(tn)
    cache = N.message_environment("one", nn)
    e = ((0, 0), (0, 1))
    N.message_update(cache, nn, e)
    m = cache[e]
    assert np.isclose(np.sum(m.data), 1.0)  # normalised by its sum


def test_contract_network_orders():
    """test_contract_network.jl:13-24: Exact with LeftAssociative and Greedy agree."""
    i, j, k = N.Index(2), N.Index(2), N.Index(5)
    A = N.itensor(np.array([[1.0, 1.0], [0.5, 1.0]]), i, j)
    B = N.itensor(np.array([2.0, 1.0]), i)
    C = N.itensor(np.array([5.0, 1.0]), j)
    D = N.itensor(np.array([-2.0, 3.0, 4.0, 5.0, 1.0]), k)
    r1 = N.contract_network([A, B, C, D], alg=N.Exact(order_alg=N.LeftAssociative()))
    r2 = N.contract_network([A, B, C, D], alg=N.Exact(order_alg=N.Greedy()))
    r3 = N.contract_network([A, B, C, D], alg=N.Exact(order_alg=N.Sweep()))
    assert np.array_equal(r1.data, r2.data)
    assert np.allclose(r3.data, r2.data, rtol=1e-14, atol=0)


def test_edge_scalars_of_a_norm_network_cache():
    """edge_scalar(cache, edge) / edge_scalars(cache) (messagecache.jl:153-178): the full
    contraction of the two messages of each edge, one value per undirected edge; the
    messages of the two directions are stored with their names in different orders."""
    rng = np.random.default_rng(21)
    links = _grid_links(2, 3, 3)
    verts = [(x, y) for x in range(2) for y in range(3)]
    site = {v: N.Index(2) for v in verts}
    tn = _random_tn(links, verts, np.complex128, rng, site)
    nn = N.normnetwork(tn)
    cache = N.message_environment("one", nn)
    for e in cache.keys():
        t = cache[e]
        data = rng.standard_normal(t.data.shape) + 1j * rng.standard_normal(t.data.shape)
        if e[0] > e[1]:  # reversed name order on one direction
            cache[e] = N.ITensor(np.transpose(data), list(reversed(t.inds)))
        else:
            cache[e] = N.ITensor(data, t.inds)
    got = N.edge_scalars(cache)
    want = []
    seen = set()
    for e in cache.keys():
        if (e[1], e[0]) in seen:
            continue
        seen.add(e)
        a, b = cache[e], cache[(e[1], e[0])]
        want.append(np.sum(a.data * b.permute(a.dimnames)))
    assert len(got) == len(links) == len(want)
    np.testing.assert_allclose(got, want, rtol=1e-12)
    e0 = next(iter(cache.keys()))
    assert np.isclose(N.edge_scalar(cache, e0), want[0], rtol=1e-12)
