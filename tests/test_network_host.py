"""Host logic of the named-tensor API mirror (no GPU): flattening of ITensorNetwork /
NormNetwork onto the C-ABI layout and back, message environments, and the reference's
argument errors (beliefpropagation.jl:16-55, contract_network.jl:12-14)."""
import numpy as np
import pytest

from itn_gb300 import ItnArgumentError
from itn_gb300 import network as N


def _triangle(rng, site=True):
    i, j, k = N.Index(2), N.Index(3), N.Index(2)
    s = [N.Index(2) for _ in range(3)]
    A = N.itensor(rng.standard_normal((2, 2, 3) if site else (2, 3)), *(([s[0]] if site else []) + [i, j]))
    B = N.itensor(rng.standard_normal((3, 2, 2) if site else (3, 2)), *([j] + ([s[1]] if site else []) + [k]))
    C = N.itensor(rng.standard_normal((2, 2, 2) if site else (2, 2)), *([k, i] + ([s[2]] if site else [])))
    return N.ITensorNetwork({"a": A, "b": B, "c": C})


def test_network_structure():
    tn = _triangle(np.random.default_rng(0))
    assert sorted(tn.edges()) == [("a", "b"), ("a", "c"), ("b", "c")]
    assert len(tn.sitenames("a")) == 1
    nn = N.normnetwork(tn)
    # link names are renamed in the bra layer, site names map to themselves
    for n, vs in tn.dimname_vertices.items():
        assert (nn.bra(n) != n) == (len(vs) == 2)


def test_flatten_roundtrip():
    tn = _triangle(np.random.default_rng(1))
    nn = N.normnetwork(tn)
    env = N.message_environment("one", nn)
    f = N._Flat(nn)
    assert f.g.layers == 2 and list(f.g.phys) == [2, 2, 2]
    back = f.unpack_messages(f.pack_messages(env, nn), env, nn)
    for e in env.edges():
        assert np.array_equal(back[e].data, env[e].data)
    # canonical tensor of vertex "b": [site, legs in CSR order]
    k = f.vidx["b"]
    legs = [f.vs[int(f.g.nbr[s])] for s in range(f.g.off[k], f.g.off[k + 1])]
    order = tn.sitenames("b") + sum((tn.linknames("b", w) for w in legs), [])
    ref = tn["b"].permute(order).ravel()
    assert np.array_equal(f.tensors[f.g.toff[k]:f.g.toff[k + 1]], ref)


def test_message_environment_shapes():
    tn = _triangle(np.random.default_rng(2))
    nn = N.normnetwork(tn)
    env = N.message_environment("one", nn)
    assert len(env) == 6
    m = env[("a", "b")]
    ket = tn.linknames("a", "b")
    assert m.dimnames == tuple(nn.bra(n) for n in ket) + tuple(ket)
    assert np.array_equal(m.data.reshape(3, 3), np.eye(3))


def test_stopping_criterion_errors():
    tn = _triangle(np.random.default_rng(3), site=False)
    msgs = N.messagecache(lambda e: N.itensor(np.ones(2), N.Index(2)), [])
    with pytest.raises(ItnArgumentError, match="must be specified"):
        N.beliefpropagation(tn, msgs)
    with pytest.raises(ItnArgumentError, match="At least one"):
        N.beliefpropagation(tn, msgs, stopping_criterion={})
    with pytest.raises(ItnArgumentError, match="Unrecognized"):
        N.beliefpropagation(tn, msgs, stopping_criterion={"maxiter": 2, "foo": 1})
    assert N.select_beliefpropagation_stopping_criterion(
        N.StopWhenAny(N.StopAfterIteration(3), N.StopWhenConverged(1e-9))) == (3, 1e-9)


def test_contract_network_unknown_algorithm():
    with pytest.raises(ItnArgumentError, match="not implemented"):
        N.contract_network([], alg="optimal")


def test_incoming_messages_exclude_reverse():
    cache = N.messagecache(lambda e: e, [(1, 2), (2, 1), (2, 3), (3, 2)])
    assert N.incoming_messages(cache, (2, 3)) == [(1, 2)]
    assert N.incoming_messages(cache, (1, 2)) == []
    assert N.incoming_messages(cache, (2, 1)) == [(3, 2)]


def test_apply_operator_argument_errors():
    """apply_gate_bp! errors (src/apply/apply_operators.jl:214-227): an operator that shares
    no index with the network, and one acting on more than two sites."""
    from itn_gb300 import network as N
    s = [N.Index(2) for _ in range(3)]
    l01, l12 = N.Index(2), N.Index(2)
    tn = N.ITensorNetwork({0: N.ITensor(np.ones((2, 2)), [s[0], l01]),
                           1: N.ITensor(np.ones((2, 2, 2)), [l01, s[1], l12]),
                           2: N.ITensor(np.ones((2, 2)), [l12, s[2]])})
    other = N.Index(2)
    op = N.operator(np.eye(2), [N.Index(2)], [other])
    with pytest.raises(N.ItnArgumentError, match="shares no indices"):
        N.apply_operator(op, tn, None)
    op3 = N.operator(np.ones((2,) * 6), [N.Index(2) for _ in range(3)], s)
    with pytest.raises(N.ItnArgumentError, match="3-site gate decomposition not implemented"):
        N.apply_operator(op3, tn, None)


def test_insertlink_and_operator_environments():
    """insertlink! (abstracttensornetwork.jl:121-133) adds a dimension-1 link and so an edge;
    operator_message_cache (test/test_apply_operator.jl:42-53) turns messages into
    operators (codomain = bra link names, domain = ket link names) that apply_operator
    reads as the same D x D environment matrices as the messages themselves."""
    rng = np.random.default_rng(5)
    s = [N.Index(2) for _ in range(3)]
    tn = N.tensornetwork(lambda v: N.ITensor(rng.standard_normal(2), [s[v]]), range(3))
    assert tn.edges() == []
    N.insertlink(tn, (0, 1))
    N.insertlink(tn, (1, 2))
    assert sorted(tn.edges()) == [(0, 1), (1, 2)]
    assert [i.dim for i in tn[1].inds] == [2, 1, 1]
    np.testing.assert_array_equal(tn[1].data.ravel(), tn[1].data[:, 0, 0])
    # a network with a two-name bond: the conversion must keep the names paired
    a, b, c = N.Index(2), N.Index(3), N.Index(2)
    tn2 = N.ITensorNetwork({0: N.ITensor(rng.standard_normal((2, 3, 2)), [a, b, s[0]]),
                            1: N.ITensor(rng.standard_normal((3, 2, 2, 2)), [b, a, c, s[1]]),
                            2: N.ITensor(rng.standard_normal((2, 2)), [c, s[2]])})
    nn = N.NormNetwork(tn2)
    msgs = N.message_environment(lambda m: rng.standard_normal(m.shape), nn)
    ops = N.operator_message_cache(nn, msgs)
    assert set(ops.keys()) == set(msgs.keys())
    for e in msgs.keys():
        names = nn.ket.linknames(*e)
        op = ops[e]
        assert isinstance(op, N.Operator)
        assert op.domain == tuple(names) and op.codomain == tuple(nn.bra(n) for n in names)
        for order in (names, names[::-1]):
            np.testing.assert_array_equal(N._env_matrix(ops, e, order), N._env_matrix(msgs, e, order))


def test_message_cache_basics():
    """test_beliefpropagation.jl:40-81: a cache of arbitrary values keyed by directed
    edge; setting a message, copyto! from pairs / a dict, and copyto! of selected edges."""
    edges = [((1, 1), (1, 2)), ((1, 2), (2, 2)), ((2, 2), (2, 3))]
    alle = edges + [(b, a) for a, b in edges]
    bpc = N.messagecache(lambda e: f"{e[0]} => {e[1]}", alle)
    assert len(bpc) == 2 * len(edges)
    assert bpc[((1, 1), (1, 2))] == "(1, 1) => (1, 2)"
    bpc[((1, 1), (1, 2))] = "new message"
    assert bpc[((1, 1), (1, 2))] == "new message"
    pairs = [(((1, 2), (2, 2)), "m1"), (((2, 2), (2, 3)), "m2")]
    for src in (pairs, dict(pairs)):
        new = bpc.copy().copyto(src)
        assert new[((1, 1), (1, 2))] == "new message"
        assert new[((1, 2), (2, 2))] == "m1" and new[((2, 2), (2, 3))] == "m2"
        assert bpc[((1, 2), (2, 2))] == "(1, 2) => (2, 2)"  # the source cache is unchanged
    dst = N.messagecache(lambda e: "", alle)
    dst.copyto(bpc, [((1, 2), (2, 2)), ((2, 2), (2, 3))])
    assert dst[((1, 1), (1, 2))] == ""
    assert dst[((1, 2), (2, 2))] == "(1, 2) => (2, 2)"
    assert dst[((2, 2), (2, 3))] == "(2, 2) => (2, 3)"


def test_ket_and_bra_views():
    """test_normnetwork.jl:106-134: the views share the graph, the ket view exposes the ket
    tensors themselves and the bra view the bra tensors; both are read-only."""
    rng = np.random.default_rng(4)
    links = {(0, 1): N.Index(2), (1, 2): N.Index(3)}
    site = {v: N.Index(2) for v in range(3)}
    ts = {}
    for v in range(3):
        inds = [site[v]] + [i for (a, b), i in links.items() if v in (a, b)]
        shape = tuple(i.dim for i in inds)
        ts[v] = N.ITensor(rng.standard_normal(shape) + 1j * rng.standard_normal(shape), inds)
    tn = N.ITensorNetwork(ts)
    nn = N.NormNetwork(tn)
    kv, bv = N.KetView(nn), N.BraView(nn)
    assert set(kv.vertices()) == set(bv.vertices()) == set(tn.vertices())
    assert set(kv.edges()) == set(bv.edges()) == set(tn.edges())
    for v in tn.vertices():
        assert kv[v] is nn.kettensor(v)
        assert bv[v].inds == nn.bratensor(v).inds
        np.testing.assert_array_equal(bv[v].data, np.conj(tn[v].data))
    assert kv.is_vertex_assigned(1) and bv.is_vertex_assigned(1)
    assert not kv.issettable() and not kv.isinsertable() and not bv.issettable() and not bv.isinsertable()
    assert bv.linknames(0, 1) == [nn.bra(n) for n in kv.linknames(0, 1)]
    with pytest.raises(TypeError):
        kv[0] = tn[0]
