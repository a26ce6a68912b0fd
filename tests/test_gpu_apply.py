"""BP simple-update gate application on the GPU (itn_apply_gates, apply_operator(s)).

Parity with the oracle (oracle/apply_oracle.py) is checked on gauge-invariant quantities:
the singular values of the new bond and the two new site tensors contracted over it (the
gauge of the new bond -- phases of singular vectors -- is arbitrary in both).  Bounds:
1e-9 relative in FP64 / complex128, 2e-4 in float32 / complex64 (FP64 arithmetic inside,
rounded at the output).  The network-level tests restate test/test_apply_operator.jl:66-145
with its tolerance rtol = eps(real(T))^(1/3): untruncated gates are exact; a truncated gate
on a tree with BP environments equals the optimal SVD truncation; apply_operators applies
a sequence.
"""
import numpy as np
import pytest

from oracle import apply_oracle as AO
from itn_gb300 import network as N
from itn_gb300.apply import Gate, apply_gates
from helpers import rand_psd, _randn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _pair(n1, n2):
    return np.tensordot(n1, n2, axes=([-1], [-1]))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-9), (np.complex128, 1e-9),
                                       (np.float32, 2e-4), (np.complex64, 2e-4)])
@pytest.mark.parametrize("maxrank", [None, 3])
def test_two_site_against_oracle(dtype, tol, maxrank):
    rng = np.random.default_rng(10)
    d, B = 2, 4
    psi1 = _randn(rng, (3, 2, d, B), dtype)     # other legs 3, 2
    psi2 = _randn(rng, (4, d, B), dtype)        # other leg 4
    e1 = [rand_psd(rng, 3, dtype), None]        # second leg without a gauge
    e2 = [rand_psd(rng, 4, dtype)]
    op = _randn(rng, (d, d, d, d), dtype)
    (g1, g2, gs), = apply_gates([Gate([psi1, psi2], [e1, e2], op)], max_rank=maxrank)
    o1, o2, os_ = AO.apply_gate_2site(psi1.astype(np.complex128 if np.dtype(dtype).kind == "c" else np.float64),
                                      psi2.astype(np.complex128 if np.dtype(dtype).kind == "c" else np.float64),
                                      [e1[0], None], e2, op, maxrank=maxrank)
    assert g1.dtype == np.dtype(dtype)
    assert len(gs) == len(os_)
    np.testing.assert_allclose(gs, os_, rtol=tol)
    assert _rel(_pair(g1, g2), _pair(o1, o2)) < tol


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_one_site_against_oracle(dtype):
    rng = np.random.default_rng(11)
    psi = _randn(rng, (3, 4, 2), dtype)
    envs = [rand_psd(rng, 3, dtype), rand_psd(rng, 4, dtype)]
    op = _randn(rng, (2, 2), dtype)
    for normalize in (False, True):
        (got,) = apply_gates([Gate([psi], [envs], op)], normalize=normalize)
        want = AO.apply_gate_1site(psi, envs, op, normalize=normalize)
        assert _rel(got, want) < 1e-10


def test_batch_equals_one_by_one():
    rng = np.random.default_rng(12)
    gates = []
    for k in range(7):
        d = 2 if k % 2 else 3
        psi1 = _randn(rng, (2, d, 3), np.float64)
        psi2 = _randn(rng, (3, 2, d, 3), np.float64)
        gates.append(Gate([psi1, psi2], [[rand_psd(rng, 2, np.float64)], [None, rand_psd(rng, 2, np.float64)]],
                          _randn(rng, (d, d, d, d), np.float64)))
    batch = apply_gates(gates, max_rank=4)
    for g, (b1, b2, bs) in zip(gates, batch):
        (s1, s2, ss), = apply_gates([g], max_rank=4)
        np.testing.assert_array_equal(bs, ss)
        np.testing.assert_array_equal(b1, s1)
        np.testing.assert_array_equal(b2, s2)


# ---- network level: the reference's apply_operator tests --------------------------------------
def _network(rng, dtype, kind, d=3):
    s = [N.Index(d) for _ in range(4)]
    if kind == "cycle":
        links = [N.Index(b) for b in (2, 3, 2, 3)]          # a(3-0) b(0-1) c(1-2) d(2-3)
        inds = [[links[0], links[1], s[0]], [links[1], links[2], s[1]],
                [links[2], links[3], s[2]], [links[3], links[0], s[3]]]
    else:
        links = [N.Index(b) for b in (3, 4, 3)]             # b(0-1) c(1-2) d(2-3)
        inds = [[s[0], links[0]], [links[0], links[1], s[1]], [links[1], links[2], s[2]], [links[2], s[3]]]
    tn = N.ITensorNetwork({v: N.ITensor(_randn(rng, [i.dim for i in inds[v]], dtype), inds[v])
                           for v in range(4)})
    return tn, s


def _dense(tn, s):
    return N.contract_network(tn).permute([i.name for i in s])


def _bp_env(tn):
    nn = N.NormNetwork(tn)
    return N.beliefpropagation(nn, N.message_environment("ones", nn),
                               stopping_criterion=dict(maxiter=100, tol=1e-13))


def _op(rng, dtype, sites):
    cod = [N.Index(i.dim) for i in sites]
    shape = [i.dim for i in cod] + [i.dim for i in sites]
    return N.operator(_randn(rng, shape, dtype), cod, sites)


def _rtol(dtype):
    return np.finfo(np.dtype(dtype)).eps ** (1 / 3)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_untruncated_gates_are_exact(dtype):
    rng = np.random.default_rng(123)
    tn, s = _network(rng, dtype, "cycle")
    env = _bp_env(tn)
    psi = _dense(tn, s)
    g1 = _op(rng, dtype, [s[1]])
    gated, _ = N.apply_operator(g1, tn, env)
    want = np.einsum("ts,asxb->atxb", g1.data, psi)
    assert _rel(_dense(gated, s), want) < _rtol(dtype)
    g2 = _op(rng, dtype, [s[1], s[2]])
    gated, _ = N.apply_operator(g2, tn, env)
    want = np.einsum("xyst,astb->axyb", g2.data, psi)
    assert _rel(_dense(gated, s), want) < _rtol(dtype)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_truncated_gate_matches_optimal_svd(k, dtype):
    rng = np.random.default_rng(123)
    tn, s = _network(rng, dtype, "path")
    env = _bp_env(tn)
    gate = _op(rng, dtype, [s[1], s[2]])
    full = np.einsum("xyst,astb->axyb", gate.data, _dense(tn, s))
    u, sv, vh = np.linalg.svd(full.reshape(9, 9).astype(np.complex128))
    want = ((u[:, :k] * sv[:k]) @ vh[:k]).reshape(full.shape)
    gated, env2 = N.apply_operator(gate, tn, env, trunc=k)
    assert _rel(_dense(gated, s), want) < _rtol(dtype)
    # the new bond's environment is diag(S) in both directions
    m = env2[(1, 2)].data
    assert m.shape == (k, k) and np.allclose(m, np.diag(np.diag(m)))


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_apply_operators_applies_a_sequence(dtype):
    rng = np.random.default_rng(123)
    tn, s = _network(rng, dtype, "cycle")
    env = _bp_env(tn)
    g1 = _op(rng, dtype, [s[1], s[2]])
    g2 = _op(rng, dtype, [s[2], s[3]])
    gated, _ = N.apply_operators([g1, g2], tn, env)
    psi = _dense(tn, s)
    want = np.einsum("xyst,astb->axyb", g1.data, psi)
    want = np.einsum("xyst,abst->abxy", g2.data, want)
    assert _rel(_dense(gated, s), want) < _rtol(dtype)


def test_rejects_bad_descriptors():
    """Host-side validation of itn_apply_gates: arrays out of range -> ITN_ERR_ARG, shapes
    beyond the kernel's limits -> ITN_ERR_UNSUPPORTED; nothing reaches the device."""
    import ctypes
    from itn_gb300 import _lib as L, ItnArgumentError, ItnError
    from itn_gb300.contract import Context
    rng = np.random.default_rng(13)
    big = Gate([_randn(rng, (2, 70), np.float64), _randn(rng, (2, 70), np.float64)], [[], []],
               _randn(rng, (2, 2, 2, 2), np.float64))
    with pytest.raises(ItnError) as ei:
        apply_gates([big])
    assert ei.value.status == L.ITN_ERR_UNSUPPORTED
    with Context() as ctx:
        g = (L.GateDesc * 1)()
        g[0].nsite, g[0].bond = 2, 2
        g[0].d[0] = g[0].d[1] = 2
        g[0].site_off[1] = 100                    # past the 8 site entries
        g[0].out_off[1] = 4
        sites, op = np.zeros(8), np.eye(4)
        out, s, chi = np.zeros(8), np.zeros(2), np.zeros(1, dtype=np.int32)
        st = ctx.lib.itn_apply_gates(ctx.ctx, L.F64, 1, g, L.ptr(sites), 8, None, 0, L.ptr(op), 16, 0, 0.0, 0,
                                     L.ptr(out), 8, L.ptr(s), 2, L.ptr(chi), None)
        assert st == L.ITN_ERR_ARG
        with pytest.raises(ItnArgumentError, match="out of range"):
            L.check(ctx.ctx, st)


# ---- the reference's own flow: random_state built by gate layers, operator environments ---------
def _random_state(rng, dtype, edges, nlayers=2, trunc=4, d=3):
    """random_state (test/test_apply_operator.jl:19-40): a product state, a dimension-1 link
    per edge (insertlink!), then nlayers layers of random two-site gates over the edges,
    each applied with apply_operator and truncation to rank ``trunc`` from identity
    environments."""
    vs = sorted({v for e in edges for v in e})
    s = {v: N.Index(d) for v in vs}
    tn = N.tensornetwork(lambda v: N.ITensor(_randn(rng, (d,), dtype), [s[v]]), vs)
    for e in edges:
        N.insertlink(tn, e)
    env = N.message_environment("one", N.NormNetwork(tn))
    for _ in range(nlayers):
        for (u, v) in edges:
            tn, env = N.apply_operator(_op(rng, dtype, [s[u], s[v]]), tn, env, trunc=trunc)
    return tn, [s[v] for v in vs]


def _operator_env(tn):
    nn = N.NormNetwork(tn)
    env = N.beliefpropagation(nn, N.message_environment("ones", nn),
                              stopping_criterion=dict(maxiter=100, tol=1e-13))
    return N.operator_message_cache(nn, env)


_CYCLE = [(0, 1), (1, 2), (2, 3), (0, 3)]
_PATH = [(0, 1), (1, 2), (2, 3)]


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_reference_flow_untruncated_gates_are_exact(dtype):
    rng = np.random.default_rng(321)
    tn, s = _random_state(rng, dtype, _CYCLE)
    assert all(i.dim <= 4 for v in tn.vertices() for i in tn[v].inds)
    env = _operator_env(tn)
    psi = _dense(tn, s)
    g1 = _op(rng, dtype, [s[1]])
    gated, _ = N.apply_operator(g1, tn, env)
    assert _rel(_dense(gated, s), np.einsum("ts,asxb->atxb", g1.data, psi)) < _rtol(dtype)
    g2 = _op(rng, dtype, [s[1], s[2]])
    gated, _ = N.apply_operator(g2, tn, env)
    assert _rel(_dense(gated, s), np.einsum("xyst,astb->axyb", g2.data, psi)) < _rtol(dtype)


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_reference_flow_truncated_gate_matches_optimal_svd(k, dtype):
    rng = np.random.default_rng(321)
    tn, s = _random_state(rng, dtype, _PATH)
    env = _operator_env(tn)
    gate = _op(rng, dtype, [s[1], s[2]])
    full = np.einsum("xyst,astb->axyb", gate.data, _dense(tn, s))
    u, sv, vh = np.linalg.svd(full.reshape(9, 9).astype(np.complex128))
    want = ((u[:, :k] * sv[:k]) @ vh[:k]).reshape(full.shape)
    gated, _ = N.apply_operator(gate, tn, env, trunc=k)
    assert _rel(_dense(gated, s), want) < _rtol(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex128])
def test_reference_flow_apply_operators_sequence(dtype):
    rng = np.random.default_rng(321)
    tn, s = _random_state(rng, dtype, _CYCLE)
    env = _operator_env(tn)
    g1 = _op(rng, dtype, [s[1], s[2]])
    g2 = _op(rng, dtype, [s[2], s[3]])
    gated, _ = N.apply_operators([g1, g2], tn, env)
    want = np.einsum("xyst,astb->axyb", g1.data, _dense(tn, s))
    want = np.einsum("xyst,abst->abxy", g2.data, want)
    assert _rel(_dense(gated, s), want) < _rtol(dtype)
