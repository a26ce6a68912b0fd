"""GPU parity of the CUDA-core BP path against the CPU oracle (C ABI, libitn_gpu.so).

Tolerances: FP64 results agree with the FP64 oracle within 1e-10 relative (messages,
per-vertex and per-edge log-scalars, total log-norm); FP32 / complex64 results within
2e-4 relative of the FP64 oracle, measured per message.
"""
import numpy as np
import pytest

from oracle import oracle as O
from itn_gb300 import BPEngine, ItnArgumentError, ItnError
from itn_gb300 import generators as GEN
from itn_gb300 import graphs as G
from helpers import load_golden, max_rel, msg_rel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 2e-4


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _engine(g, t, m0):
    e = BPEngine(g)
    e.set_tensors(t)
    e.set_messages(m0)
    return e


def _check_scalars(g, t, m, e, tol):
    ref = O.logscalars(g, t.astype(np.complex128 if np.iscomplexobj(t) else np.float64),
                       m.astype(np.complex128 if np.iscomplexobj(t) else np.float64))
    got = e.logscalars()
    assert np.max(np.abs(got["logzv"] - ref["logzv"])) < tol * max(1.0, np.max(np.abs(ref["logzv"])))
    assert np.max(np.abs(got["logze"] - ref["logze"])) < tol * max(1.0, np.max(np.abs(ref["logze"])))
    assert abs(got["totals"][0][0] - ref["total"][0]) <= tol * max(1.0, abs(ref["total"][0]))
    assert abs(got["totals"][0][1] - ref["total"][1]) <= tol * max(1.0, abs(ref["total"][1]))


def test_golden_peps4x4_parallel_fp64():
    g, d = load_golden("peps4x4_d2_D2_parallel20.npz")
    with _engine(g, d["tensors"], d["messages0"]) as e:
        r = e.run(maxiter=20)
        assert r.iterations == 20
        m = e.messages()
        assert msg_rel(g, m, d["messages"]) < FP64_TOL
        got = e.logscalars()
        assert np.max(np.abs(got["logzv"] - d["logzv"])) < FP64_TOL
        assert abs(got["totals"][0][0] - d["total"][0]) < FP64_TOL * abs(d["total"][0])


def test_golden_peps4x4_sequential_fp64():
    g, d = load_golden("peps4x4_d2_D2_sequential5.npz")
    with _engine(g, d["tensors"], d["messages0"]) as e:
        r = e.run(schedule="sequential", edges=d["edges"], maxiter=5)
        assert r.iterations == 5
        assert msg_rel(g, e.messages(), d["messages"]) < FP64_TOL


def test_golden_complex128():
    g, d = load_golden("peps3x3_c128_D3_parallel15.npz")
    with _engine(g, d["tensors"], d["messages0"]) as e:
        e.run(maxiter=15)
        assert msg_rel(g, e.messages(), d["messages"]) < FP64_TOL
        got = e.logscalars()
        assert np.max(np.abs(got["logzv"] - d["logzv"])) < FP64_TOL * 10


def test_golden_spin_ice_single_layer():
    g, d = load_golden("spinice3_sequential.npz")
    with _engine(g, d["tensors"], d["messages0"]) as e:
        r = e.run(schedule="sequential", edges=d["edges"], maxiter=10, tol=1e-10)
        assert r.iterations == int(d["iterations"])
        assert msg_rel(g, e.messages(), d["messages"]) < 1e-9
        z = np.exp(e.bethe_free_energy())
        assert abs(z / 1.5 ** 9 - 1) < 1e-6


@pytest.mark.parametrize("dtype,tol", [(np.float64, FP64_TOL), (np.float32, FP32_TOL),
                                       (np.complex128, FP64_TOL), (np.complex64, FP32_TOL)])
def test_peps16x16_D4_parallel(dtype, tol):
    """16x16 open lattice, d=2, D=4, N(0,1)/sqrt(d D^4); 50 iterations or tol 1e-10."""
    rng = np.random.default_rng(16)
    g = G.square_lattice(16, 16, 4, periodic=False, phys=2)
    t = G.random_tensors(g, rng, dtype, G.peps_scale(g))
    m0 = G.identity_messages(g, dtype)
    wide = np.complex128 if np.iscomplexobj(t) else np.float64
    ref, it, delta, at = O.bp_run(g, t.astype(wide), m0.astype(wide), maxiter=50, tol=1e-10)
    with _engine(g, t, m0) as e:
        r = e.run(maxiter=50, tol=1e-10)
        if dtype in (np.float64, np.complex128):
            assert r.iterations == it and r.at_iteration == at
            assert abs(r.delta - delta) < 1e-9
        m = e.messages()
        assert msg_rel(g, m, ref) < tol
        _check_scalars(g, t.astype(wide), ref, e, tol)


def test_sequential_matches_oracle_random_order():
    rng = np.random.default_rng(99)
    g = G.square_lattice(5, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g)
    edges = rng.permutation(g.nslots)
    edges = np.concatenate([edges, edges[:7]])  # repeated slots are allowed
    ref, *_ = O.bp_run(g, t, m0, schedule="sequential", edges=edges, maxiter=3, tol=1e-14)
    with _engine(g, t, m0) as e:
        e.run(schedule="sequential", edges=edges, maxiter=3, tol=1e-14)
        assert msg_rel(g, e.messages(), ref) < FP64_TOL


def test_single_message_update():
    rng = np.random.default_rng(4)
    g = G.square_lattice(3, 3, 2, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64)
    m0 = G.random_messages(g, rng)
    with _engine(g, t, m0) as e:
        for s in (0, 5, g.nslots - 1):
            ref = O.message_update(g, t, e.messages(), s)
            e.message_update(s)
            assert msg_rel(g, e.messages(), ref) < FP64_TOL
        ref = O.message_update(g, t, e.messages(), 3, normalize=False)
        e.message_update(3, normalize=False)
        assert msg_rel(g, e.messages(), ref) < FP64_TOL


def test_iterate_diff_device():
    rng = np.random.default_rng(2)
    g = G.square_lattice(4, 3, 3, phys=2)
    a = G.random_messages(g, rng)
    b = G.random_messages(g, rng)
    with BPEngine(g) as e:
        e.set_tensors(G.random_tensors(g, rng))
        assert abs(e.iterate_diff(a, b) - O.iterate_diff(g.moff, a, b)) < 1e-13
        assert abs(e.iterate_diff(a, a)) <= 10 * np.finfo(float).eps


@pytest.mark.parametrize("n", [3, 4])
def test_spin_ice_gpu(n):
    rng = np.random.default_rng(123)
    g = G.square_lattice(n, n, 2, periodic=True, phys=1, layers=1)
    t = GEN.spin_ice_tensors(g)
    m0 = G.random_messages(g, rng)
    with _engine(g, t, m0) as e:
        e.run(schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=10, tol=1e-10)
        z = np.exp(e.bethe_free_energy())
        assert abs(z / 1.5 ** (n * n) - 1) < 1e-6


def test_tree_exact_norm_network_gpu():
    from oracle import contract_oracle as C
    rng = np.random.default_rng(8)
    g = G.from_edges(12, G.comb_tree_edges(4, 3), 3, phys=2, layers=2)
    t = G.random_tensors(g, rng, np.complex128)
    with _engine(g, t, G.identity_messages(g, np.complex128)) as e:
        e.run(schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=1)
        z = np.exp(e.bethe_free_energy())
        zx = C.contract_norm(g, t)
        assert abs(z - zx) < 1e-10 * abs(zx)


def test_batched_uneven_networks():
    """Several independent 3-regular networks with per-edge bond dims from {2,3,4,6,8},
    complex64, in one launch; per-network log-norms against the oracle."""
    rng = np.random.default_rng(256)
    nets = []
    for n in (16, 20, 24):
        edges = G.random_regular_edges(n, 3, rng)
        bonds = rng.choice([2, 3, 4, 6, 8], size=len(edges))
        nets.append(G.from_edges(n, edges, bonds, phys=2))
    g = G.batched(nets)
    t = G.random_tensors(g, rng, np.complex64, G.peps_scale(g))
    m0 = G.identity_messages(g, np.complex64)
    with _engine(g, t, m0) as e:
        e.run(maxiter=30)
        got = e.logscalars()
        m = e.messages()
    for k, gk in enumerate(nets):
        sl = slice(int(np.searchsorted(g.net, k)), int(np.searchsorted(g.net, k, side="right")))
        v0 = sl.start
        tk = t[g.toff[v0]:g.toff[sl.stop]].astype(np.complex128)
        ref, *_ = O.bp_run(gk, tk, G.identity_messages(gk, np.complex128), maxiter=30)
        s0 = int(g.off[v0])
        mk = m[g.moff[s0]:g.moff[int(g.off[sl.stop])]]
        assert msg_rel(gk, mk, ref) < FP32_TOL
        rr = O.logscalars(gk, tk, ref)
        assert abs(got["totals"][k][0] - rr["total"][0]) < FP32_TOL * max(1, abs(rr["total"][0]))


def test_message_init_kinds():
    g = G.square_lattice(3, 3, 3, phys=2)
    with BPEngine(g) as e:
        e.set_tensors(np.ones(int(g.toff[-1])))
        e.init_messages("identity_normalized")
        assert np.array_equal(e.messages(), G.identity_messages(g))
        e.init_messages("identity")
        assert np.array_equal(e.messages(), G.identity_messages(g, normalized=False))
        e.init_messages("ones")
        assert np.array_equal(e.messages(), G.ones_messages(g))


def test_strided_upload_matches_packed():
    """Column-major tensors with a permuted index order (as a Julia array of an ITensor
    would arrive) permuted on the device into the canonical layout."""
    rng = np.random.default_rng(31)
    g = G.square_lattice(3, 4, 3, phys=2)
    t = G.random_tensors(g, rng)
    arrays, strides = [], []
    for u in range(g.nv):
        A = t[g.toff[u]:g.toff[u + 1]].reshape(g.tensor_shape(u))
        perm = rng.permutation(A.ndim)
        B = np.asfortranarray(np.transpose(A, perm))  # source axes = perm of canonical
        flat = B.ravel(order="K")
        # element stride of canonical axis a inside B
        st_by_src = [s // B.itemsize for s in B.strides]
        inv = np.argsort(perm)
        strides.extend(int(st_by_src[inv[a]]) for a in range(A.ndim))
        arrays.append(flat)
    with BPEngine(g) as e:
        e.set_tensors_strided(arrays, strides, np.float64)
        assert np.array_equal(e.tensors(), t)


def test_argument_errors():
    g = G.square_lattice(3, 3, 2, phys=2)
    with BPEngine(g) as e:
        with pytest.raises(ItnError):
            e.run(maxiter=1)  # no tensors yet
        e.set_tensors(np.ones(int(g.toff[-1])))
        e.init_messages()
        with pytest.raises(ItnArgumentError):
            e.run()  # neither maxiter nor tol
        with pytest.raises(ItnArgumentError):
            e.run(schedule="sequential", edges=[0, 10 ** 6], maxiter=1)
        with pytest.raises(ItnArgumentError):
            e.message_update(10 ** 6)
    bad = G.Graph(2, [0, 1, 2], [1, 0], [2, 3], [1, 0], [2, 2])
    with pytest.raises(ItnArgumentError):
        BPEngine(bad)


def test_zero_sum_message_is_not_normalised():
    """A message whose entries sum to zero is stored unnormalised
    (beliefpropagation.jl:248-253): with A = [[1, -1], [2, -2]] on a one-leg vertex the
    outgoing message A^T A = [[5, -5], [-5, 5]] sums to zero."""
    g = G.from_edges(2, [(0, 1)], 2, phys=2)
    A = np.array([[1.0, -1.0], [2.0, -2.0]])
    B = np.array([[1.0, 0.0], [0.0, 1.0]])
    t = np.concatenate([A.ravel(), B.ravel()])
    m0 = G.identity_messages(g)
    with _engine(g, t, m0) as e:
        e.message_update(0)
        m = e.messages()
        assert np.array_equal(m[:4], [5.0, -5.0, -5.0, 5.0])
        ref = O.message_update(g, t, m0.copy(), 0)
        assert np.array_equal(m, ref)


@pytest.mark.parametrize("dtype,tol", [(np.float32, 1e-5), (np.complex64, 1e-5), (np.float64, 1e-12)])
def test_vertex_scalars_of_d8_norm_vertices(dtype, tol):
    """Vertex and edge log-scalars on a 4x4 periodic D=8 d=2 norm network (every vertex has
    four legs of dimension 8: float32 / complex64 take the register-resident vertex-scalar
    kernel, float64 the interpreter) against the FP64 oracle, with random Hermitian PSD
    messages (no normalisation, so the scalars also carry the messages' scale)."""
    rng = np.random.default_rng(88)
    g = G.square_lattice(4, 4, 8, periodic=True, phys=2)
    t = G.random_tensors(g, rng, dtype, G.peps_scale(g))
    m = np.zeros(int(g.moff[-1]), dtype=dtype)
    cplx = np.iscomplexobj(m)
    for s in range(g.nslots):
        x = rng.standard_normal((8, 8)) + (1j * rng.standard_normal((8, 8)) if cplx else 0)
        m[g.moff[s]:g.moff[s + 1]] = (x @ np.conj(x).T / 8 + 0.5 * np.eye(8)).ravel()
    with _engine(g, t, m) as e:
        _check_scalars(g, t, m, e, tol)


@pytest.mark.parametrize("case", ["tc_mixed", "fp64_tol", "sequential", "fp32_no_logz"])
def test_one_call_solve_matches_separate_calls(case):
    """itn_bp_solve (upload, solve, log-norm, download with one host synchronisation) gives
    exactly what the separate calls give: same messages bit for bit, same iteration count and
    log-norm -- for a deferred-synchronisation run (no tolerance, tensor cores), a run with a
    tolerance, the sequential schedule, and without the log-norm."""
    rng = np.random.default_rng(31)
    kw, logz = {}, True
    if case == "tc_mixed":
        g = G.square_lattice(4, 4, 8, periodic=True, phys=2)
        t = G.random_tensors(g, rng, np.float32, G.peps_scale(g))
        m0 = G.identity_messages(g, np.float32)
        kw = dict(maxiter=6, precision="bf16", split_sweeps=2)
    elif case == "fp64_tol":
        g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
        t = G.random_tensors(g, rng, np.float64)
        m0 = G.identity_messages(g)
        kw = dict(maxiter=100, tol=1e-12)
    elif case == "sequential":
        g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
        t = G.random_tensors(g, rng, np.float64)
        m0 = G.identity_messages(g)
        kw = dict(schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=3)
    else:
        g = G.square_lattice(6, 6, 3, periodic=True, phys=2)
        t = G.random_tensors(g, rng, np.float32, G.peps_scale(g))
        m0 = G.identity_messages(g, np.float32)
        kw = dict(maxiter=9)
        logz = False
    with _engine(g, t, m0) as e:
        r1 = e.run(**kw)
        want_m = e.messages()
        want_z = e.bethe_free_energy()
    with BPEngine(g) as e:
        r2, z, m = e.solve(t, m0, logz=logz, **kw)
        assert r2.iterations == r1.iterations and r2.at_iteration == r1.at_iteration
        np.testing.assert_array_equal(m, want_m)
        if logz:
            assert z == want_z
        else:
            assert z is None
        # the context keeps the data, as after the separate calls
        np.testing.assert_array_equal(e.messages(), want_m)


@pytest.mark.parametrize("case", ["tc_mixed", "fp64_tol"])
def test_submitted_solves_on_two_contexts_match_one_call_solves(case):
    """Networks solved back to back on two contexts with itn_bp_solve_submit / _wait (the next
    network's uploads queued while the previous solve runs) give exactly what itn_bp_solve gives
    for each: same messages bit for bit, iteration counts and log-norms -- for a deferred run on
    the tensor cores and for a run with a tolerance (which completes inside the submit)."""
    if case == "tc_mixed":
        g = G.square_lattice(4, 4, 8, periodic=True, phys=2)
        dt, scale, kw = np.float32, G.peps_scale(g), dict(maxiter=6, precision="bf16", split_sweeps=2)
    else:
        g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
        dt, scale, kw = np.float64, 1.0, dict(maxiter=100, tol=1e-12)
    m0 = G.identity_messages(g, dt)
    nets = [G.random_tensors(g, np.random.default_rng(40 + k), dt, scale) for k in range(5)]
    want = []
    with BPEngine(g) as e:
        for t in nets:
            r, z, m = e.solve(t, m0, **kw)
            want.append((r.iterations, r.at_iteration, z, m.copy()))
    got = []
    with BPEngine(g) as e0, BPEngine(g) as e1:
        eng = [e0, e1]
        for k, t in enumerate(nets):
            eng[k % 2].solve_submit(t, m0, **kw)
            if k >= 1:
                got.append(eng[(k - 1) % 2].solve_wait())
        got.append(eng[(len(nets) - 1) % 2].solve_wait())
    for (it, at, z, m), (r, z2, m2) in zip(want, got):
        assert r.iterations == it and r.at_iteration == at
        assert z2 == z
        np.testing.assert_array_equal(m2, m)


def test_submitted_solve_blocks_other_calls_until_waited():
    """Between itn_bp_solve_submit and itn_bp_solve_wait every other call on the context is
    refused with ITN_ERR_STATE (the solve owns the stream's staging), a second wait is refused,
    and the context works normally after the wait."""
    from itn_gb300 import ItnError
    from itn_gb300 import _lib as L
    g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
    t = G.random_tensors(g, np.random.default_rng(7), np.float64)
    m0 = G.identity_messages(g)
    with BPEngine(g) as e:
        e.solve_submit(t, m0, maxiter=5)
        with pytest.raises(ItnError) as ei:
            e.run(maxiter=1)
        assert ei.value.status == L.ITN_ERR_STATE
        with pytest.raises(ItnError) as ei:
            e.set_tensors(t)
        assert ei.value.status == L.ITN_ERR_STATE
        r, z, m = e.solve_wait()
        assert r.iterations == 5
        with pytest.raises(RuntimeError):
            e.solve_wait()
        r2, z2, m2 = e.solve(t, m0, maxiter=5)
        np.testing.assert_array_equal(m2, m)
        assert z2 == z


def test_batched_size_classes_match_oracle():
    """A batch large enough (more than 16 items per SM) for the parallel sweep to launch its
    small vertices (at most 256 tensor entries) as a second class of one-warp CTAs: the
    messages of every network still match the oracle, in FP64 to 1e-10 and complex64 to
    the FP32 bound."""
    rng = np.random.default_rng(257)
    nets = []
    for k in range(96):
        n = 40 + 2 * (k % 13)
        edges = G.random_regular_edges(n, 3, rng)
        bonds = rng.choice([2, 3, 4, 6, 8], size=len(edges))
        nets.append(G.from_edges(n, edges, bonds, phys=2))
    g = G.batched(nets)
    sizes = np.diff(g.toff)
    assert g.nv >= 16 * 152 and (sizes <= 256).any() and (sizes > 256).any()
    for dtype, tol in ((np.float64, FP64_TOL), (np.complex64, FP32_TOL)):
        t = G.random_tensors(g, rng, dtype, G.peps_scale(g))
        m0 = G.identity_messages(g, dtype)
        with _engine(g, t, m0) as e:
            e.run(maxiter=8)
            m = e.messages()
        wide = np.complex128 if np.iscomplexobj(t) else np.float64
        ref, *_ = O.bp_run(g, t.astype(wide), m0.astype(wide), maxiter=8)
        assert msg_rel(g, m, ref) < tol


@pytest.mark.parametrize("dtype,L_,D", [(np.float32, 16, 4), (np.float64, 12, 6), (np.complex128, 6, 3)])
def test_persistent_sweeps_equal_per_sweep_launches(dtype, L_, D):
    """Small two-layer networks sweep in one persistent cooperative launch (site tensors staged
    once, a grid barrier and the outer-loop step between sweeps); the per-sweep launches run
    the same arithmetic: same iterations, at_iteration, delta and messages, bit for bit, with a
    tolerance (stopping inside a launch) and without one."""
    rng = np.random.default_rng(44)
    g = G.square_lattice(L_, L_, D, periodic=False, phys=2)
    t = G.random_tensors(g, rng, dtype, G.peps_scale(g))
    out = {}
    with BPEngine(g) as e:
        e.set_tensors(t)
        for mode in (0, 1):
            e.inject_fault("no_persistent_sweeps", mode)
            e.init_messages()
            r1 = e.run(maxiter=60, tol=1e-10)
            m1 = e.messages().copy()
            e.init_messages()
            r2 = e.run(maxiter=7)
            m2 = e.messages().copy()
            out[mode] = (r1, m1, r2, m2)
        e.inject_fault("no_persistent_sweeps", 0)
    (a1, am1, a2, am2), (b1, bm1, b2, bm2) = out[0], out[1]
    print(f"{L_}x{L_} D={D}: persistent {a1.device_ms:.3f} ms / per-sweep {b1.device_ms:.3f} ms "
          f"({a1.iterations} sweeps to 1e-10)")
    # the persistent form ran: one sweep launch (plus its barrier set-up) instead of one per sweep
    assert a1.kernel_launches < b1.kernel_launches
    assert (a1.iterations, a1.at_iteration, a1.delta) == (b1.iterations, b1.at_iteration, b1.delta)
    assert 1 < a1.iterations < 60 and a1.at_iteration == a1.iterations
    assert a2.iterations == b2.iterations == 7
    np.testing.assert_array_equal(am1, bm1)
    np.testing.assert_array_equal(am2, bm2)
