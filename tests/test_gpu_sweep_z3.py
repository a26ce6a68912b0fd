"""The grouped sweep for networks whose vertices all have three legs (random 3-regular
batches with bond dimensions up to 8: the batched uneven workload) against the oracle.

Bounds per message (each in its own scale) after the stated sweeps from the normalised
identity: FP64 / complex128 1e-12, FP32 / complex64 2e-6 (each sweep's contractions are at
most 1024 x 8 terms).  A converged run stops where the convergence test says and matches
the oracle after as many sweeps.
"""
import numpy as np
import pytest

from itn_gb300 import BPEngine
from itn_gb300 import graphs as G
from helpers import msg_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _batch(n_nets, bonds, seed, dtype):
    rng = np.random.default_rng(seed)
    nets = []
    for _ in range(n_nets):
        n = int(rng.integers(2, 20)) * 2
        edges = G.random_regular_edges(n, 3, rng)
        nets.append(G.from_edges(n, edges, rng.choice(bonds, size=len(edges)), phys=2))
    g = G.batched(nets)
    real = np.dtype(dtype).kind != "c"
    t = G.random_tensors(g, rng, np.float64 if real else np.complex128, G.peps_scale(g))
    return g, t


@pytest.mark.parametrize("dtype,tol", [(np.complex64, 2e-6), (np.complex128, 1e-12), (np.float32, 2e-6),
                                       (np.float64, 1e-12)])
@pytest.mark.parametrize("bonds", [(2, 3, 4, 6, 8), (8,), (2,), (5, 7)])
def test_grouped_sweep_matches_oracle(dtype, tol, bonds):
    from oracle import oracle as O
    g, t = _batch(12, bonds, 3 + len(bonds), dtype)
    m0 = G.identity_messages(g, t.dtype)
    ref, it, _, _ = O.bp_run(g, t, m0, maxiter=6)
    with BPEngine(g) as e:
        e.set_tensors(t.astype(dtype))
        e.init_messages()
        r = e.run(maxiter=6)
        m = e.messages().astype(t.dtype)
    assert r.iterations == 6 == it
    err = msg_rel(g, m, ref)
    print(f"{np.dtype(dtype).name} bonds {bonds}: per-message err {err:.2e}")
    assert err <= tol


def test_grouped_sweep_unnormalised_and_random_messages():
    from oracle import oracle as O
    g, t = _batch(7, (2, 3, 4, 6, 8), 9, np.complex128)
    rng = np.random.default_rng(10)
    m0 = G.random_messages(g, rng, np.complex128)
    ref, _, _, _ = O.bp_run(g, t, m0, maxiter=1, normalize=False)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        e.run(maxiter=1, normalize=False)
        assert msg_rel(g, e.messages(), ref) <= 1e-12


def test_grouped_sweep_converged_run():
    from oracle import oracle as O
    g, t = _batch(10, (2, 3, 4, 6, 8), 11, np.complex128)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        r = e.run(maxiter=300, tol=1e-10)
        m = e.messages()
    assert 1 < r.iterations < 300 and r.at_iteration == r.iterations and r.delta < 1e-10
    ref, _, _, _ = O.bp_run(g, t, G.identity_messages(g, np.complex128), maxiter=r.iterations)
    assert msg_rel(g, m, ref) <= 1e-10


def test_contexts_on_one_network_share_the_tuned_shape_bit_for_bit():
    """The grouped sweep's launch shape is autotuned once per network structure and dtype in a
    process; a second context on the same network reuses it, so the two solves agree bit for bit
    (a different shape would change the order of partial sums)."""
    g, t = _batch(40, (2, 3, 4, 6, 8), 77, np.complex64)
    out = []
    for _ in range(2):
        with BPEngine(g) as e:
            e.set_tensors(t.astype(np.complex64))
            e.init_messages()
            r = e.run(maxiter=12)
            out.append((r.iterations, e.messages().copy()))
    assert out[0][0] == out[1][0] == 12
    np.testing.assert_array_equal(out[0][1], out[1][1])
