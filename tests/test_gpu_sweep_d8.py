"""FP32 sweep kernel for lattices whose vertices all have d = 2 and four legs of dimension 8
(the plain-FP32 CUDA-core path of the 32x32 D=8 workload), against the FP64 oracle.

Bounds: one sweep from non-symmetric messages near the normalised identity within 1e-5 per
message (FP32 rounding of a 1024-term contraction); a converged run stops where the
convergence test says and its messages match the oracle's after as many sweeps within 1e-5.
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


def _case(L, seed):
    g = G.square_lattice(L, L, 8, periodic=True, phys=2)
    rng = np.random.default_rng(seed)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g) + 0.05 * G.random_messages(g, rng)
    return g, t, m0


@pytest.mark.parametrize("L,sweeps,normalize", [(3, 1, True), (4, 1, True), (4, 1, False), (5, 4, True),
                                                (8, 7, True)])
def test_sweeps_match_oracle(L, sweeps, normalize):
    from oracle import oracle as O
    g, t, m0 = _case(L, 40 + L)
    ref, it, _, _ = O.bp_run(g, t, m0, maxiter=sweeps, normalize=normalize)
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.set_messages(m0.astype(np.float32))
        r = e.run(maxiter=sweeps, normalize=normalize)
        m = e.messages().astype(np.float64)
    assert r.iterations == sweeps == it
    err = msg_rel(g, m, ref)
    print(f"{L}x{L} D=8 fp32, {sweeps} sweeps, normalize={normalize}: per-message err {err:.2e}")
    assert err < 1e-5


def test_converged_run_matches_oracle():
    from oracle import oracle as O
    g, t, _ = _case(6, 7)
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.init_messages()
        r = e.run(maxiter=200, tol=1e-6)
        m = e.messages().astype(np.float64)
    assert 1 < r.iterations < 200 and r.at_iteration == r.iterations and r.delta < 1e-6
    ref, it, _, _ = O.bp_run(g, t, G.identity_messages(g), maxiter=r.iterations)
    assert msg_rel(g, m, ref) < 1e-5
