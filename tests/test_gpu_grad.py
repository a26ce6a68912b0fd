"""Gradient of the converged BP log-norm w.r.t. every site tensor (itn_bp_grad).

The reference has no gradient, so the check is central finite differences (step 1e-4,
FP64) of the converged Bethe log-norm, evaluated by FP64 GPU solves whose parity with
the oracle is covered by test_gpu_bp.py, and by the FP64 CPU oracle itself.  Bounds: FP64
gradient within 1e-6 relative of FD per direction; the 12x12 D=6 FP32 gradient (FP64
log-scalars) within 1e-5.  The unrolled gradient (through a fixed number of sweeps, with
per-sweep checkpointing) is checked against central differences of the oracle's unrolled
log-norm.
"""
import numpy as np
import pytest

from itn_gb300 import BPEngine
from itn_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _logz(g, t, tol=1e-14, maxiter=2000):
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=maxiter, tol=tol)
        return e.bethe_free_energy()


def _numpy_direct(g, t, m):
    """(T_u(m) + T_u(m^T)) / Z_u with T_u = A_u absorbed with all incoming messages."""
    grad = np.zeros_like(t)
    for u in range(g.nv):
        A = t[g.toff[u]:g.toff[u + 1]].reshape(g.tensor_shape(u))
        for tr in (0, 1):
            T = A.copy()
            for l in range(g.degree(u)):
                s = g.off[u] + l
                mm = m[g.moff[g.rev[s]]:g.moff[g.rev[s] + 1]].reshape(g.bond[s], g.bond[s])
                T = np.moveaxis(np.tensordot(T, mm.T if tr else mm, axes=([1 + l], [1])), -1, 1 + l)
            grad[g.toff[u]:g.toff[u + 1]] += (T / np.sum(T * A)).ravel()
    return grad


def test_direct_term_matches_numpy():
    rng = np.random.default_rng(1)
    g = G.square_lattice(3, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g) + 0.01 * G.random_messages(g, rng)  # non-symmetric
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        e.run(maxiter=3)
        m = e.messages()
        grad, info = e.grad(adjoint=False)
    ref = _numpy_direct(g, t, m)
    assert np.max(np.abs(grad - ref)) < 1e-12 * np.max(np.abs(ref))


def test_fp64_gradient_against_finite_differences():
    rng = np.random.default_rng(2)
    g = G.square_lattice(4, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=2000, tol=1e-14)
        grad, info = e.grad(adjoint=True, tol=1e-12)
    h = 1e-4
    for _ in range(6):
        d = rng.standard_normal(t.size)
        d /= np.linalg.norm(d)
        fd = (_logz(g, t + h * d) - _logz(g, t - h * d)) / (2 * h)
        assert abs(grad @ d - fd) <= 1e-6 * abs(fd), (grad @ d, fd)


@pytest.mark.parametrize("normalized", [True, False])
def test_sweep_vjp_against_finite_differences(normalized):
    """<lam, J v> from central differences of one sweep equals <J^T lam, v>."""
    rng = np.random.default_rng(3)
    g = G.square_lattice(3, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g) + 0.05 * G.random_messages(g, rng)
    lam = rng.standard_normal(m0.size)
    v = rng.standard_normal(m0.size)
    h = 1e-6
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        jt = e.sweep_vjp(lam, normalized=normalized)
        outs = []
        for sgn in (1, -1):
            e.set_messages(m0 + sgn * h * v)
            e.run(maxiter=1, normalize=normalized)
            outs.append(e.messages())
    jv = (outs[0] - outs[1]) / (2 * h)
    assert abs(lam @ jv - jt @ v) <= 1e-7 * max(abs(lam @ jv), 1e-12)


def test_adjoint_fixed_point_equation():
    """The adjoint solution satisfies lambda = dL/dm + J^T lambda; at a BP fixed point
    dL/dm vanishes, so the gradient equals its direct term."""
    rng = np.random.default_rng(4)
    g = G.square_lattice(4, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=6)
        g_direct, _ = e.grad(adjoint=False)
        g_adj, info = e.grad(adjoint=True, tol=1e-13)
        e.run(maxiter=2000, tol=1e-15)
        g_conv_d, _ = e.grad(adjoint=False)
        g_conv_a, info2 = e.grad(adjoint=True, tol=1e-13)
    assert info["adjoint_iterations"] >= 1
    assert np.max(np.abs(g_adj - g_direct)) > 1e-8  # the correction is active off the fixed point
    # the fidelity tolerance 1e-15 pins message directions to ~sqrt(1e-15) ~ 3e-8, so the
    # remaining correction is of that order
    assert np.max(np.abs(g_conv_a - g_conv_d)) <= 1e-6 * np.max(np.abs(g_conv_d))


def test_peps12x12_D6_fp32_gradient():
    """12x12 open PEPS, d=2, D=6, FP32 messages and gradient, FP64 log-scalars; checked
    against central FD (step 1e-4, FP64 solves) on 32 random unit directions."""
    rng = np.random.default_rng(12)
    g = G.square_lattice(12, 12, 6, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.init_messages()
        r = e.run(maxiter=500, tol=1e-12)
        grad, info = e.grad(adjoint=True, tol=1e-6)
    h = 1e-4
    gd, fds = [], []
    for _ in range(32):
        d = rng.standard_normal(t.size)
        d /= np.linalg.norm(d)
        fds.append((_logz(g, t + h * d) - _logz(g, t - h * d)) / (2 * h))
        gd.append(grad.astype(np.float64) @ d)
    gd, fds = np.array(gd), np.array(fds)
    rel = np.linalg.norm(gd - fds) / np.linalg.norm(fds)
    print(f"12x12 D=6 fp32 gradient: BP {r.iterations} sweeps, adjoint {info['adjoint_iterations']} its, "
          f"grad {info['device_ms']:.3f} ms, rel err vs FD over 32 directions {rel:.2e} "
          f"(worst direction {np.max(np.abs(gd - fds)) / np.max(np.abs(fds)):.2e} of the largest)")
    assert rel <= 1e-5


def test_implicit_gradient_against_oracle_finite_differences():
    """The implicit (converged fixed point) FP64 gradient against central differences of the
    FP64 CPU oracle's converged Bethe log-norm (BP to 1e-14 from the identity, the same
    schedule and stopping rule): within 1e-6 relative per direction."""
    from oracle import oracle as O
    rng = np.random.default_rng(24)
    g = G.square_lattice(4, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g)

    def oracle_logz(x):
        m, it, _, _ = O.bp_run(g, x, m0, maxiter=5000, tol=1e-14)
        assert it < 5000
        return O.bethe_free_energy(g, x, m)

    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        e.run(maxiter=5000, tol=1e-14)
        grad, info = e.grad(adjoint=True, tol=1e-12)
    h = 1e-4
    for _ in range(6):
        d = rng.standard_normal(t.size)
        d /= np.linalg.norm(d)
        fd = (oracle_logz(t + h * d) - oracle_logz(t - h * d)) / (2 * h)
        assert abs(grad @ d - fd) <= 1e-6 * max(abs(fd), 1.0), (grad @ d, fd)


# ---- unrolled gradient through the sweeps, with per-sweep checkpointing -------------------------

def _oracle_unrolled_logz(g, t, m0, sweeps):
    """log Z_BP after exactly `sweeps` parallel sweeps from m0 (FP64 oracle)."""
    from oracle import oracle as O
    m, it, _, _ = O.bp_run(g, t, m0, maxiter=sweeps)
    assert it == sweeps
    return O.bethe_free_energy(g, t, m)


def test_unrolled_gradient_against_finite_differences_fp64():
    """Not converged (6 sweeps from the identity): the unrolled gradient is the exact gradient
    of the 6-sweep computation, checked by central differences of the FP64 oracle."""
    rng = np.random.default_rng(21)
    g = G.square_lattice(4, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m0)
        grad, info = e.grad(sweeps=6, checkpoint=1)
    h = 1e-4
    for _ in range(6):
        d = rng.standard_normal(t.size)
        d /= np.linalg.norm(d)
        fd = (_oracle_unrolled_logz(g, t + h * d, m0, 6) - _oracle_unrolled_logz(g, t - h * d, m0, 6)) / (2 * h)
        assert abs(grad @ d - fd) <= 1e-7 * max(abs(fd), 1.0), (grad @ d, fd)


def test_checkpointed_gradient_equals_stored_gradient_bit_for_bit():
    """12x12 open D=6 FP32: 16 sweeps differentiated with every sweep's messages kept, with
    every 4th kept (the others recomputed) and every 5th (a segment cut by the last sweep):
    identical gradients and identical final messages."""
    rng = np.random.default_rng(22)
    g = G.square_lattice(12, 12, 6, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g)).astype(np.float32)
    m0 = G.identity_messages(g, np.float32)
    with BPEngine(g) as e:
        e.set_tensors(t)
        out = []
        for k in (1, 4, 5, 16):
            e.set_messages(m0)
            grad, info = e.grad(sweeps=16, checkpoint=k)
            out.append((grad, e.messages()))
    for grad, m in out[1:]:
        np.testing.assert_array_equal(grad, out[0][0])
        np.testing.assert_array_equal(m, out[0][1])


def test_unrolled_fp32_gradient_against_finite_differences():
    """12x12 open D=6, FP32 sweeps and gradient (FP64 log-scalars), 15 sweeps from the
    identity, against central differences of the FP64 oracle: within 1e-5 relative."""
    rng = np.random.default_rng(23)
    g = G.square_lattice(12, 12, 6, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    t32 = t.astype(np.float32)
    t = t32.astype(np.float64)  # the FP32 network, in FP64
    m0 = G.identity_messages(g)
    with BPEngine(g) as e:
        e.set_tensors(t32)
        e.set_messages(m0.astype(np.float32))
        grad, info = e.grad(sweeps=15, checkpoint=4)
    grad = grad.astype(np.float64)
    h = 1e-4
    for _ in range(4):
        d = rng.standard_normal(t.size)
        d /= np.linalg.norm(d)
        fd = (_oracle_unrolled_logz(g, t + h * d, m0, 15) - _oracle_unrolled_logz(g, t - h * d, m0, 15)) / (2 * h)
        assert abs(grad @ d - fd) <= 1e-5 * abs(fd), (grad @ d, fd)


def test_unrolled_gradient_at_a_fixed_point_matches_the_implicit_one():
    """From converged messages, sweeping further changes nothing and the unrolled gradient
    over many sweeps converges to the implicit (adjoint BP) gradient."""
    rng = np.random.default_rng(24)
    g = G.square_lattice(4, 4, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=500)  # the fidelity test stops at message changes of ~sqrt(tol): sweep on
        mstar = e.messages()
        gi, _ = e.grad(adjoint=True, tol=1e-13)
        gu, _ = e.grad(sweeps=60, checkpoint=8)
        np.testing.assert_allclose(e.messages(), mstar, rtol=0, atol=1e-12)
    assert np.max(np.abs(gu - gi)) <= 1e-8 * np.max(np.abs(gi))


@pytest.mark.parametrize("dtype,L_,D", [(np.float32, 12, 6), (np.float64, 5, 3)])
def test_persistent_adjoint_equals_per_iteration_launches(dtype, L_, D):
    """The adjoint iteration as one persistent cooperative launch (tensors and value messages
    staged once, a grid barrier and the stopping rule between iterations) and as one launch
    per iteration run the same arithmetic: same iteration count, residual and gradient, bit for
    bit."""
    rng = np.random.default_rng(31)
    g = G.square_lattice(L_, L_, D, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g)).astype(dtype)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=500, tol=1e-12)
        g_p, i_p = e.grad(adjoint=True, tol=1e-6)
        e.inject_fault("no_persistent_adjoint", 1)
        g_l, i_l = e.grad(adjoint=True, tol=1e-6)
        e.inject_fault("no_persistent_adjoint", 0)
        g_p2, _ = e.grad(adjoint=True, tol=1e-6)
    print(f"{L_}x{L_} D={D} {np.dtype(dtype).name}: persistent {i_p['device_ms']:.3f} ms, "
          f"per-iteration launches {i_l['device_ms']:.3f} ms, {i_p['adjoint_iterations']} iterations")
    assert i_p["adjoint_iterations"] == i_l["adjoint_iterations"] >= 2
    assert i_p["adjoint_residual"] == i_l["adjoint_residual"]
    np.testing.assert_array_equal(g_p, g_l)
    np.testing.assert_array_equal(g_p, g_p2)


def test_persistent_adjoint_barrier_that_runs_out_reports_timeout():
    """Fault injection without a GPU fault: one CTA of the persistent adjoint launch leaves
    before the first grid barrier, the others' bounded waits (1 ms) run out, itn_bp_grad
    returns ITN_ERR_TIMEOUT, and the same context then computes the gradient normally."""
    from itn_gb300 import ItnError
    from itn_gb300 import _lib as L
    rng = np.random.default_rng(32)
    g = G.square_lattice(6, 6, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=500, tol=1e-12)
        want, _ = e.grad(adjoint=True, tol=1e-8)
        e.inject_fault("wait_ns", 1_000_000)
        e.inject_fault("stall", 1)
        with pytest.raises(ItnError) as ei:
            e.grad(adjoint=True, tol=1e-8)
        assert ei.value.status == L.ITN_ERR_TIMEOUT
        e.inject_fault("stall", 0)
        e.inject_fault("wait_ns", 0)
        got, _ = e.grad(adjoint=True, tol=1e-8)
    np.testing.assert_array_equal(got, want)
