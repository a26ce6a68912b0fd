"""contract_network on the GPU against the numpy oracle (same greedy order; the sweep order
against the oracle's greedy-order value).

Bounds: FP64 and complex128 within 1e-12 relative of the oracle (FP32 / complex64 1e-5); order independence
within 1e3 eps (test/test_contract_network.jl:26-45); the BF16-split tensor-core GEMM
within 1e-4 relative in FP32.
"""
import numpy as np
import pytest

from oracle import contract_oracle as C
from itn_gb300 import graphs as G
from itn_gb300.contract import contract_network, contract_norm_network, norm_network_tensors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def test_vector_network_orders_agree():
    """Four tensors of test_contract_network.jl:13-24: every order gives the same value."""
    A = np.array([[1.0, 1.0], [0.5, 1.0]])
    B = np.array([2.0, 1.0])
    Cc = np.array([5.0, 1.0])
    Dd = np.array([-2.0, 3.0, 4.0, 5.0, 1.0])
    ts, ls = [A, B, Cc, Dd], [["i", "j"], ["i"], ["j"], ["k"]]
    r1, l1 = contract_network(ts, ls, alg="left")
    r2, l2 = contract_network(ts, ls, alg="greedy")
    ref, lref = C.contract_network(ts, ls, "left")
    assert l1 == ["k"] and l2 == ["k"]
    assert np.array_equal(r1, ref) and np.array_equal(r2, ref)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_peps4x4_norm_network(dtype):
    rng = np.random.default_rng(44)
    g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
    t = G.random_tensors(g, rng, dtype)
    z = contract_norm_network(g, t)
    ref = C.contract_norm(g, t)
    assert abs(z - ref) <= 1e-12 * abs(ref)
    assert abs(np.imag(z)) <= 1e-12 * abs(z)


def test_order_independence_4x4_plain():
    rng = np.random.default_rng(3)
    g = G.square_lattice(4, 4, 2, phys=1, layers=1)
    t = G.random_tensors(g, rng, np.float64)
    ts, ls = C.plain_network(g, t)
    z1 = contract_network(ts, ls, alg="left")[0][()]
    z2 = contract_network(ts, ls, alg="greedy")[0][()]
    assert abs(z1 - z2) <= 1e3 * np.finfo(float).eps * abs(z1)


def test_open_indices_state_vector():
    """<psi|psi> = |psi|^2 with psi contracted on the GPU (open site indices)."""
    rng = np.random.default_rng(5)
    g = G.square_lattice(2, 3, 2, phys=2)
    t = G.random_tensors(g, rng, np.complex128)
    ts, ls = C.plain_network(g, t)
    psi, lab = contract_network(ts, ls)
    ref, lref = C.contract_network(ts, ls)
    perm = [lab.index(x) for x in lref]
    assert np.allclose(np.transpose(psi, perm), ref, rtol=1e-12, atol=0)
    assert abs(np.vdot(psi, psi) - contract_norm_network(g, t)) <= 1e-12 * abs(np.vdot(psi, psi))


def test_peps6x6_D3_norm_network():
    """Exact <psi|psi> of the 6x6 D=3 PEPS (the exact reference for the 16x16 D=4 BP
    configuration's error study): 43M-element intermediates, ~0.66 TFLOP in FP64."""
    rng = np.random.default_rng(63)
    g = G.square_lattice(6, 6, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    ts, ls = norm_network_tensors(g, t)
    z, _, ms = contract_network(ts, ls, return_time=True)
    ref = C.contract_norm(g, t)
    print(f"6x6 D=3 norm network: {ms:.1f} ms on the GPU, z = {z[()]:.6e}")
    assert abs(z[()] - ref) <= 1e-10 * abs(ref)
    # the sweep order (boundary-sweep contraction, 150x fewer multiply-adds) gives the same
    # value to FP64 rounding
    zs, _, ms_s = contract_network(ts, ls, alg="sweep", return_time=True)
    print(f"6x6 D=3 norm network, sweep order: {ms_s:.1f} ms on the GPU")
    assert abs(zs[()] - ref) <= 1e-10 * abs(ref)
    assert ms_s < ms


@pytest.mark.parametrize("dtype", [np.float32, np.complex64, np.complex128])
def test_sweep_order_contractions_against_oracle(dtype):
    """contract_network with order_alg sweep on norm and plain networks (periodic, open, with
    open indices) against the oracle's contraction."""
    rng = np.random.default_rng(21)
    tol = 1e-12 if dtype == np.complex128 else 1e-5
    for L, D, per in ((4, 2, False), (3, 3, True)):
        g = G.square_lattice(L, L, D, periodic=per, phys=2)
        t = G.random_tensors(g, rng, dtype, G.peps_scale(g))
        ts, ls = norm_network_tensors(g, t)
        z, _ = contract_network(ts, ls, alg="sweep")
        ref = C.contract_norm(g, t)
        assert abs(z[()] - ref) <= tol * abs(ref)
    g = G.square_lattice(2, 3, 2, phys=2)
    t = G.random_tensors(g, rng, dtype)
    ts, ls = C.plain_network(g, t)
    psi, lab = contract_network(ts, ls, alg="sweep")
    ref, lref = C.contract_network(ts, ls)
    perm = [lab.index(x) for x in lref]
    assert np.allclose(np.transpose(psi, perm), ref, rtol=tol, atol=tol * np.max(np.abs(ref)))


def test_bf16_split_tensor_core_gemm():
    rng = np.random.default_rng(9)
    A = rng.standard_normal((300, 257)).astype(np.float32)
    B = rng.standard_normal((257, 130)).astype(np.float32)
    out, lab = contract_network([A, B], [["m", "k"], ["k", "n"]], precision="bf16")
    ref = A.astype(np.float64) @ B.astype(np.float64)
    assert lab == ["m", "n"]
    assert np.max(np.abs(out - ref)) <= 1e-4 * np.max(np.abs(ref))
    # a norm network in FP32 through the tensor cores
    g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float32, G.peps_scale(g))
    z = contract_norm_network(g, t, precision="bf16")
    zr = C.contract_norm(g, t.astype(np.float64))
    assert abs(z - zr) <= 1e-4 * abs(zr)


def test_tf32_split_tensor_core_gemm_has_fp32_accuracy():
    """TF32 hi/lo operands (3 kind::tf32 MMAs per product, partial sums promoted to FP32
    registers after every K = 64 tile).  One pairwise step is as accurate as FP32 arithmetic:
    within 4x the FP32 CUDA-core GEMM's error (plus 2e-7) on small and large shapes and
    magnitudes down to 1e-18.  Measured on a GB300: 300 x 1031 x 130 tf32x3 6.7e-7, FP32 CUDA
    cores 1.5e-6, BF16 split 4.9e-6 (without the per-tile promotion the tensor core's own
    sum over K = 1031 gave 7.8e-6); 4 x 4 x 4 1.4e-7 vs 4.9e-8.  Chained steps: the tensor
    core's sums within a tile are not rounded like FP32 additions and their errors add up over
    a contraction's steps -- 3.6e-6 on the 32 steps of a 4x4 D=2 norm network against
    3.6e-8 for FP32 CUDA cores -- so that case is bounded at 1e-5, ten times below the BF16
    split bound of 1e-4."""
    rng = np.random.default_rng(10)
    for (m, k, n), scale in [((300, 1031, 130), 1.0), ((4, 4, 4), 1.0), ((16, 8, 16), 1e-10),
                             ((64, 64, 64), 1e-18), ((200, 300, 100), 1.0)]:
        A = (rng.standard_normal((m, k)) * scale).astype(np.float32)
        B = (rng.standard_normal((k, n)) * scale).astype(np.float32)
        ref = A.astype(np.float64) @ B.astype(np.float64)
        top = np.max(np.abs(ref))
        out, lab = contract_network([A, B], [["m", "k"], ["k", "n"]], precision="tf32x3")
        fp32, _ = contract_network([A, B], [["m", "k"], ["k", "n"]])
        err, err32 = (float(np.max(np.abs(x - ref))) / top for x in (out, fp32))
        print(f"gemm {m}x{k}x{n} (scale {scale:g}) vs FP64: tf32x3 {err:.2e}, fp32 CUDA cores {err32:.2e}")
        assert lab == ["m", "n"]
        assert err <= 4 * err32 + 2e-7 and err <= 1e-6
    # a norm network in FP32 through the tensor cores (32 chained steps)
    g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float32, G.peps_scale(g))
    z = contract_norm_network(g, t, precision="tf32x3")
    z32 = contract_norm_network(g, t)
    zr = C.contract_norm(g, t.astype(np.float64))
    e, e32 = abs(z - zr) / abs(zr), abs(z32 - zr) / abs(zr)
    print(f"4x4 D=2 norm network (every step stored in FP32): tf32x3 {e:.2e}, fp32 CUDA cores {e32:.2e}")
    assert e <= 1e-5


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
@pytest.mark.parametrize("m,k,n", [(5000, 9, 7), (7, 9, 5000), (300, 64, 32), (32, 1, 4096), (257, 3, 1),
                                   (32, 64, 256), (256, 65, 8), (33, 8, 33)])
def test_thin_pairwise_contractions(dtype, m, k, n):
    """Pairwise steps with one thin side (at most 32 rows or columns, K <= 64: the steps of a
    boundary sweep) run on the thin-operand GEMM; against numpy in FP64 / complex128."""
    rng = np.random.default_rng(m * 31 + n)
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((k, n))
    if np.dtype(dtype).kind == "c":
        a = a + 1j * rng.standard_normal((m, k))
        b = b + 1j * rng.standard_normal((k, n))
    ref = a @ b
    out, lab = contract_network([a.astype(dtype), b.astype(dtype)], [["i", "k"], ["k", "j"]])
    tol = 1e-12 if np.dtype(dtype).itemsize >= 16 or dtype == np.float64 else 1e-5
    got = out if lab == ["i", "j"] else out.T
    assert np.max(np.abs(got - ref)) <= tol * np.max(np.abs(ref)) * np.sqrt(k)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
def test_thin_steps_with_the_long_operand_out_of_order(dtype):
    """Thin steps whose long operand carries its contracted indices in the middle or first (read
    in place through a strided view instead of being permuted), with unit and adjacent free
    axes; against numpy einsum."""
    rng = np.random.default_rng(5)
    cases = [
        # long tensor (a, k, b, c) with k contracted against a thin (k, j)
        ("akbc,kj->abcj", [(40, 3, 7, 5), (3, 6)]),
        # contracted axes first and last in the long tensor, thin tensor first in the pair
        ("jkl,kabcl->jabc", [(4, 3, 2), (3, 9, 1, 30, 2)]),
        # two contracted axes split around free ones
        ("kaml,kl->am", [(2, 33, 17, 3), (2, 3)]),
    ]
    for spec, shapes in cases:
        ins, out = spec.split("->")
        labs = [list(x) for x in ins.split(",")]
        ts = []
        for sh in shapes:
            x = rng.standard_normal(sh)
            if np.dtype(dtype).kind == "c":
                x = x + 1j * rng.standard_normal(sh)
            ts.append(x)
        ref = np.einsum(spec, *ts)
        got, lab = contract_network([t.astype(dtype) for t in ts], labs)
        perm = [lab.index(x) for x in out]
        tol = 1e-12 if np.dtype(dtype) in (np.float64, np.complex128) else 1e-5
        assert np.max(np.abs(np.transpose(got, perm) - ref)) <= tol * np.max(np.abs(ref)) * 4, spec
