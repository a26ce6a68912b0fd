"""Tensor-core (tcgen05) BF16 sweep: self-test, per-update error against the FP32
CUDA-core path, split-precision recovery, and the 32x32 D=8 log-norm error against
an FP64 solve.

Stated bounds: one BF16 sweep from the same messages stays within 3e-2 relative per
message of the FP32 sweep (BF16 operands, FP32 accumulation); one TF32 sweep within 5e-3;
one split (hi/lo) sweep within 2e-4; the mixed solves (27 BF16 or TF32 + 3 split sweeps)
give the Bethe log-norm of the 32x32 periodic D=8 network within 1e-6 relative of the FP64
solve.
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


def _lattice(L, seed, dtype=np.float32):
    g = G.square_lattice(L, L, 8, periodic=True, phys=2)
    rng = np.random.default_rng(seed)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    return g, t


def test_tc_selftest():
    g = G.square_lattice(3, 3, 2, phys=2)
    with BPEngine(g) as e:
        r = e.tc_selftest()
    print("tcgen05 self-test:", r)
    assert r["m128_ok"] and r["max_err"] < 1e-6
    assert r["m64_ok"]
    assert len(set(r["lane_of_row"].tolist())) == 64


def _one_sweep(g, t, m0, **kw):
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.set_messages(m0)
        e.run(maxiter=1)
        ref = e.messages()
        e.set_messages(m0)
        e.run(maxiter=1, **kw)
        return msg_rel(g, e.messages(), ref)


@pytest.mark.parametrize("prec,split,tol", [("bf16", False, 3e-2), ("tf32", False, 5e-3), ("bf16", True, 2e-4),
                                            ("tf32x3", False, 1e-5)])
def test_one_sweep_against_fp32(prec, split, tol):
    """Non-symmetric messages near the normalised identity (the regime of a BP solve):
    a transposed bra/ket index anywhere would show up as an O(1) error."""
    g, t = _lattice(4, 1)
    rng = np.random.default_rng(5)
    m0 = G.identity_messages(g, np.float32) + 0.05 * G.random_messages(g, rng, np.float32)
    err = _one_sweep(g, t, m0, precision=prec, split_sweeps=1 if split else 0)
    print(f"{prec} split={split}: per-message rel err vs FP32 = {err:.3e}")
    assert err < tol


def test_split_recovers_ill_conditioned_update():
    """Dense positive messages make each update a sum with heavy cancellation; the
    split (hi/lo) sweep must be far more accurate than the plain BF16 one."""
    g, t = _lattice(4, 2)
    rng = np.random.default_rng(6)
    m0 = np.abs(G.random_messages(g, rng, np.float32)) + 0.1
    e_bf16 = _one_sweep(g, t, m0, precision="bf16", split_sweeps=0)
    e_split = _one_sweep(g, t, m0, precision="bf16", split_sweeps=1)
    print(f"ill-conditioned: bf16 {e_bf16:.3e} split {e_split:.3e}")
    assert e_split < 1e-2 and e_split * 20 < e_bf16
    e_x3 = _one_sweep(g, t, m0, precision="tf32x3")
    print(f"ill-conditioned: tf32x3 {e_x3:.3e}")
    assert e_x3 * 20 < e_split


@pytest.mark.parametrize("prec", ["bf16", "tf32"])
def test_mixed_logz_32x32_against_fp64(prec):
    g, t = _lattice(32, 32)
    with BPEngine(g) as e64:
        e64.set_tensors(t)
        e64.init_messages()
        e64.run(maxiter=30)
        lz64 = e64.bethe_free_energy()
        lzv64 = e64.logscalars()["logzv"][:, 0]
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.init_messages()
        r = e.run(maxiter=30, precision=prec, split_sweeps=3)
        assert r.iterations == 30
        lz = e.bethe_free_energy()
        lzv = e.logscalars()["logzv"][:, 0]
        e.init_messages()
        e.run(maxiter=30)
        lz32 = e.bethe_free_energy()
    rel = abs(lz - lz64) / abs(lz64)
    print(f"log-norm: fp64 {lz64:.12f} mixed {prec} {lz:.12f} rel {rel:.3e}; fp32 rel {abs(lz32 - lz64) / abs(lz64):.3e};"
          f" max per-site |dlogZv| {np.max(np.abs(lzv - lzv64)):.3e}")
    assert rel <= 1e-6


def test_tf32x3_solve_matches_fp32_accuracy():
    """Every sweep in TF32 hi/lo on the tensor cores: the log-norm and the per-site
    log-scalars of a 30-sweep 32x32 solve are as close to the FP64 solve as the FP32
    CUDA-core solve's are (within 3x, plus a 1e-6 floor per site)."""
    g, t = _lattice(32, 32)
    with BPEngine(g) as e64:
        e64.set_tensors(t)
        e64.init_messages()
        e64.run(maxiter=30)
        lz64 = e64.bethe_free_energy()
        lzv64 = e64.logscalars()["logzv"][:, 0]
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.init_messages()
        r = e.run(maxiter=30, precision="tf32x3")
        assert r.iterations == 30
        lz = e.bethe_free_energy()
        lzv = e.logscalars()["logzv"][:, 0]
        e.init_messages()
        e.run(maxiter=30)
        lz32 = e.bethe_free_energy()
        lzv32 = e.logscalars()["logzv"][:, 0]
    site, site32 = np.max(np.abs(lzv - lzv64)), np.max(np.abs(lzv32 - lzv64))
    print(f"tf32x3: rel {abs(lz - lz64) / abs(lz64):.3e} site {site:.3e}; fp32 rel {abs(lz32 - lz64) / abs(lz64):.3e}"
          f" site {site32:.3e}")
    assert abs(lz - lz64) <= 1e-8 * abs(lz64)
    assert site <= 3 * site32 + 1e-6


def test_tc_convergence_flag():
    g, t = _lattice(6, 3)
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.init_messages()
        r = e.run(maxiter=200, tol=1e-5, precision="bf16", split_sweeps=0)
        assert 1 <= r.iterations < 200 and r.at_iteration == r.iterations and r.delta < 1e-5


@pytest.mark.parametrize("L,n,split,prec", [(32, 7, 0, "bf16"), (32, 6, 2, "bf16"), (4, 5, 1, "bf16"),
                                            (3, 9, 0, "bf16"), (48, 5, 1, "bf16"), (32, 5, 0, "tf32"),
                                            (4, 6, 3, "tf32"), (4, 2, 0, "bf16"), (4, 1, 0, "bf16"),
                                            (4, 3, 5, "bf16"), (32, 5, 0, "tf32x3"), (4, 4, 0, "tf32x3"),
                                            (32, 7, 7, "bf16")])
def test_persistent_matches_per_sweep_launches(L, n, split, prec):
    """Without a convergence test the sweeps run as one cooperative launch per precision
    part (tagged message entries instead of kernel boundaries); with one the engine
    launches once per sweep.  Both run the same per-item arithmetic, so the messages must
    agree bit for bit -- a missed dependency would read a stale or half-written message.
    32x32 and 48x48 (about four items per group per sweep) have more half-vertex items than
    groups, 4x4 and 3x3 (the smallest periodic lattice, one CTA) fewer.  Two-sweep parts run
    as per-sweep launches in both forms, one-sweep parts read the plain input and write the
    plain output in the same sweep, and more split sweeps than sweeps makes every sweep split.
    Launches of 4 or fewer groups per CTA (split, TF32, TF32 hi/lo) deal (sweep, item) tickets
    round-robin over the whole launch; 32x32 with 7 split sweeps gives each of the 608 groups
    tickets of several sweeps."""
    g, t = _lattice(L, 11)
    rng = np.random.default_rng(12)
    m0 = G.identity_messages(g, np.float32) + 0.05 * G.random_messages(g, rng, np.float32)
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.set_messages(m0)
        r1 = e.run(maxiter=n, precision=prec, split_sweeps=split)
        a = e.messages()
        e.set_messages(m0)
        r2 = e.run(maxiter=n, tol=1e-300, precision=prec, split_sweeps=split)
        b = e.messages()
    assert r1.iterations == n and r2.iterations == n
    if n > 2:
        assert r1.kernel_launches < r2.kernel_launches
    np.testing.assert_array_equal(a, b)
