"""Parity of the benchmark workloads against the FP64 CPU oracle.

The 32x32 periodic PEPS norm network (d=2, D=8, entries N(0,1)/sqrt(d D^4), seed 32, the
benchmark's own network) is solved by the oracle in FP64 (30 parallel sweeps from the
normalised identity, beliefpropagation.jl:69-92 / :242-257) and its messages, per-vertex
log Z_v, per-edge log Z_e and Bethe log-norm (messagecache.jl:139-201) are the reference
every GPU mode is measured against:

* FP64 on CUDA cores: messages, log Z_v, log Z_e and the total within 1e-10 relative.
* FP32 on CUDA cores, and each tensor-core mode -- bf16 (27 BF16 + 3 BF16 hi/lo sweeps),
  tf32 (27 TF32 + 3 BF16 hi/lo sweeps), tf32x3 (every sweep TF32 hi/lo) -- within the bounds
  in BOUNDS: relative error of the total log-norm, the largest |delta log Z_v| over the
  sites, the largest |delta log Z_e| over the edges, and the largest per-message relative
  error (each message in its own scale).  The FP32 tensors are the FP64 ones rounded, so
  each bound includes that rounding.

The batched uneven workload (random 3-regular networks, bonds from {2,3,4,6,8}, complex
N(0,1) entries; the first 32 of the benchmark's 256 networks) is checked the same way
against the oracle in complex128: the GPU's complex128 solve within 1e-10 per message and
per scalar, its complex64 solve within 2e-6 per message and per scalar and 1e-7 on the real
part of each network's log-norm.  Measured on a GB300 (the per-site, per-edge and
per-message bounds are 2-3x these): FP64 3e-15; FP32 total 9.6e-10, site 3.2e-7, message
2.8e-7; bf16 6.7e-10 / 4.7e-6 / 3.9e-6; tf32 4.6e-10 / 1.8e-6 / 2.1e-6; tf32x3 2.3e-11 /
4.3e-7 / 4.7e-7; batched complex64 message 3.2e-7, Z_v 4.1e-7, log-norm 5.4e-9.  The total
of an FP32-accurate mode is a sum of 3072 log-scalars whose errors (~3e-7 each) have random
signs, about 2e-8 absolute on a log-norm of -4258: its bound is 5e-9 relative; the BF16 and
TF32 modes keep the 1e-6 target.
"""
import numpy as np
import pytest

from itn_gb300 import BPEngine
from itn_gb300 import graphs as G
from helpers import msg_rel

pytestmark = pytest.mark.gpu

SWEEPS = 30
# (total rel, max |d log Zv|, max |d log Ze|, max per-message rel) against the FP64 oracle
BOUNDS = {
    "fp32": (5e-9, 1e-6, 1e-6, 1e-6),
    "bf16": (1e-6, 1e-5, 1e-5, 1e-5),
    "tf32": (1e-6, 5e-6, 5e-6, 5e-6),
    "tf32x3": (5e-9, 1e-6, 1e-6, 1e-6),
}


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


@pytest.fixture(scope="module")
def headline():
    """The benchmark's network and the oracle's FP64 solve of it."""
    from oracle import oracle as O
    g = G.square_lattice(32, 32, 8, periodic=True, phys=2)
    t = G.random_tensors(g, np.random.default_rng(32), np.float64, G.peps_scale(g))
    m0 = G.identity_messages(g)
    m, it, _, _ = O.bp_run(g, t, m0, maxiter=SWEEPS)
    assert it == SWEEPS
    ref = O.logscalars(g, t, m)
    return g, t, m, ref


def _errors(g, ref_m, ref, m, ls):
    tot = abs(ls["totals"][0][0] - ref["total"][0]) / abs(ref["total"][0])
    site = float(np.max(np.abs(ls["logzv"][:, 0] - ref["logzv"][:, 0])))
    edge = float(np.max(np.abs(ls["logze"][:, 0] - ref["logze"][:, 0])))
    return tot, site, edge, msg_rel(g, m, ref_m)


def test_fp64_solve_matches_oracle(headline):
    g, t, ref_m, ref = headline
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        r = e.run(maxiter=SWEEPS)
        m = e.messages()
        ls = e.logscalars()
    assert r.iterations == SWEEPS
    tot, site, edge, mr = _errors(g, ref_m, ref, m, ls)
    print(f"fp64 vs oracle: total {tot:.2e} site {site:.2e} edge {edge:.2e} message {mr:.2e}")
    assert mr <= 1e-10
    np.testing.assert_allclose(ls["logzv"][:, 0], ref["logzv"][:, 0], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(ls["logze"][:, 0], ref["logze"][:, 0], rtol=1e-10, atol=1e-10)
    assert tot <= 1e-10
    assert int(ls["flags"][0]) == int(ref["flags"][0] | (ref["flags"][1] << 1) | (ref["flags"][2] << 2))


@pytest.mark.parametrize("mode", ["fp32", "bf16", "tf32", "tf32x3"])
def test_lower_precision_solve_against_oracle(headline, mode):
    g, t, ref_m, ref = headline
    kw = {"fp32": {}, "bf16": dict(precision="bf16", split_sweeps=3),
          "tf32": dict(precision="tf32", split_sweeps=3), "tf32x3": dict(precision="tf32x3")}[mode]
    with BPEngine(g) as e:
        e.set_tensors(t.astype(np.float32))
        e.init_messages()
        r = e.run(maxiter=SWEEPS, **kw)
        m = e.messages().astype(np.float64)
        ls = e.logscalars()
    assert r.iterations == SWEEPS
    tot, site, edge, mr = _errors(g, ref_m, ref, m, ls)
    print(f"{mode} vs FP64 oracle: total {tot:.2e} site {site:.2e} edge {edge:.2e} message {mr:.2e}")
    bt, bs, be, bm = BOUNDS[mode]
    assert tot <= bt and site <= bs and edge <= be and mr <= bm, (tot, site, edge, mr)


# ---- batched uneven networks ---------------------------------------------------------------

def _batched_subset(n_nets=32, seed=256):
    """The benchmark's graph draw (seed 256), keeping the first n_nets networks; complex
    N(0,1) tensors from a second seeded stream."""
    rng = np.random.default_rng(seed)
    nets = []
    for _ in range(256):
        n = int(rng.integers(8, 129)) * 2
        edges = G.random_regular_edges(n, 3, rng)
        bonds = rng.choice([2, 3, 4, 6, 8], size=len(edges))
        nets.append(G.from_edges(n, edges, bonds, phys=2))
    g = G.batched(nets[:n_nets])
    t = G.random_tensors(g, np.random.default_rng(seed + 1), np.complex128)
    return g, t


def _per_net_logz(g, logzv, logze):
    """Per-network sum of log Z_v minus sum of log Z_e (complex, from (re, im) pairs)."""
    und = np.flatnonzero(np.arange(g.nslots) < g.rev)
    src = np.repeat(np.arange(g.nv), np.diff(g.off))
    lv = logzv[:, 0] + 1j * logzv[:, 1]
    le = logze[:, 0] + 1j * logze[:, 1]
    out = np.zeros(g.n_nets, dtype=complex)
    np.add.at(out, g.net, lv)
    np.add.at(out, g.net[src[und]], -le)
    return out


@pytest.fixture(scope="module")
def batched():
    from oracle import oracle as O
    g, t = _batched_subset()
    m0 = G.identity_messages(g, np.complex128)
    m, it, _, _ = O.bp_run(g, t, m0, maxiter=SWEEPS)
    assert it == SWEEPS
    ref = O.logscalars(g, t, m)
    return g, t, m, ref


@pytest.mark.parametrize("dtype,bound_m,bound_z,bound_tot", [(np.complex128, 1e-10, 1e-10, 1e-12),
                                                             (np.complex64, 2e-6, 2e-6, 1e-7)])
def test_batched_uneven_against_oracle(batched, dtype, bound_m, bound_z, bound_tot):
    g, t, ref_m, ref = batched
    with BPEngine(g) as e:
        e.set_tensors(t.astype(dtype))
        e.init_messages()
        r = e.run(maxiter=SWEEPS)
        m = e.messages().astype(np.complex128)
        ls = e.logscalars()
    assert r.iterations == SWEEPS
    mr = msg_rel(g, m, ref_m)
    zv_rel = float(np.max(np.abs(ls["zv"] - ref["zv"]) / np.abs(ref["zv"])))
    ze_rel = float(np.max(np.abs(ls["ze"] - ref["ze"]) / np.abs(ref["ze"])))
    got = _per_net_logz(g, ls["logzv"], ls["logze"])
    want = _per_net_logz(g, ref["logzv"], ref["logze"])
    tot = float(np.max(np.abs(got.real - want.real) / np.abs(want.real)))
    # the imaginary part of a sum of logs is defined modulo 2 pi
    dim = np.abs(np.angle(np.exp(1j * (got.imag - want.imag))))
    print(f"batched {np.dtype(dtype).name}: message {mr:.2e} Zv {zv_rel:.2e} Ze {ze_rel:.2e} "
          f"log-norm re {tot:.2e} im {float(np.max(dim)):.2e}")
    assert mr <= bound_m and zv_rel <= bound_z and ze_rel <= bound_z
    assert tot <= bound_tot and float(np.max(dim)) <= bound_z
    # per-network totals straight from the library agree with the per-scalar sums
    np.testing.assert_allclose(ls["totals"][:, 0], got.real, rtol=1e-12, atol=1e-9)
