"""Generate the golden fixtures in tests/golden/ from the CPU oracle.

The reference (Julia ITensorNetworksNext.jl) has no stored golden vectors and cannot
run in this environment, so these fixtures are produced by the oracle after it passed
the reference's known-answer tests (tests/test_oracle_pins.py).  They freeze the seeded
inputs and outputs of the small configurations so that the GPU tests compare against
fixed numbers as well as against a live oracle run.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "itensornetworksnext.jl_gb300")]

from oracle import contract_oracle as C  # noqa: E402
from oracle import oracle as O  # noqa: E402
from itn_gb300 import generators as GEN  # noqa: E402
from itn_gb300 import graphs as G  # noqa: E402


def save(name, g, **arrays):
    np.savez_compressed(os.path.join(HERE, name), off=g.off, nbr=g.nbr, bond=g.bond, rev=g.rev,
                        phys=g.phys, layers=np.int64(g.layers), **arrays)


def main():
    # 4x4 open PEPS norm network, d=2, D=2, N(0,1) float64, normalised identity
    # messages, parallel schedule, 20 iterations; exact contraction alongside.
    rng = np.random.default_rng(20240401)
    g = G.square_lattice(4, 4, 2, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64)
    m0 = G.identity_messages(g)
    m, it, _, _ = O.bp_run(g, t, m0, maxiter=20)
    r = O.logscalars(g, t, m)
    z_exact = C.contract_norm(g, t)
    save("peps4x4_d2_D2_parallel20.npz", g, tensors=t, messages0=m0, messages=m,
         logzv=r["logzv"], logze=r["logze"], total=r["total"], z_exact=np.float64(z_exact),
         iterations=np.int64(it))
    # same network, sequential schedule (tree order + remaining edges), 5 sweeps
    edges = G.tree_edge_sequence(g)
    ms, it, _, _ = O.bp_run(g, t, m0, schedule="sequential", edges=edges, maxiter=5)
    r = O.logscalars(g, t, ms)
    save("peps4x4_d2_D2_sequential5.npz", g, tensors=t, messages0=m0, messages=ms, edges=edges,
         logzv=r["logzv"], logze=r["logze"], total=r["total"])
    # complex128 3x3 open, D=3, 15 parallel iterations
    rng = np.random.default_rng(77)
    g = G.square_lattice(3, 3, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.complex128, G.peps_scale(g))
    m0 = G.identity_messages(g, np.complex128)
    m, *_ = O.bp_run(g, t, m0, maxiter=15)
    r = O.logscalars(g, t, m)
    save("peps3x3_c128_D3_parallel15.npz", g, tensors=t, messages0=m0, messages=m,
         logzv=r["logzv"], logze=r["logze"], total=r["total"])
    # spin ice 3x3 torus, single layer, random messages, sequential, (maxiter 10, tol 1e-10)
    rng = np.random.default_rng(123)
    g = G.square_lattice(3, 3, 2, periodic=True, phys=1, layers=1)
    t = GEN.spin_ice_tensors(g)
    m0 = G.random_messages(g, rng)
    edges = G.tree_edge_sequence(g)
    m, it, delta, at = O.bp_run(g, t, m0, schedule="sequential", edges=edges, maxiter=10, tol=1e-10)
    r = O.logscalars(g, t, m)
    save("spinice3_sequential.npz", g, tensors=t, messages0=m0, messages=m, edges=edges,
         logzv=r["logzv"], logze=r["logze"], total=r["total"], iterations=np.int64(it))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
