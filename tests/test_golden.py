"""The oracle reproduces the committed golden fixtures (generated by
tests/golden/make_golden.py), and the fixtures are internally consistent."""
import numpy as np
import pytest

from oracle import contract_oracle as C
from oracle import oracle as O
from helpers import load_golden, max_rel


def test_peps4x4_parallel():
    g, d = load_golden("peps4x4_d2_D2_parallel20.npz")
    m, it, *_ = O.bp_run(g, d["tensors"], d["messages0"], maxiter=20)
    assert it == 20
    assert max_rel(m, d["messages"]) < 1e-13
    r = O.logscalars(g, d["tensors"], m)
    assert max_rel(r["logzv"], d["logzv"]) < 1e-12
    assert abs(r["total"][0] - d["total"][0]) < 1e-12 * abs(d["total"][0])
    # exact contraction of the same 4x4 norm network
    z = C.contract_norm(g, d["tensors"])
    assert abs(z - d["z_exact"]) < 1e-12 * abs(z)
    # BP is not exact on a lattice with loops, but close for this network
    assert abs(r["total"][0] - np.log(z)) < 0.5


def test_peps4x4_sequential():
    g, d = load_golden("peps4x4_d2_D2_sequential5.npz")
    m, *_ = O.bp_run(g, d["tensors"], d["messages0"], schedule="sequential", edges=d["edges"], maxiter=5)
    assert max_rel(m, d["messages"]) < 1e-13


def test_complex_parallel():
    g, d = load_golden("peps3x3_c128_D3_parallel15.npz")
    m, *_ = O.bp_run(g, d["tensors"], d["messages0"], maxiter=15)
    assert max_rel(m, d["messages"]) < 1e-13


def test_spin_ice_fixture():
    g, d = load_golden("spinice3_sequential.npz")
    m, it, *_ = O.bp_run(g, d["tensors"], d["messages0"], schedule="sequential", edges=d["edges"],
                         maxiter=10, tol=1e-10)
    assert it == int(d["iterations"])
    assert max_rel(m, d["messages"]) < 1e-13
    assert abs(np.exp(d["total"][0]) / 1.5 ** 9 - 1) < 1e-6
