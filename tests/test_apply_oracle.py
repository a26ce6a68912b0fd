"""Pins of the gate-application oracle (oracle/apply_oracle.py) against the reference's own
known answers for apply_operator (test/test_apply_operator.jl:66-145), restated on arrays:
* an untruncated gate is exact: contracting the gated network gives the operator applied
  to the contracted state (:70-91), for one- and two-site gates;
* on a tree with exact environments, a truncated two-site gate equals the globally optimal
  rank-k SVD truncation of the gated state (:93-118);
and the gram factor X^H X = env of gram_eigh_full_with_pinv.
"""
import numpy as np
import pytest

from oracle import apply_oracle as AO
from helpers import rand_psd, random_cycle4, cycle4_state, random_path4, path4_state, path_envs


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_gram_factor(dtype):
    rng = np.random.default_rng(1)
    m = rand_psd(rng, 5, dtype)
    x, xp = AO.gram_eigh_full_with_pinv(m)
    np.testing.assert_allclose(np.conj(x).T @ x, m, atol=1e-12)
    np.testing.assert_allclose(x @ xp, np.eye(5), atol=1e-10)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_untruncated_two_site_gate_is_exact(dtype):
    rng = np.random.default_rng(2)
    T = random_cycle4(rng, dtype, d=3, bonds=(2, 3, 2, 3))
    op = rng.standard_normal((3, 3, 3, 3)).astype(dtype)
    if np.dtype(dtype).kind == "c":
        op = op + 1j * rng.standard_normal((3, 3, 3, 3))
    # gate on sites 1, 2: site 1 axes [b, s1, c], site 2 axes [d, s2, c]
    psi1 = np.transpose(T[1], (0, 2, 1))          # T1[b, c, s1] -> [b, s1, c]
    psi2 = np.transpose(T[2], (1, 2, 0))          # T2[c, d, s2] -> [d, s2, c]
    e1, e2 = rand_psd(rng, T[1].shape[0], dtype), rand_psd(rng, T[2].shape[1], dtype)
    n1, n2, s = AO.apply_gate_2site(psi1, psi2, [e1], [e2], op)
    T2 = list(T)
    T2[1] = np.transpose(n1, (0, 2, 1))           # [b, chi, s1]
    T2[2] = np.transpose(n2, (2, 0, 1))           # [chi, d, s2]
    got = cycle4_state(T2)
    want = np.einsum("xyst,astb->axyb", op, cycle4_state(T))
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-10 * np.abs(want).max())


@pytest.mark.parametrize("k", [1, 2, 3])
@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_truncated_gate_matches_optimal_svd_on_tree(k, dtype):
    rng = np.random.default_rng(3)
    T = random_path4(rng, dtype, d=3, bonds=(3, 4, 3))
    op = rng.standard_normal((3, 3, 3, 3)).astype(dtype)
    if np.dtype(dtype).kind == "c":
        op = op + 1j * rng.standard_normal((3, 3, 3, 3))
    psi1 = np.transpose(T[1], (0, 2, 1))          # T1[b, c, s1] -> [b, s1, c]
    psi2 = np.transpose(T[2], (1, 2, 0))          # T2[c, d, s2] -> [d, s2, c]
    eb, ed = path_envs(T)
    n1, n2, s = AO.apply_gate_2site(psi1, psi2, [eb], [ed], op, maxrank=k)
    T2 = list(T)
    T2[1] = np.transpose(n1, (0, 2, 1))
    T2[2] = np.transpose(n2, (2, 0, 1))
    got = path4_state(T2)
    full = np.einsum("xyst,astb->axyb", op, path4_state(T))
    u, sv, vh = np.linalg.svd(full.reshape(9, 9))
    want = ((u[:, :k] * sv[:k]) @ vh[:k]).reshape(full.shape)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9 * np.abs(want).max())


def test_one_site_gate_normalized():
    rng = np.random.default_rng(4)
    psi = rng.standard_normal((2, 3, 3))
    envs = [rand_psd(rng, 2, np.float64), rand_psd(rng, 3, np.float64)]
    op = rng.standard_normal((3, 3))
    out = AO.apply_gate_1site(psi, envs, op, normalize=True)
    x0 = AO.gram_eigh_full_with_pinv(envs[0])[0]
    x1 = AO.gram_eigh_full_with_pinv(envs[1])[0]
    g = np.einsum("ia,jb,abs->ijs", x0, x1, out)
    assert abs(np.linalg.norm(g) - 1) < 1e-12
    raw = np.einsum("ts,abs->abt", op, psi)
    np.testing.assert_allclose(out / np.linalg.norm(out), raw / np.linalg.norm(raw), atol=1e-12)
