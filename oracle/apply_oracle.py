"""BP simple-update gate application oracle (numpy).  TEST INFRASTRUCTURE ONLY.

Restates apply_gate_bp! (src/apply/apply_operators.jl:209-283):

* one-site gate (:229-246): psi_v <- op applied on the site index; with ``normalize`` the
  result is divided by the norm of psi_v with the gauges of all incoming environment
  messages absorbed on its link legs.
* two-site gate on neighbours v1, v2 (:248-283): gauges X_e with X_e^H X_e = env[e] and
  their pseudo-inverses are absorbed on the other legs of each site; each gauged site is
  split by a compact QR into Q (other legs) and R (site index and shared bond); the
  operator is applied to R1 * R2, the result is split by a truncated SVD, sqrt(S) is
  absorbed into both halves, Q and the inverse gauges are re-applied, and the
  environment of the new bond in both directions becomes diag(S) (normalised by its
  norm when ``normalize``).

The matrix routines live in un-vendored dependencies: ``gram_eigh_full`` and
``gram_eigh_full_with_pinv`` in TensorAlgebra 0.16 (MatrixAlgebra), ``qr_compact`` and
``svd_trunc`` / ``truncrank`` in MatrixAlgebraKit.  They are restated from their
definitions: for a Hermitian positive semi-definite M = U diag(w) U^H the gram factor is
X = diag(sqrt w) U^H (so X^H X = M) and its pseudo-inverse U diag(1/sqrt w) (w above a
relative cutoff); QR and SVD are numpy.linalg's compact factorisations; ``truncrank(k)``
keeps the k largest singular values.

Array conventions (shared with the GPU entry point): a site tensor is an array with axes
[other legs..., site index, shared bond] (the shared bond axis is absent for a one-site
gate); an environment message is a D x D matrix M[bra, ket]; a two-site operator is an
array op[s1', s2', s1, s2], a one-site operator op[s', s].
"""
from __future__ import annotations

import numpy as np

PINV_RTOL = 1e-12


def gram_eigh_full_with_pinv(m):
    """(X, X^+) with X^H X = m for Hermitian PSD m (TensorAlgebra gram_eigh_full_with_pinv)."""
    m = 0.5 * (np.asarray(m) + np.conj(np.asarray(m)).T)
    w, u = np.linalg.eigh(m)
    w = np.clip(w, 0.0, None)
    keep = w > PINV_RTOL * max(w.max(initial=0.0), np.finfo(float).tiny)
    sq = np.sqrt(w)
    x = (sq[:, None] * np.conj(u).T)
    inv = np.zeros_like(sq)
    inv[keep] = 1.0 / sq[keep]
    xp = u * inv[None, :]
    return x, xp


def _apply_on_axis(t, mat, axis):
    """t[..., a, ...] <- sum_c mat[a, c] t[..., c, ...]"""
    out = np.tensordot(mat, t, axes=([1], [axis]))
    return np.moveaxis(out, 0, axis)


def apply_gate_1site(psi, envs, op, normalize=False):
    """psi: [other legs..., s]; envs: one D x D matrix per other leg (None = no gauge)."""
    out = _apply_on_axis(psi, np.asarray(op), psi.ndim - 1)
    if normalize:
        g = out
        for j, m in enumerate(envs):
            if m is not None:
                g = _apply_on_axis(g, gram_eigh_full_with_pinv(m)[0], j)
        out = out / np.linalg.norm(g)
    return out


def _truncate(s, maxrank, cutoff):
    k = len(s)
    if maxrank is not None and maxrank > 0:
        k = min(k, maxrank)
    if cutoff is not None and cutoff > 0:
        k = min(k, int(np.sum(s > cutoff)))
    return max(k, 1)


def apply_gate_2site(psi1, psi2, envs1, envs2, op, maxrank=None, cutoff=None, normalize=False):
    """psi_i: [other legs..., s_i, b] (b = the bond joining the two sites); envs_i: one
    matrix per other leg.  Returns (new psi1 [others..., s1, c], new psi2 [others..., s2, c], S)."""
    op = np.asarray(op)
    gs = []
    for psi, envs in ((psi1, envs1), (psi2, envs2)):
        x = psi
        inv = []
        for j, m in enumerate(envs):
            if m is None:
                inv.append(None)
                continue
            g, gp = gram_eigh_full_with_pinv(m)
            x = _apply_on_axis(x, g, j)
            inv.append(gp)
        gs.append((x, inv))
    (a1, inv1), (a2, inv2) = gs
    o1, o2 = a1.shape[:-2], a2.shape[:-2]
    d1, d2, bond = a1.shape[-2], a2.shape[-2], a1.shape[-1]
    q1, r1 = np.linalg.qr(a1.reshape(-1, d1 * bond))
    q2, r2 = np.linalg.qr(a2.reshape(-1, d2 * bond))
    k1, k2 = r1.shape[0], r2.shape[0]
    r1 = r1.reshape(k1, d1, bond)
    r2 = r2.reshape(k2, d2, bond)
    t = np.einsum("asb,ctb->asct", r1, r2)                    # [k1, s1, k2, s2]
    theta = np.einsum("xyst,asct->axcy", op, t)               # [k1, s1', k2, s2']
    u, s, vh = np.linalg.svd(theta.reshape(k1 * d1, k2 * d2), full_matrices=False)
    chi = _truncate(s, maxrank, cutoff)
    u, s, vh = u[:, :chi], s[:chi], vh[:chi]
    if normalize:
        s = s / np.linalg.norm(s)
    sq = np.sqrt(s)
    r1n = (u * sq[None, :]).reshape(k1, d1, chi)
    r2n = (sq[:, None] * vh).reshape(chi, k2, d2)
    n1 = np.tensordot(q1, r1n, axes=([1], [0])).reshape(*o1, d1, chi)
    n2 = np.tensordot(q2, np.transpose(r2n, (1, 2, 0)), axes=([1], [0])).reshape(*o2, d2, chi)
    for j, gp in enumerate(inv1):
        if gp is not None:
            n1 = _apply_on_axis(n1, gp, j)
    for j, gp in enumerate(inv2):
        if gp is not None:
            n2 = _apply_on_axis(n2, gp, j)
    return n1, n2, s
