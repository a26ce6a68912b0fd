"""Single-layer network generators used as known-answer inputs.

* ``delta_network``  -- delta tensors on every vertex (ITensorNetworkGenerators/delta_network.jl:44-53)
* ``ising_network``  -- classical Ising partition function: deltas with a square-root bond
  matrix applied on each edge end (ITensorNetworkGenerators/ising_network.jl:7-51), so that
  contracting a link gives exp(beta * (J s1 s2 + h1 s1 + h2 s2)), h split by degree
* ``spin_ice_network`` -- the 2-in-2-out tensor of test_beliefpropagation.jl:16-36, whose
  BP partition function is 1.5^(n^2) on an n x n torus

All return packed row-major tensors for a ``Graph`` with ``layers=1`` and ``phys=1``.
"""
from __future__ import annotations

import itertools

import numpy as np

from .graphs import Graph


def _apply_leg(T, leg, M, side):
    """Contract matrix M into axis ``leg`` of T: side 0 uses M[s, a], side 1 M[a, s]."""
    Mx = M if side == 0 else M.T
    T = np.moveaxis(T, leg, -1)
    T = T @ Mx
    return np.moveaxis(T, -1, leg)


def delta_tensors(g: Graph, dtype=np.float64):
    out = np.zeros(int(g.toff[-1]), dtype=dtype)
    for u in range(g.nv):
        dims = g.legs(u)
        T = np.zeros(dims, dtype=dtype)
        for i in range(min(dims) if dims else 1):
            T[(i,) * len(dims)] = 1
        out[g.toff[u]:g.toff[u + 1]] = T.ravel()
    return out


def sqrt_ising_bond(beta, J=1.0, h=0.0, deg1=1, deg2=1):
    h1 = h / deg1
    h2 = h / deg2
    m = np.array([[np.exp(beta * (J + h1 + h2)), np.exp(beta * (-J + h1 - h2))],
                  [np.exp(beta * (-J - h1 + h2)), np.exp(beta * (J - h1 - h2))]])
    w, v = np.linalg.eig(m)
    r = v @ np.diag(np.sqrt(w.astype(complex))) @ np.linalg.inv(v)
    return np.real_if_close(r).real


def ising_network(g: Graph, beta, J=1.0, h=0.0, dtype=np.float64):
    """Packed tensors for the Ising model on ``g`` (bond dims must be 2)."""
    if np.any(g.bond != 2):
        raise ValueError("Ising links have dimension 2")
    ts = []
    for u in range(g.nv):
        dims = g.legs(u)
        T = np.zeros(dims)
        for i in range(2):
            T[(i,) * len(dims)] = 1.0
        ts.append(T)
    for u in range(g.nv):
        for leg, s in enumerate(range(g.off[u], g.off[u + 1])):
            w = int(g.nbr[s])
            first = s < g.rev[s]  # the edge's first end carries rows, the other columns
            a, b = (u, w) if first else (w, u)
            M = sqrt_ising_bond(beta, J, h, g.degree(a), g.degree(b))
            ts[u] = _apply_leg(ts[u], leg, M, 0 if first else 1)
    out = np.zeros(int(g.toff[-1]), dtype=dtype)
    for u in range(g.nv):
        out[g.toff[u]:g.toff[u + 1]] = ts[u].ravel()
    return out


def spin_ice_tensors(g: Graph, dtype=np.float64):
    """T[i, j, k, l] = 1 if i + j + k + l == 2 (test_beliefpropagation.jl:16-36)."""
    out = np.zeros(int(g.toff[-1]), dtype=dtype)
    for u in range(g.nv):
        dims = g.legs(u)
        T = np.zeros(dims, dtype=dtype)
        for idx in itertools.product(*[range(d) for d in dims]):
            if sum(idx) == 2:
                T[idx] = 1
        out[g.toff[u]:g.toff[u + 1]] = T.ravel()
    return out


def f_1d_ising(beta, N, J=1.0, h=0.0, periodic=True):
    """Free-energy density of the N-site Ising chain (test/utils.jl:12-39)."""
    if periodic:
        r = np.sqrt(np.sinh(beta * h) ** 2 + np.exp(-4 * beta * J))
        lp = np.exp(beta * J) * (np.cosh(beta * h) + r)
        lm = np.exp(beta * J) * (np.cosh(beta * h) - r)
        Z = lp ** N + lm ** N
        return -(np.log(Z) / (beta * N))
    if N == 1:
        return 2 * np.cosh(beta * h)
    T = np.array([[np.exp(beta * (J + h)), np.exp(-beta * J)],
                  [np.exp(-beta * J), np.exp(beta * (J - h))]])
    b = np.array([np.exp(beta * h / 2), np.exp(-beta * h / 2)])
    Z = b @ np.linalg.matrix_power(T, N - 1) @ b
    return -(np.log(Z) / (beta * N))


def beta_c_2d_ising():
    return np.log(1 + np.sqrt(2)) / 2


def f_2d_ising(beta, J=1.0, npts=20001):
    """Onsager free energy density (test/utils.jl:6-11), integral by Simpson's rule."""
    k = 2 * np.sinh(2 * beta * J) / np.cosh(2 * beta * J) ** 2
    th = np.linspace(0, np.pi, npts)
    y = np.log((1 + np.sqrt(np.abs(1 - (k * np.sin(th)) ** 2))) / 2)
    h = th[1] - th[0]
    integral = h / 3 * (y[0] + y[-1] + 4 * y[1:-1:2].sum() + 2 * y[2:-1:2].sum())
    return (-np.log(2 * np.cosh(2 * beta * J)) - integral / (2 * np.pi)) / beta
