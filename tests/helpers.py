"""Shared helpers for the tests (fixture loading, error metrics)."""
import os

import numpy as np

from itn_gb300 import graphs as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name)))
    g = G.Graph(int(len(d["off"]) - 1), d["off"], d["nbr"], d["bond"], d["rev"], d["phys"],
                int(d["layers"]))
    return g, d


def max_rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def msg_rel(g, a, b):
    """Largest per-message relative error (each message measured in its own scale)."""
    worst = 0.0
    for s in range(g.nslots):
        x = a[g.moff[s]:g.moff[s + 1]]
        y = b[g.moff[s]:g.moff[s + 1]]
        worst = max(worst, float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300)))
    return worst


# ---- small states for the gate-application tests --------------------------------------------
def rand_psd(rng, n, dtype):
    """Random Hermitian positive definite n x n matrix (an environment message)."""
    b = rng.standard_normal((n, n))
    if np.dtype(dtype).kind == "c":
        b = b + 1j * rng.standard_normal((n, n))
    return (b @ np.conj(b).T + 0.1 * np.eye(n)).astype(dtype)


def _randn(rng, shape, dtype):
    a = rng.standard_normal(shape)
    if np.dtype(dtype).kind == "c":
        a = a + 1j * rng.standard_normal(shape)
    return a.astype(dtype)


def random_cycle4(rng, dtype, d=3, bonds=(2, 3, 2, 3)):
    """4-cycle with bonds a(3-0), b(0-1), c(1-2), d(2-3): T0[a,b,s], T1[b,c,s], T2[c,d,s], T3[d,a,s]."""
    a, b, c, dd = bonds
    return [_randn(rng, (a, b, d), dtype), _randn(rng, (b, c, d), dtype),
            _randn(rng, (c, dd, d), dtype), _randn(rng, (dd, a, d), dtype)]


def cycle4_state(T):
    return np.einsum("abw,bcx,cdy,daz->wxyz", *T)


def random_path4(rng, dtype, d=3, bonds=(3, 4, 3)):
    """Path 0-1-2-3 with bonds b(0-1), c(1-2), d(2-3): T0[s,b], T1[b,c,s], T2[c,d,s], T3[d,s]."""
    b, c, dd = bonds
    return [_randn(rng, (d, b), dtype), _randn(rng, (b, c, d), dtype),
            _randn(rng, (c, dd, d), dtype), _randn(rng, (dd, d), dtype)]


def path4_state(T):
    return np.einsum("wb,bcx,cdy,dz->wxyz", *T)


def path_envs(T):
    """Exact environments (bra, ket) of the legs b (edge 0 -> 1) and d (edge 3 -> 2)."""
    eb = np.einsum("sb,sk->bk", np.conj(T[0]), T[0])
    ed = np.einsum("bs,ks->bk", np.conj(T[3]), T[3])
    return eb, ed
