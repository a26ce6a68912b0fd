"""Exact network contraction oracle (numpy).  TEST INFRASTRUCTURE ONLY.

Restates contract_network(tn; alg=Exact(order_alg)) (src/contract_network.jl:7-58):
an evaluation order is chosen (Greedy by default, LeftAssociative on request) and
the network is materialised by pairwise contractions.  The pairwise products are
numpy.tensordot here; in the reference they are ITensorBase/TensorAlgebra calls.

Tensors are given as (array, labels); equal labels on two tensors are contracted,
labels that occur once stay open (sorted by first appearance in the result).
"""
from __future__ import annotations

import numpy as np


def _contract_pair(a, la, b, lb):
    shared = [x for x in la if x in lb]
    ia = [la.index(x) for x in shared]
    ib = [lb.index(x) for x in shared]
    out = np.tensordot(a, b, axes=(ia, ib))
    lo = [x for x in la if x not in shared] + [x for x in lb if x not in shared]
    return out, lo


def contraction_order_greedy(shapes, labels):
    """Greedy pairwise order: repeatedly contract the pair whose result grows the
    network least (size(out) - size(a) - size(b)), preferring pairs that share labels.
    Returns a list of (i, j) positions in a working list that shrinks by one per step."""
    shapes = [tuple(s) for s in shapes]
    labels = [list(l) for l in labels]
    dims = {}
    for s, l in zip(shapes, labels):
        for d, x in zip(s, l):
            dims[x] = d
    order = []
    while len(labels) > 1:
        best = None
        n = len(labels)
        for i in range(n):
            for j in range(i + 1, n):
                shared = set(labels[i]) & set(labels[j])
                lo = [x for x in labels[i] if x not in shared] + \
                     [x for x in labels[j] if x not in shared]
                so = int(np.prod([dims[x] for x in lo], dtype=np.float64))
                sa = int(np.prod([dims[x] for x in labels[i]], dtype=np.float64))
                sb = int(np.prod([dims[x] for x in labels[j]], dtype=np.float64))
                key = (0 if shared else 1, so - sa - sb, so)
                if best is None or key < best[0]:
                    best = (key, i, j, lo)
        _, i, j, lo = best
        order.append((i, j))
        labels = [l for k, l in enumerate(labels) if k not in (i, j)] + [lo]
    return order


def contract_network(tensors, labels, order="greedy"):
    """Returns (array, open_labels).  ``order`` is "greedy", "left" (left-associative:
    ((t0*t1)*t2)*...) or an explicit list of (i, j) steps."""
    ts = [np.asarray(t) for t in tensors]
    ls = [list(l) for l in labels]
    if len(ts) == 0:
        raise ValueError("empty network")
    if order == "left":
        acc, lacc = ts[0], ls[0]
        for t, l in zip(ts[1:], ls[1:]):
            acc, lacc = _contract_pair(acc, lacc, t, l)
        return acc, lacc
    steps = contraction_order_greedy([t.shape for t in ts], ls) if order == "greedy" else order
    for i, j in steps:
        out, lo = _contract_pair(ts[i], ls[i], ts[j], ls[j])
        ts = [t for k, t in enumerate(ts) if k not in (i, j)] + [out]
        ls = [l for k, l in enumerate(ls) if k not in (i, j)] + [lo]
    return ts[0], ls[0]


def graph_tensors(g, packed):
    """Split packed site tensors into per-vertex arrays shaped [phys, legs...]."""
    out = []
    for u in range(g.nv):
        shp = (int(g.phys[u]),) + tuple(int(b) for b in g.bond[g.off[u]:g.off[u + 1]])
        out.append(np.asarray(packed[g.toff[u]:g.toff[u + 1]]).reshape(shp))
    return out


def _edge_id(g, s):
    return int(min(s, g.rev[s]))


def norm_network(g, packed):
    """The double-layer network <psi|psi> of NormNetwork (normnetwork.jl:49-54):
    ket A_u with (site, ket links) and conj(A_u) with (site, bra links); the site
    index is shared by ket and bra, link names differ between layers."""
    ts, ls = [], []
    for u, A in enumerate(graph_tensors(g, packed)):
        legs = [_edge_id(g, s) for s in range(g.off[u], g.off[u + 1])]
        ts.append(A)
        ls.append([("s", u)] + [("k", e) for e in legs])
        ts.append(np.conj(A))
        ls.append([("s", u)] + [("b", e) for e in legs])
    return ts, ls


def plain_network(g, packed):
    """Single-layer network (tensors contracted over shared links; site index open
    when phys > 1)."""
    ts, ls = [], []
    for u, A in enumerate(graph_tensors(g, packed)):
        legs = [_edge_id(g, s) for s in range(g.off[u], g.off[u + 1])]
        if A.shape[0] == 1:
            ts.append(A.reshape(A.shape[1:]))
            ls.append([("k", e) for e in legs])
        else:
            ts.append(A)
            ls.append([("s", u)] + [("k", e) for e in legs])
    return ts, ls


def contract_norm(g, packed, order="greedy"):
    ts, ls = norm_network(g, packed)
    out, lo = contract_network(ts, ls, order)
    assert not lo
    return out[()]


def contract_plain(g, packed, order="greedy"):
    ts, ls = plain_network(g, packed)
    out, lo = contract_network(ts, ls, order)
    return out, lo
