"""contract_network on the GPU (src/contract_network.jl:7-58 of ITensorNetworksNext.jl).

``contract_network(tensors, labels; alg, precision)`` contracts a list of tensors whose
axes carry labels (any hashable): a label on two tensors is summed over, a label on one
tensor stays open.  The pairwise order is chosen by the library's C++ greedy rule (or
left-associative, or "sweep": the cheaper of the greedy order and running-product sweeps, or an
explicit step list); every pairwise step runs on the device as a permute + GEMM (CUDA cores, or
tcgen05 with BF16 / TF32 hi/lo split operands for float32).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .graphs import Graph

_ALG = {"greedy": 0, "left": 1, "sweep": 3}
_PREC = {"native": L.PREC_NATIVE, "bf16": L.PREC_BF16, "tf32x3": L.PREC_TF32X3}


class Context:
    """A bare device context (stream + buffers) for calls that need no network upload."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        self.ctx = ctypes.c_void_p()
        st = self.lib.itn_create(ctypes.byref(self.ctx), int(device), 0)
        if st != L.ITN_OK:
            raise L.ItnError(st, f"itn_create failed: {self.lib.itn_status_string(st).decode()}")

    def close(self):
        if self.ctx:
            self.lib.itn_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _flatten(tensors, labels):
    ids = {}
    ranks, lab, dims = [], [], []
    for t, ls in zip(tensors, labels):
        if np.ndim(t) != len(ls):
            raise ValueError("each tensor needs one label per axis")
        ranks.append(len(ls))
        for x, d in zip(ls, np.shape(t)):
            lab.append(ids.setdefault(x, len(ids)))
            dims.append(int(d))
    inv = {v: k for k, v in ids.items()}
    return (np.asarray(ranks, dtype=np.int32), np.asarray(lab, dtype=np.int64),
            np.asarray(dims, dtype=np.int64), inv)


def contraction_order(shapes, labels, alg="greedy"):
    """The library's pairwise order (host computation, no GPU): a list of (i, j) steps on a
    working list that drops both and appends the result (labels free(i) ++ free(j))."""
    lib = L.load()
    ranks, lab, dims, _ = _flatten([np.empty(s, dtype=np.int8) for s in shapes], labels)
    n = len(shapes)
    steps = np.zeros(max(2 * (n - 1), 1), dtype=np.int32)
    st = lib.itn_contraction_order(n, L.ptr(ranks), L.ptr(lab), L.ptr(dims), _ALG[alg], L.ptr(steps))
    if st != L.ITN_OK:
        raise L.ItnArgumentError(st, "itn_contraction_order rejected the network")
    return [(int(steps[2 * k]), int(steps[2 * k + 1])) for k in range(n - 1)]


def contract_network(tensors, labels, *, alg="greedy", steps=None, precision="native", context=None,
                     return_time=False):
    """Exact contraction; returns (array, open_labels) [, device_ms]."""
    ts = [np.ascontiguousarray(t) for t in tensors]
    dt = np.result_type(*[t.dtype for t in ts])
    if dt not in L.DTYPE_CODE:
        dt = np.dtype(np.complex128) if dt.kind == "c" else np.dtype(np.float64)
    ts = [np.ascontiguousarray(t, dtype=dt) for t in ts]
    ranks, lab, dims, inv = _flatten(ts, labels)
    ctx = context or Context()
    try:
        ptrs = (ctypes.c_void_p * len(ts))(*[t.ctypes.data for t in ts])
        if steps is not None:
            a = 2
            st_arr = np.asarray(steps, dtype=np.int32).ravel()
        else:
            a = _ALG[alg]
            st_arr = None
        # open labels: those appearing once
        from collections import Counter
        cnt = Counter(lab.tolist())
        size = int(np.prod([d for x, d in zip(lab, dims) if cnt[int(x)] == 1], dtype=np.int64))
        out = np.empty(max(size, 1), dtype=dt)
        rank = ctypes.c_int32()
        olab = np.zeros(48, dtype=np.int64)
        odim = np.zeros(48, dtype=np.int64)
        ms = ctypes.c_double()
        stt = ctx.lib.itn_contract_network(
            ctx.ctx, L.DTYPE_CODE[dt], len(ts), L.ptr(ranks), L.ptr(lab), L.ptr(dims), ptrs, a,
            L.ptr(st_arr), _PREC[precision], L.ptr(out), out.size, ctypes.byref(rank), L.ptr(olab),
            L.ptr(odim), ctypes.byref(ms))
        L.check(ctx.ctx, stt)
    finally:
        if context is None:
            ctx.close()
    r = rank.value
    res = out[:size].reshape(tuple(int(d) for d in odim[:r]))
    labels_out = [inv[int(x)] for x in olab[:r]]
    return (res, labels_out, ms.value) if return_time else (res, labels_out)


def norm_network_tensors(g: Graph, packed):
    """<psi|psi> as a tensor list (NormNetwork, normnetwork.jl:49-54): ket A_u with (site,
    ket links), conj(A_u) with (site, bra links); links named by undirected edge."""
    ts, ls = [], []
    for u in range(g.nv):
        A = np.asarray(packed[g.toff[u]:g.toff[u + 1]]).reshape(g.tensor_shape(u))
        legs = [int(min(s, g.rev[s])) for s in range(g.off[u], g.off[u + 1])]
        ts.append(A)
        ls.append([("s", u)] + [("k", e) for e in legs])
        ts.append(np.conj(A))
        ls.append([("s", u)] + [("b", e) for e in legs])
    return ts, ls


def plain_network_tensors(g: Graph, packed):
    """A single-layer network (a partition function such as ising_network / delta_network)
    as a tensor list: tensor u with its links named by undirected edge, the site index
    (when phys > 1) left open."""
    ts, ls = [], []
    for u in range(g.nv):
        A = np.asarray(packed[g.toff[u]:g.toff[u + 1]]).reshape(g.tensor_shape(u))
        legs = [("k", int(min(s, g.rev[s]))) for s in range(g.off[u], g.off[u + 1])]
        if A.shape[0] == 1:
            ts.append(A.reshape(A.shape[1:]))
            ls.append(legs)
        else:
            ts.append(A)
            ls.append([("s", u)] + legs)
    return ts, ls


def contract_plain_network(g: Graph, packed, **kw):
    """Exact contraction of a single-layer network (contract_network(tn),
    contract_network.jl:7-58); a scalar for a closed network."""
    ts, ls = plain_network_tensors(g, packed)
    out, lo = contract_network(ts, ls, **kw)[:2]
    return out[()] if not lo else (out, lo)


def contract_norm_network(g: Graph, packed, **kw):
    """Exact <psi|psi> of a PEPS given as a Graph + packed site tensors."""
    ts, ls = norm_network_tensors(g, packed)
    out, lo = contract_network(ts, ls, **kw)[:2]
    return out[()]
