"""BP simple-update gate application on the GPU (src/apply/apply_operators.jl:209-283).

Array-level batch interface over ``itn_apply_gates``: every gate of a batch runs in its own
CTA, so one call applies a whole layer of gates on disjoint sites.

A one-site gate is ``Gate(sites=[psi], envs=[[M_0, ...]], op=op)`` with psi an array
[other legs..., s] and op[s', s]; a two-site gate is ``Gate(sites=[psi1, psi2],
envs=[envs1, envs2], op=op)`` with psi_i [other legs..., s_i, b] (b the bond joining the
two sites, last axis of both) and op[s1', s2', s1, s2].  envs_i holds one D x D
environment message M[bra, ket] per other leg (None: no gauge on that leg).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .contract import Context


@dataclass
class Gate:
    sites: list
    envs: list
    op: np.ndarray
    extra: dict = field(default_factory=dict)


def _chi_cap(g: Gate):
    if len(g.sites) == 1:
        return 1
    caps = []
    for psi in g.sites:
        p = int(np.prod(psi.shape[:-2], dtype=np.int64))
        d, b = psi.shape[-2], psi.shape[-1]
        caps.append(d * min(p, d * b))
    return min(caps)


def apply_gates(gates, *, max_rank=None, cutoff=None, normalize=False, context=None, return_time=False):
    """Apply a batch of gates.  Returns a list with, per gate, the new site array (one-site)
    or (new psi1 [others..., s1, c], new psi2 [others..., s2, c], S) (two-site);
    ``return_time`` adds the device time in ms."""
    gates = list(gates)
    if not gates:
        return ([], 0.0) if return_time else []
    arrays = []
    for g in gates:
        arrays += list(g.sites) + [g.op] + [m for es in g.envs for m in es if m is not None]
    dt = np.result_type(*[np.asarray(a).dtype for a in arrays])
    if dt.kind == "c":
        dt = np.dtype(np.complex64) if dt == np.complex64 else np.dtype(np.complex128)
    elif dt == np.float32:
        dt = np.dtype(np.float32)
    else:
        dt = np.dtype(np.float64)
    site_parts, env_parts, op_parts = [], [], []
    n_site = n_env = n_op = n_out = n_s = 0
    descs = (L.GateDesc * len(gates))()
    caps = []
    for k, g in enumerate(gates):
        ns = len(g.sites)
        if ns not in (1, 2) or len(g.envs) != ns:
            raise L.ItnArgumentError(L.ITN_ERR_ARG, "a gate acts on one or two sites with one env list per site")
        D = descs[k]
        D.nsite = ns
        cap = _chi_cap(g)
        caps.append(cap)
        for i, psi in enumerate(g.sites):
            psi = np.ascontiguousarray(np.asarray(psi, dtype=dt))
            others = psi.shape[:-2] if ns == 2 else psi.shape[:-1]
            D.d[i] = psi.shape[-2] if ns == 2 else psi.shape[-1]
            D.nleg[i] = len(others)
            if len(others) > 6:
                raise L.ItnArgumentError(L.ITN_ERR_UNSUPPORTED, "at most 6 other legs per site")
            if len(g.envs[i]) != len(others):
                raise L.ItnArgumentError(L.ITN_ERR_ARG, "one environment (or None) per other leg")
            for j, dim in enumerate(others):
                D.leg_dim[i][j] = int(dim)
                m = g.envs[i][j]
                if m is None:
                    D.env_off[i][j] = -1
                else:
                    m = np.ascontiguousarray(np.asarray(m, dtype=dt))
                    if m.shape != (dim, dim):
                        raise L.ItnArgumentError(L.ITN_ERR_ARG, "environment shape does not match its leg")
                    D.env_off[i][j] = n_env
                    env_parts.append(m.ravel())
                    n_env += m.size
            D.site_off[i] = n_site
            site_parts.append(psi.ravel())
            n_site += psi.size
            p = int(np.prod(others, dtype=np.int64))
            D.out_off[i] = n_out
            n_out += p * int(D.d[i]) * cap
        if ns == 2:
            b0, b1 = g.sites[0].shape[-1], g.sites[1].shape[-1]
            if b0 != b1:
                raise L.ItnArgumentError(L.ITN_ERR_ARG, "the two sites disagree on the shared bond dimension")
            D.bond = int(b0)
            D.s_off = n_s
            n_s += cap
        op = np.ascontiguousarray(np.asarray(g.op, dtype=dt))
        D.op_off = n_op
        op_parts.append(op.ravel())
        n_op += op.size
    sites = np.concatenate(site_parts)
    envs = np.concatenate(env_parts) if env_parts else np.zeros(1, dtype=dt)
    ops = np.concatenate(op_parts)
    out = np.zeros(max(n_out, 1), dtype=dt)
    s_out = np.zeros(max(n_s, 1), dtype=np.float64)
    bonds = np.zeros(len(gates), dtype=np.int32)
    ms = ctypes.c_double(0.0)
    own = context is None
    ctx = Context() if own else context
    try:
        st = ctx.lib.itn_apply_gates(ctx.ctx, L.DTYPE_CODE[dt], len(gates), descs, L.ptr(sites), sites.size,
                                     L.ptr(envs), n_env, L.ptr(ops), ops.size,
                                     int(max_rank) if max_rank else 0, float(cutoff) if cutoff else 0.0,
                                     1 if normalize else 0, L.ptr(out), out.size, L.ptr(s_out), s_out.size,
                                     L.ptr(bonds), ctypes.byref(ms))
        if st != L.ITN_OK:
            L.check(ctx.ctx, st)
    finally:
        if own:
            ctx.close()
    res = []
    for k, g in enumerate(gates):
        D = descs[k]
        if len(g.sites) == 1:
            shape = g.sites[0].shape
            res.append(out[D.out_off[0]:D.out_off[0] + int(np.prod(shape))].reshape(shape).copy())
            continue
        chi = int(bonds[k])
        pair = []
        for i, psi in enumerate(g.sites):
            others = psi.shape[:-2]
            shape = tuple(others) + (psi.shape[-2], chi)
            size = int(np.prod(shape))
            pair.append(out[D.out_off[i]:D.out_off[i] + size].reshape(shape).copy())
        res.append((pair[0], pair[1], s_out[D.s_off:D.s_off + chi].copy()))
    return (res, ms.value) if return_time else res
