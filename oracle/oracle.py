"""CPU oracle for the belief-propagation / contract_network hot path.

TEST INFRASTRUCTURE ONLY.  The tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` import this module to compare against; the GPU library
(``libitn_gpu.so``) and the ``itn_gb300`` package never import, link or call it.

The BP arithmetic lives in ``bp_oracle.c`` (a C restatement of
src/beliefpropagation/beliefpropagation.jl and messagecache.jl, OpenMP over edges).
This module builds it with gcc and wraps it with ctypes.  ``contract_oracle.py`` holds
the exact-contraction restatement (numpy).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libbp_oracle.so")
_lock = threading.Lock()
_lib = None

_SUFFIX = {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32",
           np.dtype(np.complex128): "c128", np.dtype(np.complex64): "c64"}


def build(force: bool = False) -> str:
    """Compile bp_oracle.c into oracle/_build/libbp_oracle.so (gcc, OpenMP)."""
    os.makedirs(_BUILD, exist_ok=True)
    src = os.path.join(_HERE, "bp_oracle.c")
    hdr = os.path.join(_HERE, "bp_oracle_impl.h")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True, cwd=_HERE)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _Graph(ctypes.Structure):
    _fields_ = [("nv", ctypes.c_int64),
                ("off", ctypes.c_void_p), ("nbr", ctypes.c_void_p), ("rev", ctypes.c_void_p),
                ("toff", ctypes.c_void_p), ("moff", ctypes.c_void_p),
                ("bond", ctypes.c_void_p), ("phys", ctypes.c_void_p),
                ("layers", ctypes.c_int32), ("pad", ctypes.c_int32)]


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_LIB_PATH)
            for suf in ("f64", "f32", "c128", "c64"):
                f = getattr(lib, f"orc_bp_run_{suf}")
                f.restype = ctypes.c_int
                f.argtypes = [ctypes.POINTER(_Graph), ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                              ctypes.c_double, ctypes.c_int, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_int)]
                f = getattr(lib, f"orc_bp_sweeps_{suf}")
                f.restype = ctypes.c_int
                f.argtypes = [ctypes.POINTER(_Graph), ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int]
                f = getattr(lib, f"orc_message_update_{suf}")
                f.restype = ctypes.c_int
                f.argtypes = [ctypes.POINTER(_Graph), ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_int64, ctypes.c_int]
                f = getattr(lib, f"orc_iterate_diff_{suf}")
                f.restype = ctypes.c_double
                f.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
                f = getattr(lib, f"orc_logscalars_{suf}")
                f.restype = ctypes.c_int
                f.argtypes = [ctypes.POINTER(_Graph), ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            lib.orc_max_threads.restype = ctypes.c_int
            _lib = lib
    return _lib


def max_threads() -> int:
    return int(_load().orc_max_threads())


class OracleGraph:
    """Holds contiguous int arrays for the C struct (kept alive with it)."""

    def __init__(self, g):
        self.off = np.ascontiguousarray(g.off, dtype=np.int64)
        self.nbr = np.ascontiguousarray(g.nbr, dtype=np.int64)
        self.rev = np.ascontiguousarray(g.rev, dtype=np.int64)
        self.toff = np.ascontiguousarray(g.toff, dtype=np.int64)
        self.moff = np.ascontiguousarray(g.moff, dtype=np.int64)
        self.bond = np.ascontiguousarray(g.bond, dtype=np.int32)
        self.phys = np.ascontiguousarray(g.phys, dtype=np.int32)
        self.layers = int(g.layers)
        self.nv = int(g.nv)
        self.s = _Graph(self.nv, self.off.ctypes.data, self.nbr.ctypes.data,
                        self.rev.ctypes.data, self.toff.ctypes.data, self.moff.ctypes.data,
                        self.bond.ctypes.data, self.phys.ctypes.data, self.layers, 0)


def _suffix(arr):
    try:
        return _SUFFIX[arr.dtype]
    except KeyError:
        raise TypeError(f"unsupported dtype {arr.dtype}") from None


def bp_run(g, tensors, messages, *, schedule="parallel", edges=None, maxiter=None, tol=None,
           normalize=True, nthreads=0):
    """Run BP on a copy of ``messages``; returns (messages, iterations, delta, at_iteration).

    Mirrors beliefpropagation(factors, messages; edges, stopping_criterion=(; maxiter, tol)).
    """
    lib = _load()
    og = OracleGraph(g)
    t = np.ascontiguousarray(tensors)
    m = np.array(messages, dtype=t.dtype, copy=True, order="C")
    suf = _suffix(t)
    if schedule == "parallel":
        sch, ed, ne = 0, None, 0
    elif schedule == "sequential":
        if edges is None:
            raise ValueError("sequential schedule needs an explicit edge (slot) list")
        ed = np.ascontiguousarray(edges, dtype=np.int64)
        sch, ne = 1, len(ed)
    else:
        raise ValueError(schedule)
    it = ctypes.c_int()
    dl = ctypes.c_double()
    at = ctypes.c_int()
    st = getattr(lib, f"orc_bp_run_{suf}")(
        ctypes.byref(og.s), t.ctypes.data, m.ctypes.data, sch,
        None if ed is None else ed.ctypes.data, ne,
        -1 if maxiter is None else int(maxiter), -1.0 if tol is None else float(tol),
        int(bool(normalize)), int(nthreads), ctypes.byref(it), ctypes.byref(dl), ctypes.byref(at))
    if st:
        raise ValueError(f"oracle bp_run failed with status {st}")
    return m, it.value, dl.value, at.value


def bp_sweeps(g, tensors, messages, nsweeps, *, normalize=True, nthreads=0):
    """Fixed number of parallel sweeps, in place on ``messages`` (timed CPU baseline)."""
    lib = _load()
    og = OracleGraph(g)
    t = np.ascontiguousarray(tensors)
    assert messages.flags.c_contiguous and messages.dtype == t.dtype
    st = getattr(lib, f"orc_bp_sweeps_{_suffix(t)}")(
        ctypes.byref(og.s), t.ctypes.data, messages.ctypes.data, int(nsweeps),
        int(bool(normalize)), int(nthreads))
    if st:
        raise ValueError(f"oracle bp_sweeps failed with status {st}")
    return messages


def message_update(g, tensors, messages, slot, *, normalize=True):
    """In-place single-edge update (reference message_update!)."""
    lib = _load()
    og = OracleGraph(g)
    t = np.ascontiguousarray(tensors)
    assert messages.flags.c_contiguous and messages.dtype == t.dtype
    st = getattr(lib, f"orc_message_update_{_suffix(t)}")(
        ctypes.byref(og.s), t.ctypes.data, messages.ctypes.data, int(slot), int(bool(normalize)))
    if st:
        raise ValueError(f"oracle message_update failed with status {st}")
    return messages


def iterate_diff(moff, m1, m2):
    lib = _load()
    moff = np.ascontiguousarray(moff, dtype=np.int64)
    a = np.ascontiguousarray(m1)
    b = np.ascontiguousarray(m2, dtype=a.dtype)
    return float(getattr(lib, f"orc_iterate_diff_{_suffix(a)}")(
        len(moff) - 1, moff.ctypes.data, a.ctypes.data, b.ctypes.data))


def logscalars(g, tensors, messages):
    """Returns dict(zv, ze, logzv, logze, total, flags) following bethe_free_energy."""
    lib = _load()
    og = OracleGraph(g)
    t = np.ascontiguousarray(tensors)
    m = np.ascontiguousarray(messages, dtype=t.dtype)
    nv = og.nv
    ne = int(np.sum(np.arange(len(og.rev)) < og.rev))
    zv = np.zeros(nv, dtype=t.dtype)
    ze = np.zeros(ne, dtype=t.dtype)
    lzv = np.zeros((nv, 2))
    lze = np.zeros((ne, 2))
    tot = np.zeros(2)
    flags = np.zeros(3, dtype=np.int32)
    st = getattr(lib, f"orc_logscalars_{_suffix(t)}")(
        ctypes.byref(og.s), t.ctypes.data, m.ctypes.data, zv.ctypes.data, ze.ctypes.data,
        lzv.ctypes.data, lze.ctypes.data, tot.ctypes.data, flags.ctypes.data)
    if st:
        raise ValueError(f"oracle logscalars failed with status {st}")
    return dict(zv=zv, ze=ze, logzv=lzv, logze=lze, total=tot, flags=flags)


def bethe_free_energy(g, tensors, messages):
    """bethe_free_energy (messagecache.jl:185-201): real unless a promotion happened."""
    r = logscalars(g, tensors, messages)
    if r["flags"][2]:
        return -np.inf
    re, im = r["total"]
    cplx = np.iscomplexobj(tensors) or bool(r["flags"][0]) or bool(r["flags"][1])
    return complex(re, im) if cplx else float(re)
