"""Array-level engine over the C ABI: one device context per network.

``BPEngine`` holds a network (``graphs.Graph``), its site tensors and its messages on
the GPU and exposes the hot-path operations with the reference's semantics:
``run`` = beliefpropagation (beliefpropagation.jl:69-92), ``message_update`` =
message_update! (:242-257), ``logscalars`` / ``bethe_free_energy`` =
messagecache.jl:139-201, ``iterate_diff`` = beliefpropagation.jl:261-267.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .graphs import Graph

_PREC = {"native": L.PREC_NATIVE, "bf16": L.PREC_BF16, "tf32": L.PREC_TF32, "tf32x3": L.PREC_TF32X3}


@dataclass
class RunResult:
    iterations: int
    at_iteration: int
    delta: float
    device_ms: float
    kernel_launches: int


class BPEngine:
    def __init__(self, graph: Graph, device: int = 0):
        self.lib = L.load()
        self.graph = graph
        self._ctx = ctypes.c_void_p()
        st = self.lib.itn_create(ctypes.byref(self._ctx), int(device), 0)
        if st != L.ITN_OK:
            raise L.ItnError(st, f"itn_create failed: {self.lib.itn_status_string(st).decode()}")
        self._keep = []
        self.dtype = None
        g = graph
        self._off = np.ascontiguousarray(g.off, dtype=np.int64)
        self._nbr = np.ascontiguousarray(g.nbr, dtype=np.int64)
        self._bond = np.ascontiguousarray(g.bond, dtype=np.int32)
        self._rev = np.ascontiguousarray(g.rev, dtype=np.int64)
        self._phys = np.ascontiguousarray(g.phys, dtype=np.int32)
        self._net = np.ascontiguousarray(g.net, dtype=np.int32)
        self._check(self.lib.itn_graph_upload(
            self._ctx, g.nv, L.ptr(self._off), L.ptr(self._nbr), L.ptr(self._bond),
            L.ptr(self._rev), L.ptr(self._phys), int(g.layers), L.ptr(self._net)))
        self.n_undirected = int(np.sum(np.arange(g.nslots) < g.rev))

    # -- life cycle ---------------------------------------------------------------------
    def close(self):
        if self._ctx:
            self.lib.itn_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        L.check(self._ctx, st)

    # -- data ---------------------------------------------------------------------------
    def set_tensors(self, packed: np.ndarray):
        a = np.ascontiguousarray(packed)
        if a.size != int(self.graph.toff[-1]):
            raise ValueError("packed tensor size does not match the network")
        code = L.DTYPE_CODE[a.dtype]
        self._check(self.lib.itn_tensors_upload(self._ctx, code, L.ptr(a)))
        self.dtype = a.dtype

    def set_tensors_strided(self, arrays, strides, dtype):
        """arrays[u]: any ndarray whose elements are addressed by ``strides`` (element
        strides per canonical axis, flattened in vertex order)."""
        dt = np.dtype(dtype)
        arrs = [np.asarray(a, dtype=dt) for a in arrays]
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        st = np.ascontiguousarray(strides, dtype=np.int64)
        self._check(self.lib.itn_tensors_upload_strided(self._ctx, L.DTYPE_CODE[dt], ptrs, L.ptr(st)))
        self.dtype = dt

    def tensors(self) -> np.ndarray:
        out = np.empty(int(self.graph.toff[-1]), dtype=self.dtype)
        self._check(self.lib.itn_tensors_download(self._ctx, L.DTYPE_CODE[self.dtype], L.ptr(out)))
        return out

    def set_messages(self, packed: np.ndarray):
        a = np.ascontiguousarray(packed, dtype=self.dtype)
        if a.size != int(self.graph.moff[-1]):
            raise ValueError("packed message size does not match the network")
        self._check(self.lib.itn_messages_upload(self._ctx, L.DTYPE_CODE[self.dtype], L.ptr(a)))

    def init_messages(self, kind: str = "identity_normalized"):
        k = {"identity_normalized": L.MSG_IDENTITY_NORMALIZED, "identity": L.MSG_IDENTITY,
             "ones": L.MSG_ONES}[kind]
        self._check(self.lib.itn_messages_init(self._ctx, k))

    def messages(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(int(self.graph.moff[-1]), dtype=self.dtype)
        self._check(self.lib.itn_messages_download(self._ctx, L.DTYPE_CODE[self.dtype], L.ptr(out)))
        return out

    # -- hot path ------------------------------------------------------------------------
    def _opts(self, schedule, edges, maxiter, tol, normalize, precision, split_sweeps):
        o = L.BpOpts()
        o.schedule = {"parallel": L.SCHED_PARALLEL, "sequential": L.SCHED_SEQUENTIAL}[schedule]
        o.maxiter = -1 if maxiter is None else int(maxiter)
        o.tol = -1.0 if tol is None else float(tol)
        o.normalize = int(bool(normalize))
        o.precision = _PREC[precision]
        o.split_sweeps = int(split_sweeps)
        ed = None
        if edges is not None:
            ed = np.ascontiguousarray(edges, dtype=np.int64)
            o.edges = ed.ctypes.data
            o.n_edges = len(ed)
        return o, ed

    def solve(self, tensors: np.ndarray, messages: np.ndarray, *, messages_out: np.ndarray | None = None,
              logz: bool = True, schedule="parallel", edges=None, maxiter=None, tol=None, normalize=True,
              precision="native", split_sweeps=0):
        """Upload, solve, log-norm and download in one call with one host synchronisation
        (itn_bp_solve).  Returns (RunResult, log-norm or None, messages)."""
        t = np.ascontiguousarray(tensors)
        m = np.ascontiguousarray(messages, dtype=t.dtype)
        if t.size != int(self.graph.toff[-1]) or m.size != int(self.graph.moff[-1]):
            raise ValueError("packed tensor or message size does not match the network")
        out = messages_out if messages_out is not None else np.empty(int(self.graph.moff[-1]), dtype=t.dtype)
        if out.dtype != t.dtype or out.size != m.size or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("messages_out must be a contiguous array of the network's message size and dtype")
        o, _keep = self._opts(schedule, edges, maxiter, tol, normalize, precision, split_sweeps)
        r = L.BpResult()
        nn = self.graph.n_nets
        tot = np.empty((nn, 2)) if logz else None
        fl = np.empty(nn, dtype=np.int32) if logz else None
        self._check(self.lib.itn_bp_solve(self._ctx, L.DTYPE_CODE[t.dtype], L.ptr(t), L.ptr(m), ctypes.byref(o),
                                          ctypes.byref(r), L.ptr(out), L.ptr(tot), L.ptr(fl)))
        self.dtype = t.dtype
        res = RunResult(r.iterations, r.at_iteration, r.delta, r.device_ms, r.kernel_launches)
        return res, (self._bethe(tot, fl) if logz else None), out

    def solve_submit(self, tensors: np.ndarray, messages: np.ndarray, *, messages_out: np.ndarray | None = None,
                     logz: bool = True, schedule="parallel", edges=None, maxiter=None, tol=None, normalize=True,
                     precision="native", split_sweeps=0) -> None:
        """Queue what `solve` does and return without waiting (itn_bp_solve_submit); `solve_wait`
        returns its (RunResult, log-norm or None, messages).  The arrays are kept alive until
        then.  With two engines on one device, the uploads of one network overlap the solve of
        the other."""
        t = np.ascontiguousarray(tensors)
        m = np.ascontiguousarray(messages, dtype=t.dtype)
        if t.size != int(self.graph.toff[-1]) or m.size != int(self.graph.moff[-1]):
            raise ValueError("packed tensor or message size does not match the network")
        out = messages_out if messages_out is not None else np.empty(int(self.graph.moff[-1]), dtype=t.dtype)
        if out.dtype != t.dtype or out.size != m.size or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("messages_out must be a contiguous array of the network's message size and dtype")
        o, keep = self._opts(schedule, edges, maxiter, tol, normalize, precision, split_sweeps)
        self._check(self.lib.itn_bp_solve_submit(self._ctx, L.DTYPE_CODE[t.dtype], L.ptr(t), L.ptr(m),
                                                 ctypes.byref(o), L.ptr(out), 1 if logz else 0))
        self.dtype = t.dtype
        self._submitted = (t, m, out, o, keep, logz)

    def solve_wait(self):
        """Wait for the solve queued by `solve_submit` (itn_bp_solve_wait)."""
        sub = getattr(self, "_submitted", None)
        if sub is None:
            raise RuntimeError("no solve was submitted")
        out, logz = sub[2], sub[5]
        r = L.BpResult()
        nn = self.graph.n_nets
        tot = np.empty((nn, 2)) if logz else None
        fl = np.empty(nn, dtype=np.int32) if logz else None
        self._submitted = None
        self._check(self.lib.itn_bp_solve_wait(self._ctx, ctypes.byref(r), L.ptr(tot), L.ptr(fl)))
        res = RunResult(r.iterations, r.at_iteration, r.delta, r.device_ms, r.kernel_launches)
        return res, (self._bethe(tot, fl) if logz else None), out

    def run(self, *, schedule="parallel", edges=None, maxiter=None, tol=None, normalize=True,
            precision="native", split_sweeps=0) -> RunResult:
        o, _keep = self._opts(schedule, edges, maxiter, tol, normalize, precision, split_sweeps)
        r = L.BpResult()
        self._check(self.lib.itn_bp_run(self._ctx, ctypes.byref(o), ctypes.byref(r)))
        return RunResult(r.iterations, r.at_iteration, r.delta, r.device_ms, r.kernel_launches)

    def message_update(self, slot: int, normalize: bool = True):
        self._check(self.lib.itn_message_update(self._ctx, int(slot), int(bool(normalize))))

    def iterate_diff(self, m1, m2) -> float:
        a = np.ascontiguousarray(m1)
        b = np.ascontiguousarray(m2, dtype=a.dtype)
        out = ctypes.c_double()
        self._check(self.lib.itn_iterate_diff(self._ctx, L.DTYPE_CODE[a.dtype], L.ptr(a), L.ptr(b),
                                              ctypes.byref(out)))
        return out.value

    def grad(self, *, adjoint=True, maxiter=200, tol=1e-10, normalized=True, sweeps=0, checkpoint=1):
        """Gradient of bethe_free_energy w.r.t. every site tensor; returns (packed gradient,
        info dict).  sweeps == 0: at the current (converged) messages, with the implicit
        adjoint correction when ``adjoint``.  sweeps > 0: runs that many parallel sweeps
        from the current messages and differentiates through them exactly, keeping every
        ``checkpoint``-th sweep's messages (the others are recomputed)."""
        o = L.GradOpts(int(bool(adjoint)), int(maxiter), float(tol), int(bool(normalized)), int(sweeps),
                       int(checkpoint), 0)
        r = L.GradResult()
        out = np.empty(int(self.graph.toff[-1]), dtype=self.dtype)
        self._check(self.lib.itn_bp_grad(self._ctx, ctypes.byref(o), L.ptr(out), ctypes.byref(r)))
        return out, dict(adjoint_iterations=r.adjoint_iterations, adjoint_residual=r.adjoint_residual,
                         device_ms=r.device_ms)

    def sweep_vjp(self, cot_out, normalized=True) -> np.ndarray:
        """J^T cot_out for one parallel sweep at the current messages."""
        a = np.ascontiguousarray(cot_out, dtype=self.dtype)
        out = np.empty_like(a)
        self._check(self.lib.itn_sweep_vjp(self._ctx, int(bool(normalized)), L.ptr(a), L.ptr(out)))
        return out

    def inject_fault(self, kind: str, value: int):
        """Test hook (itn_inject_fault): ``"wait_ns"`` sets the elapsed-time limit of the
        persistent launches' device waits (the tensor-core sweep's waits on other items'
        messages, the grid barriers; <= 0: the default); ``"stall"`` (1 / 0) makes one such
        wait look for a message or arrival that never comes; ``"alloc"``
        makes the next ``value`` device allocations on this thread fail;
        ``"no_persistent_adjoint"`` (1 / 0) runs the gradient's adjoint iteration as one launch
        per iteration instead of one persistent launch; ``"no_persistent_sweeps"`` (1 / 0) the
        same for the CUDA-core parallel sweeps of small networks."""
        k = {"wait_ns": L.FAULT_WAIT_NS, "alloc": L.FAULT_ALLOC, "stall": L.FAULT_STALL,
             "no_persistent_adjoint": L.FAULT_NO_PERSISTENT_ADJOINT,
             "no_persistent_sweeps": L.FAULT_NO_PERSISTENT_SWEEPS}[kind]
        self._check(self.lib.itn_inject_fault(self._ctx, k, int(value)))

    def tc_selftest(self) -> dict:
        """Run the one-CTA tcgen05 self-test (exact BF16 products, M=64 lane map)."""
        a = ctypes.c_int32()
        b = ctypes.c_int32()
        err = ctypes.c_double()
        lanes = np.empty(64, dtype=np.int32)
        self._check(self.lib.itn_tc_selftest(self._ctx, ctypes.byref(a), ctypes.byref(b),
                                             ctypes.byref(err), L.ptr(lanes)))
        return dict(m128_ok=bool(a.value), m64_ok=bool(b.value), max_err=err.value,
                    lane_of_row=lanes)

    def logscalars(self) -> dict:
        g = self.graph
        nn = g.n_nets
        zv = np.empty(g.nv, dtype=self.dtype)
        ze = np.empty(self.n_undirected, dtype=self.dtype)
        lzv = np.empty((g.nv, 2))
        lze = np.empty((self.n_undirected, 2))
        tot = np.empty((nn, 2))
        fl = np.empty(nn, dtype=np.int32)
        self._check(self.lib.itn_logscalars(self._ctx, L.ptr(zv), L.ptr(ze), L.ptr(lzv), L.ptr(lze),
                                            L.ptr(tot), L.ptr(fl)))
        return dict(zv=zv, ze=ze, logzv=lzv, logze=lze, totals=tot, flags=fl)

    def bethe_free_energy(self, net: int | None = None):
        """bethe_free_energy (messagecache.jl:185-201) of one network (or a list for all)."""
        nn = self.graph.n_nets
        tot = np.empty((nn, 2))
        fl = np.empty(nn, dtype=np.int32)
        # only the per-network totals and flags are read back
        self._check(self.lib.itn_logscalars(self._ctx, None, None, None, None, L.ptr(tot), L.ptr(fl)))
        return self._bethe(tot, fl, net)

    def _bethe(self, tot, fl, net=None):
        """bethe_free_energy from the per-network totals and flags of itn_logscalars."""
        nn = self.graph.n_nets
        r = dict(totals=tot, flags=fl)
        out = []
        for k in range(nn):
            f = int(r["flags"][k])
            if f & 4:
                out.append(-np.inf)
                continue
            re, im = r["totals"][k]
            cplx = np.iscomplexobj(np.empty(0, self.dtype)) or bool(f & 1) or bool(f & 2)
            out.append(complex(re, im) if cplx else float(re))
        return out if net is None and len(out) != 1 else out[0 if net is None else net]
