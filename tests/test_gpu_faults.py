"""Failure detection without faulting the GPU.

* A persistent tensor-core sweep in which one wait looks for a message that nothing writes
  (the stall fault), with the wait limit cut to 1 ms, gives up: every group stops early,
  waits for its own copies, frees its tensor memory and the call returns ITN_ERR_TIMEOUT.
  The same context then solves the network again without the fault and matches a fresh
  solve bit for bit (the GPU and the context stayed usable).
* The same for the persistent CUDA-core sweep of a small network: one CTA never arrives at
  the first grid barrier, the others' waits run out after 1 ms and the call returns
  ITN_ERR_TIMEOUT; the context then solves again bit for bit.
* A device allocation failure forced on the host makes the call that allocates return
  ITN_ERR_OOM; the context recovers once allocations succeed again.
"""
import numpy as np
import pytest

from itn_gb300 import BPEngine, ItnError
from itn_gb300 import _lib as L
from itn_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib_built):
    return lib_built


def _lattice(L_, seed=5):
    g = G.square_lattice(L_, L_, 8, periodic=True, phys=2)
    t = G.random_tensors(g, np.random.default_rng(seed), np.float64, G.peps_scale(g)).astype(np.float32)
    return g, t


def test_tensor_core_wait_that_runs_out_reports_timeout():
    g, t = _lattice(32)
    with BPEngine(g) as ref:
        ref.set_tensors(t)
        ref.init_messages()
        ref.run(maxiter=12, precision="bf16", split_sweeps=2)
        want = ref.messages()
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.inject_fault("wait_ns", 1_000_000)
        e.inject_fault("stall", 1)
        e.init_messages()
        with pytest.raises(ItnError) as ei:
            e.run(maxiter=12, precision="bf16", split_sweeps=2)
        assert ei.value.status == L.ITN_ERR_TIMEOUT
        assert "bounded device wait" in str(ei.value)
        # no fault, default limit: the same context solves the network again
        e.inject_fault("stall", 0)
        e.inject_fault("wait_ns", 0)
        e.init_messages()
        r = e.run(maxiter=12, precision="bf16", split_sweeps=2)
        assert r.iterations == 12
        np.testing.assert_array_equal(e.messages(), want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_persistent_sweep_barrier_that_runs_out_reports_timeout(dtype):
    g = G.square_lattice(12, 12, 4, periodic=False, phys=2)
    t = G.random_tensors(g, np.random.default_rng(9), dtype, G.peps_scale(g))
    with BPEngine(g) as ref:
        ref.set_tensors(t)
        ref.init_messages()
        ref.run(maxiter=40, tol=1e-10)
        want = ref.messages()
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.inject_fault("wait_ns", 1_000_000)
        e.inject_fault("stall", 1)
        e.init_messages()
        with pytest.raises(ItnError) as ei:
            e.run(maxiter=40, tol=1e-10)
        assert ei.value.status == L.ITN_ERR_TIMEOUT
        assert "bounded device wait" in str(ei.value)
        e.init_messages()
        with pytest.raises(ItnError) as ei:  # without a tolerance: one chunk of 5 sweeps
            e.run(maxiter=5)
        assert ei.value.status == L.ITN_ERR_TIMEOUT
        e.inject_fault("stall", 0)
        e.inject_fault("wait_ns", 0)
        e.init_messages()
        r = e.run(maxiter=40, tol=1e-10)
        assert 1 < r.iterations < 40
        np.testing.assert_array_equal(e.messages(), want)


def test_forced_allocation_failure_reports_oom_and_recovers():
    g, t = _lattice(4)
    t64 = t.astype(np.float64)
    with BPEngine(g) as ref:
        ref.set_tensors(t64)
        ref.init_messages()
        ref.run(maxiter=3)
        want = ref.messages()
    with BPEngine(g) as e:
        e.inject_fault("alloc", 1)
        with pytest.raises(ItnError) as ei:
            e.set_tensors(t64)  # the tensor buffer is the first allocation: it fails
        assert ei.value.status == L.ITN_ERR_OOM
        # the failed upload left no tensors behind: a solve is refused, not run on stale data
        with pytest.raises(ItnError) as ei2:
            e.init_messages()
        assert ei2.value.status == L.ITN_ERR_STATE
        e.set_tensors(t64)  # allocations succeed again
        e.init_messages()
        e.run(maxiter=3)
        np.testing.assert_array_equal(e.messages(), want)
