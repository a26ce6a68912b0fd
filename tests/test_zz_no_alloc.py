"""itn_logz_static_scratch: the Bethe log-norm computed without any device allocation.

It serves callers whose GPU memory is owned by their own pooling allocator (a CUDA.jl
memory pool, a serving process that reserves HBM at start-up), where a cudaMalloc inside
the library would fail or bypass the pool.  The test hands it device buffers (allocated
here by torch, standing in for such a pool) and checks its result against the context
entry point itn_logscalars on two calls in a row -- the second call reuses the shared
static scratch left by the first -- and, in FP64, against the CPU oracle.  Tolerances as
elsewhere: 1e-10 relative in FP64, 2e-4 in FP32.  Collected last on purpose (file name) so a
stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from itn_gb300 import BPEngine
from itn_gb300 import _lib as L
from itn_gb300 import generators as GEN
from itn_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(lib_built):
    return L.load(lib_built)


def _dev(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def _static_logz(lib, torch, g, t, m, code, max_tensor=None, phys=None):
    dev = dict(
        off=_dev(torch, g.off.astype(np.int32)), rev=_dev(torch, g.rev.astype(np.int32)),
        bond=_dev(torch, g.bond.astype(np.int32)),
        phys=_dev(torch, (g.phys if phys is None else phys).astype(np.int32)),
        toff=_dev(torch, g.toff.astype(np.int64)), moff=_dev(torch, g.moff.astype(np.int64)),
        tens=_dev(torch, t), msgs=_dev(torch, m))
    total = torch.zeros(2, dtype=torch.float64, device="cuda")
    flags = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    if max_tensor is None:
        max_tensor = int(np.max(np.diff(g.toff)))
    results = []
    for _ in range(2):  # two calls in a row share the static scratch
        total.zero_()
        st = lib.itn_logz_static_scratch(
            0, stream, code, int(g.layers), g.nv, g.nslots, max_tensor,
            dev["off"].data_ptr(), dev["rev"].data_ptr(), dev["bond"].data_ptr(), dev["phys"].data_ptr(),
            dev["toff"].data_ptr(), dev["moff"].data_ptr(), dev["tens"].data_ptr(), dev["msgs"].data_ptr(),
            total.data_ptr(), flags.data_ptr(), err, len(err))
        assert st == L.ITN_OK, err.value
        torch.cuda.synchronize()
        results.append((total.cpu().numpy().copy(), int(flags.cpu().item())))
    return results


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-10), (np.float32, 2e-4), (np.complex128, 1e-10),
                                       (np.complex64, 2e-4)])
def test_static_scratch_matches_logscalars(lib, dtype, tol):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    g = G.square_lattice(6, 6, 4, periodic=True, phys=2)
    t = G.random_tensors(g, rng, dtype, G.peps_scale(g))
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.init_messages()
        e.run(maxiter=25)
        m = e.messages()
        ref = e.logscalars()
    code = L.DTYPE_CODE[np.dtype(dtype)]
    for total, flags in _static_logz(lib, torch, g, t, m, code):
        assert flags == int(ref["flags"][0])
        assert abs(total[0] - ref["totals"][0][0]) <= tol * abs(ref["totals"][0][0])
        # complex: the imaginary part of a sum of logs is defined modulo 2 pi
        dim = np.angle(np.exp(1j * (total[1] - ref["totals"][0][1])))
        assert abs(dim) <= tol * max(1.0, abs(ref["totals"][0][1]))


def test_static_scratch_against_the_fp64_oracle(lib):
    """The same log-norm against the CPU oracle's FP64 restatement of bethe_free_energy
    (messagecache.jl:185-201) on the same tensors and messages, within 1e-10 relative, on two
    calls in a row."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    rng = np.random.default_rng(17)
    g = G.square_lattice(5, 5, 3, periodic=False, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m, _, _, _ = O.bp_run(g, t, G.identity_messages(g), maxiter=20)
    ref = O.logscalars(g, t, m)["total"][0]
    for total, flags in _static_logz(lib, torch, g, t, m, L.F64):
        assert flags == 0
        assert abs(total[0] - ref) <= 1e-10 * abs(ref)


def test_static_scratch_flags_vertices_it_cannot_contract(lib):
    """A max_tensor_elems below the largest tensor (bit 3), a vertex with 17 legs (bit 4)
    and a one-layer vertex with a physical index (bit 5) each give NaN and their flag bit,
    and the call after them, with the right sizes, is exact again (the bits start at zero
    on every call)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    g = G.square_lattice(4, 4, 2, periodic=True, phys=2)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    m = G.identity_messages(g)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(m)
        ref = e.logscalars()["totals"][0][0]
    for total, flags in _static_logz(lib, torch, g, t, m, L.F64, max_tensor=int(np.max(np.diff(g.toff))) - 1):
        assert flags & 8 and np.isnan(total[0])
    for total, flags in _static_logz(lib, torch, g, t, m, L.F64):
        assert flags == 0 and abs(total[0] - ref) <= 1e-10 * abs(ref)
    # a star: vertex 0 with 17 legs of dimension 2 (2 * 2^17 tensor entries)
    star = G.from_edges(18, [(0, k) for k in range(1, 18)], 2, phys=2)
    ts = G.random_tensors(star, rng, np.float64)
    for total, flags in _static_logz(lib, torch, star, ts, G.identity_messages(star), L.F64):
        assert flags & 16 and np.isnan(total[0])
    # one-layer network handed a physical dimension of 2 on vertex 5
    gp = G.square_lattice(4, 4, 2, periodic=True, phys=1, layers=1)
    tp = G.random_tensors(gp, rng, np.float64)
    phys = gp.phys.copy()
    phys[5] = 2
    for total, flags in _static_logz(lib, torch, gp, tp, G.identity_messages(gp), L.F64, phys=phys):
        assert flags & 32 and np.isnan(total[0])


def test_static_scratch_plain_network(lib):
    """One-layer network (spin ice on a 4x4 torus) through the same entry point."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(123)
    g = G.square_lattice(4, 4, 2, periodic=True, phys=1, layers=1)
    t = GEN.spin_ice_tensors(g)
    with BPEngine(g) as e:
        e.set_tensors(t)
        e.set_messages(G.random_messages(g, rng))
        e.run(schedule="sequential", edges=G.tree_edge_sequence(g), maxiter=10, tol=1e-10)
        m = e.messages()
        ref = e.logscalars()
    for total, flags in _static_logz(lib, torch, g, t, m, L.F64):
        assert abs(total[0] - ref["totals"][0][0]) <= 1e-10 * abs(ref["totals"][0][0])


def test_static_scratch_rejects_oversized_network(lib):
    torch = pytest.importorskip("torch")
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    err = ctypes.create_string_buffer(256)
    p = x.data_ptr()
    st = lib.itn_logz_static_scratch(0, None, L.F64, 2, 4, 8, 10 ** 7, p, p, p, p, p, p, p, p, p, p,
                                     err, len(err))
    assert st == L.ITN_ERR_ARG
    assert b"static scratch" in err.value
