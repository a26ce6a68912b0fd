"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, exports every
symbol include/itn_gpu.h declares, and fails cleanly (status code, no abort) when no
device is present."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "itn_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|const char \*|void)\s*\*?\s*(itn_\w+)\s*\(", txt, re.M)))


def test_header_lists_entry_points():
    syms = declared_symbols()
    assert "itn_bp_run" in syms and "itn_logscalars" in syms and len(syms) >= 15


def test_library_exports_declared_symbols(lib_built):
    lib = ctypes.CDLL(lib_built)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(lib_built):
    from itn_gb300 import _lib as L
    assert sorted(L.EXPORTED) == declared_symbols()


def test_abi_version_and_status_strings(lib_built):
    from itn_gb300 import _lib as L
    lib = L.load(lib_built)
    assert lib.itn_abi_version() == 2
    assert lib.itn_status_string(0) == b"ok"
    assert lib.itn_status_string(1) == b"invalid argument"


def test_null_arguments_rejected(lib_built):
    from itn_gb300 import _lib as L
    lib = L.load(lib_built)
    assert lib.itn_create(None, 0, 0) == L.ITN_ERR_ARG
    assert lib.itn_destroy(None) == L.ITN_ERR_ARG
    assert lib.itn_bp_run(None, None, None) == L.ITN_ERR_ARG
    assert lib.itn_bp_solve(None, 0, None, None, None, None, None, None, None) == L.ITN_ERR_ARG
    assert lib.itn_bp_solve_submit(None, 0, None, None, None, None, 1) == L.ITN_ERR_ARG
    assert lib.itn_bp_solve_wait(None, None, None, None) == L.ITN_ERR_ARG
    assert lib.itn_last_error(None) == b"null context"


def test_create_without_gpu_reports_status(lib_built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from itn_gb300 import _lib as L
    lib = L.load(lib_built)
    ctx = ctypes.c_void_p()
    st = lib.itn_create(ctypes.byref(ctx), 0, 0)
    assert st == L.ITN_ERR_CUDA and not ctx.value


def test_missing_library_fails_loudly(tmp_path):
    """Without libitn_gpu.so there is no fallback: loading raises."""
    import importlib
    from itn_gb300 import _lib as L
    saved = L._lib
    try:
        L._lib = None
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            L.load(str(tmp_path / "libitn_gpu.so"))
    finally:
        L._lib = saved


def test_gate_descriptor_layout(lib_built):
    """ctypes mirror of itn_gate_desc matches the C layout (216 bytes; the C client checks
    the same numbers with sizeof / offsetof)."""
    from itn_gb300 import _lib as L
    assert ctypes.sizeof(L.GateDesc) == 216
    assert L.GateDesc.site_off.offset == 72 and L.GateDesc.s_off.offset == 208
    lib = L.load(lib_built)
    assert lib.itn_apply_gates(None, 1, 0, None, None, 0, None, 0, None, 0, 0, 0.0, 0, None, 0, None, 0,
                               None, None) == L.ITN_ERR_ARG


def test_header_constants_match_python_binding():
    """Every enum constant of the header (status codes, dtypes, schedules, precisions,
    message initialisations, fault kinds) has the same value in the ctypes binding, under
    its own name (ITN_OK, ITN_ERR_*) or without the ITN_ prefix (F32, PREC_*, FAULT_*...)."""
    from itn_gb300 import _lib as L
    txt = open(HEADER).read()
    consts = {}
    for body in re.findall(r"enum\s*\{([^}]*)\}", txt):
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        for name, val in re.findall(r"(ITN_\w+)\s*=\s*(\d+)", body):
            consts[name] = int(val)
    assert len(consts) >= 26 and "ITN_FAULT_NO_PERSISTENT_SWEEPS" in consts
    for name, val in consts.items():
        py = getattr(L, name, None)
        if py is None:
            py = getattr(L, name[len("ITN_"):], None)
        assert py == val, (name, val, py)
