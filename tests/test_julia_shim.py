"""The Julia shim (itensornetworksnext.jl_gb300/julia/ITensorNetworksNextGPU.jl) against the C
header, without Julia: every `ccall` names an exported entry point with the same number of
arguments and the same argument classes (pointer / int32 / int64 / double) as its prototype in
include/itn_gpu.h, the Julia mirrors of the C structs list the same field types in the same
order, and tests/c/julia_shim_replay.c (which replays the shim's calls from C) compiles; with
a GPU it runs them on a small norm network against closed forms."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

JL = os.path.join(ROOT, "itensornetworksnext.jl_gb300", "julia", "ITensorNetworksNextGPU.jl")
HEADER = os.path.join(ROOT, "include", "itn_gpu.h")
REPLAY = os.path.join(ROOT, "tests", "c", "julia_shim_replay.c")


def _split_top(s):
    """Split on commas not nested in braces or parentheses."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "{(":
            depth += 1
        elif ch in "})":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _jl_class(t):
    t = t.strip()
    if t.startswith(("Ptr{", "Ref{")) or t == "Cstring":
        return "ptr"
    return {"Int32": "i32", "Int64": "i64", "Float64": "f64", "Cvoid": "void"}[t]


def _c_class(t):
    t = t.strip()
    if "*" in t:
        return "ptr"
    t = t.replace("const", "").split()[0]
    return {"int32_t": "i32", "int64_t": "i64", "double": "f64", "void": "void"}[t]


def jl_ccalls():
    txt = open(JL).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+),\s*libitn\),\s*(\w+(?:\{[^}]*\})?),\s*\(", txt):
        # the argument-type tuple: up to the matching parenthesis
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(txt[i], 0)
            i += 1
        args = _split_top(txt[m.end():i - 1])
        calls.append((m.group(1), _jl_class(m.group(2)), [_jl_class(a) for a in args]))
    return calls


def c_prototypes():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"(int32_t|const char \*)\s*(itn_\w+)\s*\(([^;]*?)\);", txt, re.S):
        ret = "ptr" if "*" in m.group(1) else "i32"
        args = [a for a in _split_top(m.group(3)) if a.strip() != "void"]
        protos[m.group(2)] = (ret, [_c_class(a.rsplit(" ", 1)[0] if "*" not in a else a) for a in args])
    return protos


def test_every_ccall_matches_its_prototype():
    protos = c_prototypes()
    calls = jl_ccalls()
    names = {n for n, _, _ in calls}
    # the shim's plug-in points reach these entry points
    for need in ("itn_bp_run", "itn_message_update", "itn_logscalars", "itn_contract_network", "itn_bp_grad",
                 "itn_tensors_upload_strided", "itn_messages_upload", "itn_messages_download"):
        assert need in names, need
    for name, ret, args in calls:
        assert name in protos, name
        pret, pargs = protos[name]
        assert ret == pret, (name, ret, pret)
        assert args == pargs, (name, args, pargs)


def _jl_struct(name):
    txt = open(JL).read()
    m = re.search(r"struct %s\n(.*?)\nend" % name, txt, re.S)
    fields = [ln.split("::")[1].strip() for ln in m.group(1).splitlines() if "::" in ln]
    return [_jl_class(f) for f in fields]


def _c_struct(name):
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*%s;" % name, txt, re.S)
    out = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, names = ("ptr", decl) if "*" in decl else (decl.split()[0], decl)
        n = len(names.split(","))
        cls = "ptr" if typ == "ptr" else _c_class(typ)
        out += [cls] * n
    return out


@pytest.mark.parametrize("jl,c", [("ItnBpOpts", "itn_bp_opts"), ("ItnBpResult", "itn_bp_result"),
                                  ("ItnGradOpts", "itn_grad_opts"), ("ItnGradResult", "itn_grad_result")])
def test_julia_structs_mirror_the_c_structs(jl, c):
    assert _jl_struct(jl) == _c_struct(c)


def _build_replay(lib, tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    exe = str(tmp_path / "julia_shim_replay")
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-O2", "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"), REPLAY, "-o", exe,
                    "-L", libdir, "-litn_gpu", f"-Wl,-rpath,{libdir}", "-lm"], check=True)
    return exe


def test_replay_compiles_with_the_julia_layouts(lib_built, tmp_path):
    exe = _build_replay(lib_built, tmp_path)
    r = subprocess.run([exe, "host"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


@pytest.mark.gpu
def test_replay_of_the_shim_calls_on_a_gpu(lib_built, tmp_path):
    exe = _build_replay(lib_built, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
