"""The C ABI from C: tests/c/abi_client.c is compiled with gcc against include/itn_gpu.h
and linked to libitn_gpu.so.  CPU mode checks host-only entry points and clean failure
without a device; the gpu-marked variant also runs a two-site solve."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c", "abi_client.c")


def _build(lib, tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    exe = str(tmp_path / "abi_client")
    libdir = os.path.dirname(lib)
    subprocess.run(["gcc", "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                    "-L", libdir, "-litn_gpu", f"-Wl,-rpath,{libdir}", "-lm"], check=True)
    return exe


def test_c_client_host_only(lib_built, tmp_path):
    exe = _build(lib_built, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


@pytest.mark.gpu
def test_c_client_gpu(lib_built, tmp_path):
    exe = _build(lib_built, tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
