"""The C ABI from a plain C99 program (no C++ in the header, no Python):
compiles tests/c_abi/host_calls.c against include/fwi_psv.h, links the
library and runs the host-only entry points."""
import os
import shutil
import subprocess

import pytest

from fwi_cuda_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plain_c_caller(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    _lib.lib()  # builds the library when it is missing
    so = _lib.LIB
    exe = tmp_path / "host_calls"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_abi", "host_calls.c"),
                    "-o", str(exe), so, "-lm", "-Wl,-rpath," + os.path.dirname(so)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok ")


def test_reference_side_binding_compiles_and_links(tmp_path):
    # the C++ the reference's GPU branch would hold (the integration guide's
    # example), against the header and the library's exported symbols
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    _lib.lib()
    so = _lib.LIB
    exe = tmp_path / "reference_binding"
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_abi", "reference_binding.cpp"), "-o", str(exe),
                    so, "-Wl,-rpath," + os.path.dirname(so)], check=True)
    # GPU_CODE is 0 in the test binary: it links and exits without device work
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
