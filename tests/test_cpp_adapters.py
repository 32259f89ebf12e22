"""The C++ adapter header (include/gbfv_alsfvm.hpp): it compiles on the CPU;
its test program, written like the reference's library tests, passes on the
GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_alsfvm_adapters.cpp")
CUDA = "/usr/local/cuda"


def compile_cmd(out, syntax_only=False):
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include")]
    if syntax_only:
        return cmd + ["-fsyntax-only", SRC]
    lib = os.path.join(ROOT, "alsvinn_gb300", "lib")
    return cmd + [SRC, "-o", out, "-L" + lib, "-lgbfv", "-L" + os.path.join(CUDA, "lib64"), "-lcudart",
                  "-Wl,-rpath," + lib, "-Wl,-rpath," + os.path.join(CUDA, "lib64")]


def test_adapter_header_compiles():
    p = subprocess.run(compile_cmd(None, syntax_only=True), capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


@pytest.mark.gpu
def test_adapters_pass_their_tests(cuda_device, tmp_path):
    exe = str(tmp_path / "test_alsfvm_adapters")
    p = subprocess.run(compile_cmd(exe), capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
