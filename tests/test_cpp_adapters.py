"""The C++ adapter header (include/gbfv_alsfvm.hpp) and the fast special
functions of the kernels: both test programs compile on the CPU and pass on
the GPU (the adapters' one is written like the reference's library tests)."""
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


PLATFORM = os.path.join(ROOT, "tests", "cpp", "test_alsvinn_platform.cpp")
REFBUILD = os.path.join(ROOT, "oracle", "refbuild")
REF_LIB = os.path.join(ROOT, "oracle", "_ref")


def reference_root():
    """The reference sources: REF_ROOT, else the location the reference
    recipe names; None where they are absent (as on the GPU machine)."""
    ref = os.environ.get("REF_ROOT")
    if not ref:
        p = subprocess.run(["make", "-s", "--no-print-directory", "-C", REFBUILD, "print-ref"], capture_output=True,
                           text=True)
        ref = p.stdout.strip() if p.returncode == 0 else ""
    return ref if ref and os.path.isdir(os.path.join(ref, "alsfvm", "include")) else None


def test_platform_classes_build_against_the_reference(tmp_path):
    """include/gbfv_alsvinn.hpp's classes derive from the reference's own
    Memory<real>, NumericalFlux, Reconstruction, Boundary and CellComputer:
    compiled against the reference's headers (with the oracle build's
    stand-ins for Boost and MPI) and linked with the reference's CPU library
    and libgbfv.so, every pure virtual is implemented with its signature."""
    ref = reference_root()
    if ref is None or not os.path.exists(os.path.join(REF_LIB, "libalsref.so")):
        pytest.skip("the reference's sources or its CPU build are absent")
    cxx = shutil.which("g++") or "g++"
    lib = os.path.join(ROOT, "alsvinn_gb300", "lib")
    exe = str(tmp_path / "test_alsvinn_platform")
    cmd = [cxx, "-std=c++17", "-O1", "-fopenmp", "-I" + os.path.join(REFBUILD, "stubs"),
           "-I" + os.path.join(ref, "alsfvm", "include"), "-I" + os.path.join(ref, "alsutils", "include"),
           "-I" + os.path.join(ref, "alsuq", "include"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(CUDA, "include"), PLATFORM, "-o", exe, "-L" + REF_LIB, "-lalsref", "-L" + lib, "-lgbfv",
           "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + REF_LIB, "-Wl,-rpath," + lib,
           "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "linked" in r.stdout, r.stdout + r.stderr


SPECIAL = os.path.join(ROOT, "tests", "cpp", "test_special_functions.cu")


def _nvcc_cmd(out):
    nvcc = os.path.join(CUDA, "bin", "nvcc")
    return [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
            "-I" + os.path.join(ROOT, "alsvinn_gb300", "csrc"), SPECIAL, "-o", out]


def test_special_function_test_compiles(tmp_path):
    p = subprocess.run(_nvcc_cmd(str(tmp_path / "sf")), capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


@pytest.mark.gpu
def test_special_functions_meet_their_error_bounds(cuda_device, tmp_path):
    exe = str(tmp_path / "sf")
    p = subprocess.run(_nvcc_cmd(exe), capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
