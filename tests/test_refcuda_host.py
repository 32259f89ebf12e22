"""The host driver of the reference's own CUDA kernels (oracle/refcuda),
without a GPU: the library builds, exports every entry point refcuda.h
declares, and for each configuration it drives its table of kernel names
matches exactly one kernel of the cubins compiled from the reference's
sources (their symbol names as nm lists them)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from alsvinn_gb300 import _build
from oracle import refcuda

HEADER = os.path.join(os.path.dirname(refcuda.__file__), "refcuda", "refcuda.h")
CONFIGS = [("euler1", "hll3", "neumann"), ("euler2", "hll3", "periodic"), ("euler3", "hll3", "periodic"),
           ("euler2", "hll", "neumann"), ("euler3", "hll", "neumann")]


@pytest.fixture(scope="module")
def library():
    try:
        _build.build_refcuda()
    except RuntimeError as e:
        pytest.skip("nvcc cannot build oracle/librefcuda.so here: %s" % str(e)[:200])
    return refcuda.load()


def test_exports_every_declared_entry_point(library):
    names = re.findall(r"\b(refcuda_[a-z_]+)\s*\(", open(HEADER).read())
    assert len(set(names)) >= 9
    for n in set(names):
        assert hasattr(library, n), n


def test_a_solver_without_a_gpu_fails_with_a_message(library):
    with pytest.raises(refcuda.RefCudaError):
        refcuda.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (8, 8, 1), (0, 0, 0), (1, 1, 0))
    with pytest.raises(refcuda.RefCudaError) as e:
        refcuda.Solver("burgers", "godunov", "weno2", "rungekutta3", "periodic", (8, 1, 1), (0, 0, 0), (1, 1, 1))
    assert "euler" in str(e.value)


@pytest.mark.parametrize("eq,flux,bc", CONFIGS)
def test_kernel_table_matches_one_kernel_each(library, eq, flux, bc):
    cubins = [os.path.join(refcuda.CUBIN_DIR, c) for c in refcuda.CUBINS]
    if not all(os.path.exists(c) for c in cubins):
        pytest.skip("the reference's CUDA kernels are not compiled here")
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    symbols = []
    for c in cubins:
        out = subprocess.run(["nm", "-C", c], capture_output=True, text=True, check=True).stdout
        symbols += [line.split(" ", 2)[2] for line in out.splitlines() if line.count(" ") >= 2]
    dim = int(eq[-1])
    needles = refcuda.kernel_names(eq, flux, bc)
    assert len(needles) == 1 + 3 * dim + 2 * dim + 3
    for n in needles:
        hits = [s for s in symbols if n in s]
        assert len(hits) == 1, (n, hits[:3])
