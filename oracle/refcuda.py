"""ctypes binding of oracle/librefcuda.so, the host driver of the reference's
own CUDA kernels (oracle/refcuda/refcuda.cu; the kernels are the reference's
sources compiled for sm_103a into oracle/_ref/cuda/*.cubin by
oracle/refbuild/Makefile, target `cuda`).

Test and baseline infrastructure: only the tests and bench.py's reference arm
use it, as the reference's GPU path to compare with and to time beside the
product's kernels.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librefcuda.so")
CUBIN_DIR = os.path.join(HERE, "_ref", "cuda")
CUBINS = ("NumericalFluxCUDA.cubin", "ReconstructionCUDA.cubin", "BoundaryCUDA.cubin", "vector_operations.cubin",
          "CUDACellComputer.cubin")

_lib = None


def missing():
    """Why the reference's CUDA path cannot run here, or None."""
    if not os.path.exists(LIB):
        return "oracle/librefcuda.so is not built"
    absent = [c for c in CUBINS if not os.path.exists(os.path.join(CUBIN_DIR, c))]
    if absent:
        return ("the reference's CUDA kernels are not compiled (oracle/_ref/cuda: %s); they build where the "
                "reference sources are" % ", ".join(absent))
    return None


def load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(LIB)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.refcuda_error.restype = ctypes.c_char_p
        lib.refcuda_create.argtypes = [ctypes.c_char_p] * 6 + [P, P, P, D, D, ctypes.POINTER(P)]
        lib.refcuda_create.restype = I
        lib.refcuda_destroy.argtypes = [P]
        lib.refcuda_set_state.argtypes = [P, P]
        lib.refcuda_get_state.argtypes = [P, P]
        lib.refcuda_run.argtypes = [P, D, I, I, ctypes.POINTER(D), ctypes.POINTER(I)]
        lib.refcuda_last_ms.argtypes = [P]
        lib.refcuda_last_ms.restype = ctypes.c_float
        lib.refcuda_launches.argtypes = [P]
        lib.refcuda_launches.restype = ctypes.c_long
        lib.refcuda_padded_cells.argtypes = [P]
        lib.refcuda_padded_cells.restype = ctypes.c_long
        lib.refcuda_kernel_names.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                             I]
        _lib = lib
    return _lib


class RefCudaError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise RefCudaError(load().refcuda_error().decode())


def kernel_names(equation, flux, boundary):
    """The demangled-name fragments of the kernels a configuration launches
    (no GPU needed)."""
    buf = ctypes.create_string_buffer(1 << 16)
    _check(load().refcuda_kernel_names(equation.encode(), flux.encode(), boundary.encode(), buf, len(buf)))
    return [n for n in buf.value.decode().split("\n") if n]


class Solver:
    """The reference's cuda-platform Simulator step for Euler / WENO2 /
    HLL or HLL3 / FE, RK2 or RK3 / periodic or Neumann."""

    def __init__(self, equation, flux, reconstruction, integrator, boundary, n, lower, upper, gamma=1.4, cfl=0.4):
        lib = load()
        self.h = ctypes.c_void_p()
        n3 = (ctypes.c_int * 3)(*n)
        lo = (ctypes.c_double * 3)(*lower)
        hi = (ctypes.c_double * 3)(*upper)
        _check(lib.refcuda_create(CUBIN_DIR.encode(), equation.encode(), flux.encode(), reconstruction.encode(),
                                  integrator.encode(), boundary.encode(), n3, lo, hi, gamma, cfl,
                                  ctypes.byref(self.h)))
        self.padded = lib.refcuda_padded_cells(self.h)
        self.nvar = {"euler1": 3, "euler2": 4, "euler3": 5}[equation]

    def close(self):
        if self.h:
            load().refcuda_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.nvar, self.padded)
        _check(load().refcuda_set_state(self.h, U.ctypes.data))

    def get_state(self):
        out = np.empty((self.nvar, self.padded))
        _check(load().refcuda_get_state(self.h, out.ctypes.data))
        return out

    def run(self, end_time, number_of_saves=0, max_steps=0):
        t = ctypes.c_double()
        k = ctypes.c_int()
        _check(load().refcuda_run(self.h, end_time, number_of_saves, max_steps, ctypes.byref(t), ctypes.byref(k)))
        return t.value, k.value

    def last_ms(self):
        return float(load().refcuda_last_ms(self.h))

    def launches(self):
        return int(load().refcuda_launches(self.h))
