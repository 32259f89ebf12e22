"""GB300-native implementation of alsvinn's explicit finite-volume step and
ensemble statistics: hand-written sm_103a CUDA kernels behind the C ABI in
include/gbfv.h (built in-tree as alsvinn_gb300/lib/libgbfv.so)."""
from . import lib  # noqa: F401
from .lib import FP32, FP64, FP64_EXACT, GbfvError, Solver, Stats  # noqa: F401

__all__ = ["lib", "Solver", "Stats", "GbfvError", "FP64", "FP64_EXACT", "FP32"]
