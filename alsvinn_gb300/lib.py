"""ctypes binding of the gbfv C ABI (include/gbfv.h).

The library is the in-tree alsvinn_gb300/lib/libgbfv.so. There is no CPU
fallback: loading fails loudly when the library is missing, and every call
that returns a negative status raises GbfvError with the library's message.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libgbfv.so")

FP64, FP64_EXACT, FP32, FP64_DF = 0, 1, 2, 3
OK, ERR_ARGUMENT, ERR_CUDA, ERR_CONSTRAINT, ERR_MEMORY, ERR_UNSUPPORTED = 0, -1, -2, -3, -4, -5

_c_int3 = ctypes.c_int * 3
_c_double3 = ctypes.c_double * 3


ERR_ARGUMENT = -1  # GBFV_ERR_ARGUMENT


class GbfvError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("gbfv error %d: %s" % (code, message))
        self.code = code


class _Desc(ctypes.Structure):
    _fields_ = [
        ("equation", ctypes.c_char_p),
        ("flux", ctypes.c_char_p),
        ("reconstruction", ctypes.c_char_p),
        ("integrator", ctypes.c_char_p),
        ("boundary", ctypes.c_char_p),
        ("n", ctypes.c_int * 3),
        ("lower", ctypes.c_double * 3),
        ("upper", ctypes.c_double * 3),
        ("gamma", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("precision", ctypes.c_int),
    ]


_lib = None

# name -> (restype, argtypes)
_SIGNATURES = {
    "gbfv_last_error": (ctypes.c_char_p, []),
    "gbfv_version": (ctypes.c_char_p, []),
    "gbfv_ghost_cells": (ctypes.c_int, [ctypes.c_char_p]),
    "gbfv_num_variables": (ctypes.c_int, [ctypes.c_char_p]),
    "gbfv_create": (ctypes.c_int, [ctypes.POINTER(_Desc), ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_extents": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_set_primitive": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_set_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_state_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_advance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int]),
    "gbfv_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gbfv_profile_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_double)]),
    "gbfv_advance_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_int]),
    "gbfv_compute_flux": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_double)]),
    "gbfv_reconstruct": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "gbfv_apply_boundary": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_obeys_constraints": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gbfv_stats_create": (ctypes.c_int, [ctypes.c_longlong, ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_stats_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_stats_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_stats_add_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "gbfv_stats_add_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_stats_merge": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_stats_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_stats_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_generator_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_generator_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_generator_uniform": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                              ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "gbfv_advance_schedule": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gbfv_structure_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_structure_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_structure_add_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "gbfv_structure_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_structure_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_structure_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_structure_create_basic": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_functional_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                              ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                              ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_functional_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_functional_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int)]),
    "gbfv_functional_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_functional_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
    "gbfv_functional_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_uniform": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_void_p]),
    "gbfv_advance_noalloc": (ctypes.c_int, [ctypes.POINTER(_Desc), ctypes.c_void_p,
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong),
                                            ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]),
    "gbfv_batch_create": (ctypes.c_int, [ctypes.POINTER(_Desc), ctypes.c_longlong, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_batch_member_bytes": (ctypes.c_longlong, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gbfv_batch_free_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                             ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_add": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int)]),
    "gbfv_batch_remove": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gbfv_batch_advance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int]),
    "gbfv_batch_member_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_member_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "gbfv_batch_stats_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_stats_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_stats_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_batch_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_batch_select_candidate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gbfv_batch_set_statistics_saves": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gbfv_batch_stats_export_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                    ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_current_candidate": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                                    ctypes.POINTER(ctypes.c_int)]),
    "gbfv_batch_autotune_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "gbfv_candidate_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gbfv_candidate_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "gbfv_select_candidate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gbfv_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                     ctypes.c_int]),
    "gbfv_current_candidate": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gbfv_init_sod": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "gbfv_init_kelvin_helmholtz": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "gbfv_init_taylor_green": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "gbfv_init_burgers_sine": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_void_p]),
    "gbfv_test_tma_wait_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint]),
    "gbfv_memory_op": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int,
                                      ctypes.c_void_p]),
    "gbfv_memory_op_scalar": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_longlong,
                                             ctypes.c_int, ctypes.c_void_p]),
    "gbfv_memory_make_zero": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p]),
    "gbfv_memory_add_linear_combination": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                                          ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                                          ctypes.c_double, ctypes.c_void_p, ctypes.c_double,
                                                          ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int,
                                                          ctypes.c_void_p]),
    "gbfv_memory_add_power": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p]),
    "gbfv_memory_subtract_power": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                                  ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p]),
    "gbfv_memory_total_variation": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                                   ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                                   ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "gbfv_compute_flux_region": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]),
    "gbfv_reconstruct_vars": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]),
    "gbfv_apply_boundary_vars": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_obeys_constraints_vars": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                                   ctypes.c_void_p]),
    "gbfv_prim_to_cons_vars": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "gbfv_extra_variables_vars": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p]),
    "gbfv_max_wave_speed_vars": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
}

NOALLOC_SCRATCH_BYTES = 32 << 20

MEMORY_ADD, MEMORY_SUBTRACT, MEMORY_MULTIPLY, MEMORY_DIVIDE = 0, 1, 2, 3


def _ptrs(ptrs):
    """A C array of device pointers (one per variable)."""
    return (ctypes.c_void_p * len(ptrs))(*[ctypes.c_void_p(int(p)) for p in ptrs])


def memory_op(op, a_dev, b_dev, count, precision=0, stream=None):
    """a op= b on device arrays (gbfv_memory_op)."""
    _check(load().gbfv_memory_op(op, ctypes.c_void_p(a_dev), ctypes.c_void_p(b_dev), count, precision,
                                 ctypes.c_void_p(stream)))


def memory_op_scalar(op, a_dev, scalar, count, precision=0, stream=None):
    _check(load().gbfv_memory_op_scalar(op, ctypes.c_void_p(a_dev), float(scalar), count, precision,
                                        ctypes.c_void_p(stream)))


def memory_make_zero(a_dev, count, precision=0, stream=None):
    _check(load().gbfv_memory_make_zero(ctypes.c_void_p(a_dev), count, precision, ctypes.c_void_p(stream)))


def memory_add_linear_combination(v1, a1, a2, v2, a3, v3, a4, v4, a5, v5, count, precision=0, stream=None):
    vp = [ctypes.c_void_p(x) for x in (v1, v2, v3, v4, v5)]
    _check(load().gbfv_memory_add_linear_combination(vp[0], a1, a2, vp[1], a3, vp[2], a4, vp[3], a5, vp[4], count,
                                                     precision, ctypes.c_void_p(stream)))


def memory_add_power(a_dev, b_dev, power, count, factor=1.0, precision=0, stream=None):
    _check(load().gbfv_memory_add_power(ctypes.c_void_p(a_dev), ctypes.c_void_p(b_dev), power, factor, count,
                                        precision, ctypes.c_void_p(stream)))


def memory_subtract_power(a_dev, b_dev, power, count, precision=0, stream=None):
    _check(load().gbfv_memory_subtract_power(ctypes.c_void_p(a_dev), ctypes.c_void_p(b_dev), power, count,
                                             precision, ctypes.c_void_p(stream)))


def memory_total_variation(a_dev, extents, p, direction, start, end, precision=0, stream=None):
    r = ctypes.c_double()
    _check(load().gbfv_memory_total_variation(ctypes.c_void_p(a_dev), _c_int3(*extents), int(p), int(direction),
                                              _c_int3(*start), _c_int3(*end), precision, ctypes.byref(r),
                                              ctypes.c_void_p(stream)))
    return r.value


def make_desc(equation, flux, reconstruction, integrator, boundary, n, lower, upper, gamma=1.4, cfl=0.475,
              precision=FP64):
    """A gbfv_desc; the returned tuple keeps the name buffers alive."""
    keep = [s.encode() for s in (equation, flux, reconstruction, integrator, boundary)]
    d = _Desc()
    d.equation, d.flux, d.reconstruction, d.integrator, d.boundary = keep
    d.n = _c_int3(*n)
    d.lower = _c_double3(*lower)
    d.upper = _c_double3(*upper)
    d.gamma = gamma
    d.cfl = cfl
    d.precision = precision
    return d, keep


def advance_noalloc(desc, state_dev, t, steps, end_time, number_of_saves=0, max_steps=0, stream=None):
    """gbfv_advance_noalloc on a caller-owned device state; returns (t, steps)."""
    tt = ctypes.c_double(t)
    ss = ctypes.c_longlong(steps)
    _check(load().gbfv_advance_noalloc(ctypes.byref(desc), ctypes.c_void_p(state_dev), ctypes.byref(tt),
                                       ctypes.byref(ss), end_time, number_of_saves, max_steps,
                                       ctypes.c_void_p(stream)))
    return tt.value, ss.value


def exported_names():
    """The entry points include/gbfv.h declares."""
    return sorted(_SIGNATURES)


def load():
    """Loads libgbfv.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("alsvinn_gb300 native library missing: %s (run __graft_entry__.build())" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc):
    if rc < 0:
        raise GbfvError(rc, load().gbfv_last_error().decode())
    return rc


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def ghost_cells(reconstruction):
    return _check(load().gbfv_ghost_cells(reconstruction.encode()))


def num_variables(equation):
    return _check(load().gbfv_num_variables(equation.encode()))


def uniform(dimension, sample, lower=0.0, upper=1.0):
    out = np.zeros(dimension)
    _check(load().gbfv_uniform(dimension, sample, lower, upper, _ptr(out)))
    return out


def init_sod(n, lower=(-5.0, 0.0, 0.0), upper=(5.0, 1.0, 1.0)):
    prim = np.zeros((3, n))
    _check(load().gbfv_init_sod(_c_int3(n, 1, 1), _c_double3(*lower), _c_double3(*upper), _ptr(prim)))
    return prim


def init_kelvin_helmholtz(n, sample=0, X=None, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 0.0)):
    """KH initial data; X defaults to the generator's 40 draws of `sample`."""
    X = uniform(40, sample) if X is None else np.ascontiguousarray(X, dtype=np.float64)
    prim = np.zeros((4, n * n))
    _check(load().gbfv_init_kelvin_helmholtz(_c_int3(n, n, 1), _c_double3(*lower), _c_double3(*upper), _ptr(X),
                                             _ptr(prim)))
    return prim


def init_taylor_green(n, lower=(0.0, 0.0, 0.0), upper=(2 * np.pi, 2 * np.pi, 2 * np.pi)):
    prim = np.zeros((5, n ** 3))
    _check(load().gbfv_init_taylor_green(_c_int3(n, n, n), _c_double3(*lower), _c_double3(*upper), _ptr(prim)))
    return prim


def init_burgers_sine(n, phase, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0)):
    prim = np.zeros((1, n))
    _check(load().gbfv_init_burgers_sine(_c_int3(n, 1, 1), _c_double3(*lower), _c_double3(*upper), phase,
                                         _ptr(prim)))
    return prim


class _Schedule(ctypes.Structure):
    _fields_ = [("end_time", ctypes.c_double), ("save_interval", ctypes.c_double * 2),
                ("max_steps", ctypes.c_int), ("stop_at_save", ctypes.c_int)]


class Generator:
    """The run-wide mt19937_64 of alsuq's STLMersenne (gbfv_generator_*)."""

    def __init__(self):
        h = ctypes.c_void_p()
        _check(load().gbfv_generator_create(ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_generator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def uniform(self, dimension, component, sample, lower=0.0, upper=1.0):
        out = ctypes.c_double()
        _check(load().gbfv_generator_uniform(self.h, int(dimension), int(component), int(sample), float(lower),
                                             float(upper), ctypes.byref(out)))
        return out.value


class Solver:
    """One grid on the GPU: the handle of gbfv_create."""

    def __init__(self, equation, flux, reconstruction, integrator, boundary, n, lower, upper,
                 gamma=1.4, cfl=0.475, precision=FP64):
        lib = load()
        self._keep = [s.encode() for s in (equation, flux, reconstruction, integrator, boundary)]
        d = _Desc()
        d.equation, d.flux, d.reconstruction, d.integrator, d.boundary = self._keep
        d.n = _c_int3(*n)
        d.lower = _c_double3(*lower)
        d.upper = _c_double3(*upper)
        d.gamma = gamma
        d.cfl = cfl
        d.precision = precision
        h = ctypes.c_void_p()
        _check(lib.gbfv_create(ctypes.byref(d), ctypes.byref(h)))
        self.h = h
        self.equation = equation
        self.precision = precision
        self.n = tuple(n)
        self.nvar = num_variables(equation)
        t = _c_int3()
        total = ctypes.c_longlong()
        _check(lib.gbfv_extents(h, t, ctypes.byref(total)))
        self.padded = tuple(t)
        self.total = total.value
        self.dtype = np.float32 if precision == FP32 else np.float64

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_primitive(self, prim):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        _check(load().gbfv_set_primitive(self.h, _ptr(prim)))

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.size == self.nvar * self.total
        _check(load().gbfv_set_state(self.h, _ptr(U)))

    def get_state(self):
        U = np.zeros((self.nvar, self.total))
        _check(load().gbfv_get_state(self.h, _ptr(U)))
        return U

    def state_device(self):
        p = ctypes.c_void_p()
        _check(load().gbfv_state_device(self.h, ctypes.byref(p)))
        return p.value

    def advance(self, end_time, number_of_saves=0, max_steps=0):
        return _check(load().gbfv_advance(self.h, end_time, number_of_saves, max_steps))

    def advance_schedule(self, end_time, save_interval=(0.0, 0.0), max_steps=0, stop_at_save=False):
        """gbfv_advance_schedule: returns the saved mask of the last step."""
        sch = _Schedule(float(end_time), (ctypes.c_double * 2)(*save_interval), int(max_steps), int(bool(stop_at_save)))
        mask = ctypes.c_int()
        _check(load().gbfv_advance_schedule(self.h, ctypes.byref(sch), ctypes.byref(mask)))
        return mask.value

    def advance_host(self, U, end_time, number_of_saves=0, max_steps=0):
        assert U.dtype == np.float64 and U.flags.c_contiguous and U.size == self.nvar * self.total
        return _check(load().gbfv_advance_host(self.h, _ptr(U), end_time, number_of_saves, max_steps))

    def time(self):
        t = ctypes.c_double()
        s = ctypes.c_longlong()
        dt = ctypes.c_double()
        _check(load().gbfv_time(self.h, ctypes.byref(t), ctypes.byref(s), ctypes.byref(dt)))
        return t.value, s.value, dt.value

    def stream(self):
        p = ctypes.c_void_p()
        _check(load().gbfv_stream(self.h, ctypes.byref(p)))
        return p.value

    def profile(self, enable=True):
        _check(load().gbfv_profile(self.h, 1 if enable else 0))

    # -- stage kernel candidates and the autotuner -------------------------

    def candidates(self):
        """[(tile (x, y, z), threads, tma)] of the scheme's stage kernel
        configurations; index 0 is the default."""
        n = ctypes.c_int()
        _check(load().gbfv_candidate_count(self.h, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            tile = (ctypes.c_int * 3)()
            th, tma = ctypes.c_int(), ctypes.c_int()
            _check(load().gbfv_candidate_info(self.h, i, tile, ctypes.byref(th), ctypes.byref(tma)))
            out.append((tuple(tile), th.value, bool(tma.value)))
        return out

    def select_candidate(self, idx):
        """Pins candidate idx (-1: let the autotuner choose at the next advance)."""
        _check(load().gbfv_select_candidate(self.h, int(idx)))

    def current_candidate(self):
        i = ctypes.c_int()
        _check(load().gbfv_current_candidate(self.h, ctypes.byref(i)))
        return i.value

    def autotune(self):
        """Runs the autotuner now: (chosen index, [mean ms per stage launch of
        one step, or -1 where not eligible])."""
        n = len(self.candidates())
        ms = (ctypes.c_double * max(n, 1))()
        chosen = ctypes.c_int()
        _check(load().gbfv_autotune(self.h, ctypes.byref(chosen), ms, n))
        return chosen.value, list(ms)[:n]

    def profile_read(self):
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        k = ctypes.c_longlong()
        _check(load().gbfv_profile_read(self.h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(k)))
        return ms.value, n.value, k.value

    def compute_flux(self, state_dev, out_dev):
        ws = _c_double3()
        _check(load().gbfv_compute_flux(self.h, ctypes.c_void_p(state_dev), ctypes.c_void_p(out_dev), ws))
        return list(ws)

    def reconstruct(self, direction, state_dev, left_dev, right_dev):
        _check(load().gbfv_reconstruct(self.h, direction, ctypes.c_void_p(state_dev), ctypes.c_void_p(left_dev),
                                       ctypes.c_void_p(right_dev)))

    def apply_boundary(self, state_dev):
        _check(load().gbfv_apply_boundary(self.h, ctypes.c_void_p(state_dev)))

    def obeys_constraints(self, state_dev):
        ok = ctypes.c_int()
        _check(load().gbfv_obeys_constraints(self.h, ctypes.c_void_p(state_dev), ctypes.byref(ok)))
        return bool(ok.value)

    def test_tma_wait_limit(self, extra_bytes):
        """Test hook: TMA halo waits of this solver's stage launches run out
        their time limit (see gbfv_test_tma_wait_limit); 0 restores."""
        _check(load().gbfv_test_tma_wait_limit(self.h, int(extra_bytes)))

    # one device array per variable (a reference Volume's layout)
    def compute_flux_region(self, state_vars, out_vars, start=(0, 0, 0), end=(0, 0, 0), stream=None):
        ws = _c_double3()
        _check(load().gbfv_compute_flux_region(self.h, _ptrs(state_vars), _ptrs(out_vars), ws, _c_int3(*start),
                                               _c_int3(*end), ctypes.c_void_p(stream)))
        return list(ws)

    def reconstruct_vars(self, direction, state_vars, left_vars, right_vars, start=(0, 0, 0), end=(0, 0, 0),
                         stream=None):
        _check(load().gbfv_reconstruct_vars(self.h, direction, _ptrs(state_vars), _ptrs(left_vars),
                                            _ptrs(right_vars), _c_int3(*start), _c_int3(*end),
                                            ctypes.c_void_p(stream)))

    def apply_boundary_vars(self, vars_, stream=None):
        _check(load().gbfv_apply_boundary_vars(self.h, _ptrs(vars_), ctypes.c_void_p(stream)))

    def obeys_constraints_vars(self, vars_, stream=None):
        ok = ctypes.c_int()
        _check(load().gbfv_obeys_constraints_vars(self.h, _ptrs(vars_), ctypes.byref(ok), ctypes.c_void_p(stream)))
        return bool(ok.value)

    def prim_to_cons_vars(self, prim_vars, cons_vars, stream=None):
        _check(load().gbfv_prim_to_cons_vars(self.h, _ptrs(prim_vars), _ptrs(cons_vars), ctypes.c_void_p(stream)))

    def extra_variables_vars(self, cons_vars, extra_vars, stream=None):
        _check(load().gbfv_extra_variables_vars(self.h, _ptrs(cons_vars), _ptrs(extra_vars) if extra_vars else None,
                                                ctypes.c_void_p(stream)))

    def max_wave_speed_vars(self, cons_vars, direction, stream=None):
        w = ctypes.c_double()
        _check(load().gbfv_max_wave_speed_vars(self.h, _ptrs(cons_vars), direction, ctypes.byref(w),
                                               ctypes.c_void_p(stream)))
        return w.value


class Stats:
    """Streaming FP64 mean / variance (gbfv_stats_*)."""

    def __init__(self, count):
        h = ctypes.c_void_p()
        _check(load().gbfv_stats_create(count, ctypes.byref(h)))
        self.h = h
        self.count = count

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_stats_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        _check(load().gbfv_stats_reset(self.h))

    def add_device(self, ptr, precision=FP64):
        _check(load().gbfv_stats_add_device(self.h, ctypes.c_void_p(ptr), precision))

    def add_host(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        assert x.size == self.count
        _check(load().gbfv_stats_add_host(self.h, _ptr(x)))

    def merge(self, other):
        _check(load().gbfv_stats_merge(self.h, other.h))

    def result(self):
        m = np.zeros(self.count)
        v = np.zeros(self.count)
        n = ctypes.c_longlong()
        _check(load().gbfv_stats_result(self.h, _ptr(m), _ptr(v), ctypes.byref(n)))
        return m, v, n.value

    def export(self):
        """(count, mean, M2): the raw Welford triple for a cross-rank merge."""
        m = np.zeros(self.count)
        q = np.zeros(self.count)
        n = ctypes.c_longlong()
        _check(load().gbfv_stats_export(self.h, _ptr(m), _ptr(q), ctypes.byref(n)))
        return n.value, m, q


class _FunctionalParams(ctypes.Structure):
    _fields_ = [("degree", ctypes.c_int), ("min_value", ctypes.c_double), ("max_value", ctypes.c_double),
                ("variable_mask", ctypes.c_uint), ("gamma", ctypes.c_double), ("p", ctypes.c_double),
                ("number_of_h", ctypes.c_int), ("direction", ctypes.c_int)]


VARIABLE_NAMES = {"burgers": ["u"], "euler1": ["rho", "mx", "E"], "euler2": ["rho", "mx", "my", "E"],
                  "euler3": ["rho", "mx", "my", "mz", "E"]}


def variable_mask(equation, variables):
    """Bit mask of the named variables ("rho E" or a list); 0 (all) when empty.
    Unknown names raise, as the reference's LegendrePointWise does."""
    names = VARIABLE_NAMES[equation]
    mask = 0
    for v in (variables.split() if isinstance(variables, str) else list(variables or [])):
        if v not in names:
            raise GbfvError(ERR_ARGUMENT, "Unknown variable name given to the functional: %s" % v)
        mask |= 1 << names.index(v)
    return mask


class Functional:
    """A functional of one state (gbfv_functional_*): identity, moment,
    legendre_pointwise, log_entropy, bv, bv_direction, structure_cube.
    apply() adds weight times the functional of a device state into the
    accumulator; result() returns (nvar, output cells)."""

    def __init__(self, name, equation, boundary, n, ghosts, lower, upper, degree=0, min_value=0.0, max_value=1.0,
                 variables="", gamma=1.4, p=1.0, number_of_h=1, direction=0):
        prm = _FunctionalParams(int(degree), float(min_value), float(max_value), variable_mask(equation, variables),
                                float(gamma), float(p), int(number_of_h), int(direction))
        h = ctypes.c_void_p()
        _check(load().gbfv_functional_create(name.encode(), equation.encode(), boundary.encode(), _c_int3(*n),
                                             int(ghosts), _c_double3(*lower), _c_double3(*upper),
                                             ctypes.byref(prm), ctypes.byref(h)))
        self.h = h
        self.name = name
        size = _c_int3()
        nv = ctypes.c_int()
        _check(load().gbfv_functional_size(h, size, ctypes.byref(nv)))
        self.size = tuple(size)
        self.nvar = nv.value

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_functional_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        _check(load().gbfv_functional_reset(self.h))

    def apply(self, ptr, precision=FP64, weight=1.0):
        _check(load().gbfv_functional_apply(self.h, ctypes.c_void_p(ptr), precision, float(weight)))

    def result(self):
        out = np.zeros((self.nvar, int(np.prod(self.size))))
        _check(load().gbfv_functional_result(self.h, _ptr(out)))
        return out


class Structure:
    """Cube structure function statistic (gbfv_structure_*)."""

    def __init__(self, boundary, n, ghosts, nvar, number_of_h, p, direction=None):
        """direction None: the cube structure function (structure_cube);
        0, 1, 2: the axis structure function along that axis (structure_basic)."""
        h = ctypes.c_void_p()
        if direction is None:
            _check(load().gbfv_structure_create(boundary.encode(), _c_int3(*n), int(ghosts), int(nvar),
                                                int(number_of_h), float(p), ctypes.byref(h)))
        else:
            _check(load().gbfv_structure_create_basic(boundary.encode(), _c_int3(*n), int(ghosts), int(nvar),
                                                      int(number_of_h), float(p), int(direction), ctypes.byref(h)))
        self.h = h
        self.nvar = int(nvar)
        self.number_of_h = int(number_of_h)

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_structure_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_device(self, ptr, precision=FP64):
        _check(load().gbfv_structure_add_device(self.h, ctypes.c_void_p(ptr), precision))

    def result(self):
        out = np.zeros((self.nvar, self.number_of_h))
        n = ctypes.c_longlong()
        _check(load().gbfv_structure_result(self.h, _ptr(out), ctypes.byref(n)))
        return out, n.value

    def export(self):
        """(count, sums): the raw sums for a cross-rank merge."""
        out = np.zeros((self.nvar, self.number_of_h))
        n = ctypes.c_longlong()
        _check(load().gbfv_structure_export(self.h, _ptr(out), ctypes.byref(n)))
        return n.value, out


class Batch:
    """An ensemble of grids advanced together (gbfv_batch_*)."""

    def __init__(self, equation, flux, reconstruction, integrator, boundary, pool_bytes, max_members,
                 gamma=1.4, cfl=0.475, precision=FP64, dim=2):
        n = (8, 8 if dim > 1 else 1, 8 if dim > 2 else 1)
        self._desc, self._keep = make_desc(equation, flux, reconstruction, integrator, boundary, n, (0, 0, 0),
                                           (1, 1, 1), gamma=gamma, cfl=cfl, precision=precision)
        h = ctypes.c_void_p()
        _check(load().gbfv_batch_create(ctypes.byref(self._desc), int(pool_bytes), int(max_members),
                                        ctypes.byref(h)))
        self.h = h
        self.nvar = num_variables(equation)
        self.precision = precision

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def member_bytes(self, n):
        return _check(load().gbfv_batch_member_bytes(self.h, _c_int3(*n)))

    def free_bytes(self):
        t = ctypes.c_longlong()
        lg = ctypes.c_longlong()
        _check(load().gbfv_batch_free_bytes(self.h, ctypes.byref(t), ctypes.byref(lg)))
        return t.value, lg.value

    def add(self, n, lower, upper, prim, group=-1):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        slot = ctypes.c_int()
        _check(load().gbfv_batch_add(self.h, _c_int3(*n), _c_double3(*lower), _c_double3(*upper), _ptr(prim),
                                     int(group), ctypes.byref(slot)))
        return slot.value

    def remove(self, slot):
        _check(load().gbfv_batch_remove(self.h, int(slot)))

    def advance(self, end_time, number_of_saves=0, max_steps=0):
        _check(load().gbfv_batch_advance(self.h, end_time, number_of_saves, max_steps))

    def set_member_end(self, slot, end_time, number_of_saves=1):
        """The member's own end time (and save clamp)."""
        _check(load().gbfv_batch_set_member_end(self.h, int(slot), float(end_time), int(number_of_saves)))

    def set_member_write_interval(self, slot, interval):
        """The member's second save clamp (the fvm writer's interval)."""
        _check(load().gbfv_batch_set_member_write_interval(self.h, int(slot), float(interval)))

    def member_status(self, slot):
        """(status, failed step): 0 fine, 1 constraint check failed, 2 halo copy timed out."""
        st = ctypes.c_int()
        fs = ctypes.c_int()
        _check(load().gbfv_batch_member_status(self.h, int(slot), ctypes.byref(st), ctypes.byref(fs)))
        return st.value, fs.value

    def member_time(self, slot):
        t = ctypes.c_double()
        s = ctypes.c_longlong()
        _check(load().gbfv_batch_member_time(self.h, int(slot), ctypes.byref(t), ctypes.byref(s)))
        return t.value, s.value

    def member_state(self, slot, total):
        U = np.zeros((self.nvar, total))
        _check(load().gbfv_batch_member_state(self.h, int(slot), _ptr(U)))
        return U

    def stats(self, group, total):
        m = np.zeros((self.nvar, total))
        v = np.zeros((self.nvar, total))
        c = ctypes.c_longlong()
        _check(load().gbfv_batch_stats_result(self.h, int(group), _ptr(m), _ptr(v), ctypes.byref(c)))
        return m, v, c.value

    def stats_export(self, group, total, save=-1):
        """(count, mean, M2) of one group at statistics save `save` (-1: the
        last): the raw Welford triple for a cross-rank merge
        (alsvinn_gb300.uq.combine_statistics)."""
        m = np.zeros((self.nvar, total))
        q = np.zeros((self.nvar, total))
        c = ctypes.c_longlong()
        _check(load().gbfv_batch_stats_export_save(self.h, int(group), int(save), _ptr(m), _ptr(q), ctypes.byref(c)))
        return c.value, m, q

    def set_statistics_saves(self, saves):
        """Statistics at `saves` save times (before the first member joins)."""
        _check(load().gbfv_batch_set_statistics_saves(self.h, int(saves)))

    def stats_reset(self):
        _check(load().gbfv_batch_stats_reset(self.h))

    def launches(self):
        n = ctypes.c_longlong()
        _check(load().gbfv_batch_launches(self.h, ctypes.byref(n)))
        return n.value

    def stream(self):
        p = ctypes.c_void_p()
        _check(load().gbfv_batch_stream(self.h, ctypes.byref(p)))
        return p.value

    def select_candidate(self, idx):
        """Pins stage kernel candidate idx for the ensemble (-1: autotuner)."""
        _check(load().gbfv_batch_select_candidate(self.h, int(idx)))

    def current_candidate(self):
        """(candidate index, members staged by TMA)."""
        i, m = ctypes.c_int(), ctypes.c_int()
        _check(load().gbfv_batch_current_candidate(self.h, ctypes.byref(i), ctypes.byref(m)))
        return i.value, m.value

    def autotune_result(self, n=8):
        ms = (ctypes.c_double * n)()
        _check(load().gbfv_batch_autotune_result(self.h, ms, n))
        return list(ms)


REQUEST_BURGERS, REQUEST_KELVIN_HELMHOLTZ = 0, 1


class _Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("n", ctypes.c_int), ("end_time", ctypes.c_double),
                ("phase", ctypes.c_double), ("sample", ctypes.c_int), ("arrival", ctypes.c_double),
                ("keep", ctypes.c_int), ("initial_primitive", ctypes.c_void_p)]


_SIGNATURES.update({
    "gbfv_batch_finished": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int)]),
    "gbfv_batch_active": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "gbfv_server_create": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "gbfv_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbfv_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_int)]),
    "gbfv_server_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "gbfv_server_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)]),
    "gbfv_server_final_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong]),
    "gbfv_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_server_stats_at": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "gbfv_batch_set_member_end": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int]),
    "gbfv_batch_set_member_write_interval": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
    "gbfv_batch_member_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int)]),
    "gbfv_server_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
})


class Server:
    """Continuous-batching request loop (gbfv_server_*)."""

    def __init__(self, budget_bytes, precision=FP32, max_slots=4096):
        h = ctypes.c_void_p()
        _check(load().gbfv_server_create(int(budget_bytes), precision, int(max_slots), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().gbfv_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, kind, n, end_time, phase=0.0, sample=0, arrival=0.0, keep=False, initial=None):
        """Queues a request; `initial` (optional) is the caller's interior
        primitive initial data (copied at submission)."""
        buf = None
        if initial is not None:
            buf = np.ascontiguousarray(initial, dtype=np.float64)
        r = _Request(kind, n, end_time, phase, sample, arrival, 1 if keep else 0,
                     buf.ctypes.data if buf is not None else None)
        i = ctypes.c_int()
        _check(load().gbfv_server_submit(self.h, ctypes.byref(r), ctypes.byref(i)))
        return i.value

    def run(self, steps_per_chunk=16):
        _check(load().gbfv_server_run(self.h, int(steps_per_chunk)))

    def result(self, rid):
        a, ad, f = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        s = ctypes.c_longlong()
        st = ctypes.c_int()
        _check(load().gbfv_server_result(self.h, int(rid), ctypes.byref(a), ctypes.byref(ad), ctypes.byref(f),
                                         ctypes.byref(s), ctypes.byref(st)))
        return {"arrival": a.value, "admit": ad.value, "finish": f.value, "steps": s.value, "status": st.value}

    def final_state(self, rid, size):
        U = np.zeros(size)
        _check(load().gbfv_server_final_state(self.h, int(rid), _ptr(U), int(size)))
        return U

    def stats(self, kind, n, size, end_time=None):
        m = np.zeros(size)
        v = np.zeros(size)
        c = ctypes.c_longlong()
        if end_time is None:
            _check(load().gbfv_server_stats(self.h, int(kind), int(n), _ptr(m), _ptr(v), ctypes.byref(c)))
        else:
            _check(load().gbfv_server_stats_at(self.h, int(kind), int(n), float(end_time), _ptr(m), _ptr(v),
                                               ctypes.byref(c)))
        return m, v, c.value

    def launches(self):
        n = ctypes.c_longlong()
        _check(load().gbfv_server_launches(self.h, ctypes.byref(n)))
        return n.value
