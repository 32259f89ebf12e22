"""ctypes binding of the CPU oracle (oracle/libfvoracle.so).

TEST INFRASTRUCTURE: imported only by tests/, the smoke check and the CPU
baseline leg of bench.py, as the checker. Signatures mirror oracle/fvoracle.h.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfvoracle.so")
D = ctypes.c_double
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import sys
            sys.path.insert(0, os.path.dirname(HERE))
            from alsvinn_gb300 import _build
            _build.build_oracle()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.fv_last_error.restype = ctypes.c_char_p
        _lib.fv_last_loop_seconds.restype = ctypes.c_double
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _i3(v):
    return (ctypes.c_int * 3)(*v)


def _d3(v):
    return (ctypes.c_double * 3)(*v)


def _check(rc):
    if rc < 0:
        raise RuntimeError("oracle: " + load().fv_last_error().decode())
    return rc


def set_threads(n):
    load().fv_set_threads(int(n))


def get_threads():
    return load().fv_get_threads()


def ghost_cells(recon):
    return _check(load().fv_ghost_cells(recon.encode()))


def boundary(bc, n, ghosts, U):
    U = np.ascontiguousarray(U, dtype=np.float64).copy()
    _check(load().fv_boundary(bc.encode(), _i3(n), ghosts, U.shape[0], _p(U)))
    return U


def compute_flux(equation, flux, recon, n, gamma, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    out = np.zeros_like(U)
    ws = (D * 3)()
    _check(load().fv_compute_flux(equation.encode(), flux.encode(), recon.encode(), _i3(n), D(gamma), _p(U),
                                  _p(out), ws))
    return out, list(ws)


def reconstruct(equation, recon, n, gamma, direction, U, left=None, right=None):
    U = np.ascontiguousarray(U, dtype=np.float64)
    left = np.zeros_like(U) if left is None else left.copy()
    right = np.zeros_like(U) if right is None else right.copy()
    _check(load().fv_reconstruct(equation.encode(), recon.encode(), _i3(n), D(gamma), direction, _p(U),
                                 _p(left), _p(right)))
    return left, right


def run(equation, flux, recon, integrator, bc, n, lower, upper, gamma, cfl, end_time, number_of_saves,
        max_steps, prim, ghosts, nvar):
    dim = 3 if n[2] > 1 else (2 if n[1] > 1 else 1)
    t = [n[d] + 2 * ghosts if d < dim else n[d] for d in range(3)]
    out = np.zeros((nvar, t[0] * t[1] * t[2]))
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    tt = D()
    st = ctypes.c_int()
    rc = load().fv_run(equation.encode(), flux.encode(), recon.encode(), integrator.encode(), bc.encode(),
                       _i3(n), _d3(lower), _d3(upper), D(gamma), D(cfl), D(end_time), number_of_saves,
                       max_steps, _p(prim), _p(out), ctypes.byref(tt), ctypes.byref(st), None, 0)
    return rc, out, tt.value, st.value


def last_loop_seconds():
    """Seconds the last run() spent in its step loop (setup excluded)."""
    return load().fv_last_loop_seconds()


def prim_to_cons(equation, n, ghosts, gamma, prim_padded):
    prim_padded = np.ascontiguousarray(prim_padded, dtype=np.float64)
    out = np.zeros_like(prim_padded)
    _check(load().fv_prim_to_cons(equation.encode(), _i3(n), ghosts, D(gamma), _p(prim_padded), _p(out)))
    return out


def obeys_constraints(equation, n, ghosts, gamma, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    return bool(_check(load().fv_obeys_constraints(equation.encode(), _i3(n), ghosts, D(gamma), _p(U))))


def uniform(dimension, sample, lower=0.0, upper=1.0):
    out = np.zeros(dimension)
    _check(load().fv_uniform(dimension, sample, D(lower), D(upper), _p(out)))
    return out


def generate_sequence(dims, sample_start, nsamples, lowers=None, uppers=None):
    """Runner-order parameter draws: array (nsamples, sum(dims))."""
    dims = [int(d) for d in dims]
    lowers = np.zeros(len(dims)) if lowers is None else np.asarray(lowers, dtype=np.float64)
    uppers = np.ones(len(dims)) if uppers is None else np.asarray(uppers, dtype=np.float64)
    out = np.zeros((nsamples, sum(dims)))
    di = (ctypes.c_int * len(dims))(*dims)
    _check(load().fv_generate_sequence(len(dims), di, _p(np.ascontiguousarray(lowers)),
                                       _p(np.ascontiguousarray(uppers)), ctypes.c_longlong(sample_start),
                                       ctypes.c_longlong(nsamples), _p(out)))
    return out


def structure_cube(equation, boundary, n, ghosts, number_of_h, p, U):
    """One sample's cube structure function: (nvar, number_of_h)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    out = np.zeros((U.shape[0], number_of_h))
    _check(load().fv_structure_cube(equation.encode(), boundary.encode(), _i3(n), int(ghosts), int(number_of_h),
                                    D(p), _p(U), _p(out)))
    return out


VARIABLE_NAMES = {"burgers": ["u"], "euler1": ["rho", "mx", "E"], "euler2": ["rho", "mx", "my", "E"],
                  "euler3": ["rho", "mx", "my", "mz", "E"]}


def variable_mask(equation, variables):
    """Bit mask of the named variables ("rho E"); 0 (all) for an empty list."""
    names = VARIABLE_NAMES[equation]
    mask = 0
    for v in (variables.split() if isinstance(variables, str) else list(variables or [])):
        mask |= 1 << names.index(v)
    return mask


def functional(name, equation, boundary, n, ghosts, lower, upper, U, weight=1.0, degree=0, min_value=0.0,
               max_value=1.0, variables="", gamma=1.4, p=1.0, number_of_h=1, direction=0):
    """weight times functional `name` of one padded state (structure_cube:
    the functional itself, which ignores the weight); returns (values
    (nvar, output cells), output extents)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    nv = U.shape[0]
    size = (ctypes.c_int * 3)()
    cap = max(int(np.prod(n)), int(number_of_h), 1)
    buf = np.zeros(nv * cap)
    _check(load().fv_functional(name.encode(), equation.encode(), boundary.encode(), _i3(n), int(ghosts), _d3(lower),
                                _d3(upper), int(degree), D(min_value), D(max_value),
                                ctypes.c_uint(variable_mask(equation, variables)), D(gamma), D(p), int(number_of_h),
                                int(direction), D(weight), _p(U), _p(buf), size))
    cells = size[0] * size[1] * size[2]
    return buf[:nv * cells].reshape(nv, cells), tuple(size)


def structure_basic(equation, boundary, n, ghosts, number_of_h, p, direction, U):
    """One sample's axis structure function (StructureBasic): (nvar, number_of_h)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    out = np.zeros((U.shape[0], number_of_h))
    _check(load().fv_structure_basic(equation.encode(), boundary.encode(), _i3(n), int(ghosts), int(number_of_h),
                                     D(p), int(direction), _p(U), _p(out)))
    return out


def meanvar(samples):
    samples = [np.ascontiguousarray(s, dtype=np.float64) for s in samples]
    count = samples[0].size
    arr = (ctypes.c_void_p * len(samples))(*[s.ctypes.data for s in samples])
    m = np.zeros(samples[0].shape)
    v = np.zeros(samples[0].shape)
    _check(load().fv_meanvar(ctypes.c_long(count), len(samples), arr, _p(m), _p(v)))
    return m, v
