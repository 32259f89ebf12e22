"""Generates the golden fixtures in this directory from the reference's own
CPU implementation, built unmodified from its sources by oracle/refbuild
(make -C oracle/refbuild REF=<path to alsvinn>) into oracle/_ref/libalsref.so.

Run once from the repository root:  python tests/golden/make_golden.py
The fixtures are small .npz files; the tests compare the C oracle (and through
it the CUDA path) against them, so they pin the oracle to the reference itself.
The generator draws must be requested in increasing sample order in one fresh
process (the reference's mt19937_64 is process-wide).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import workloads  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libalsref.so")
R = ctypes.CDLL(LIB)
R.ref_last_error.restype = ctypes.c_char_p
D = ctypes.c_double


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def i3(v):
    return (ctypes.c_int * 3)(*v)


def d3(v):
    return (ctypes.c_double * 3)(*v)


def check(rc):
    if rc != 0:
        raise RuntimeError(R.ref_last_error().decode())


def padded_shape(n, g):
    dim = 3 if n[2] > 1 else (2 if n[1] > 1 else 1)
    return [n[d] + 2 * g if d < dim else n[d] for d in range(3)]


def flux_cases():
    rng = np.random.default_rng(20240601)
    out = {}
    grids = {"euler1": (24, 1, 1), "euler2": (10, 9, 1), "euler3": (9, 8, 8), "burgers": (24, 1, 1)}
    fluxes = {"euler1": ["hll", "hll3"], "euler2": ["hll", "hll3"], "euler3": ["hll", "hll3"],
              "burgers": ["godunov"]}
    for eq, n in grids.items():
        for fl in fluxes[eq]:
            for rc in workloads.RECONSTRUCTIONS:
                g = workloads.ghost_cells(rc)
                t = padded_shape(n, g)
                U = workloads.smooth_random_state(eq, t, rng)
                o = np.zeros_like(U)
                ws = (D * 3)()
                check(R.ref_compute_flux(eq.encode(), fl.encode(), rc.encode(), i3(n), D(1.4), P(U), P(o), ws))
                key = f"{eq}_{fl}_{rc}"
                out[key + "_U"] = U
                out[key + "_L"] = o
                out[key + "_ws"] = np.array(list(ws))
    np.savez_compressed(os.path.join(HERE, "flux.npz"), **out)


def region_cases():
    """Region calls of the reference's NumericalFlux (start / end), the calls
    ConservedSystem makes for the interior and the side strips plus boxes of
    other shapes; `out` starts from one random fill per case (out0), which
    cells outside the region keep."""
    rng = np.random.default_rng(20240615)
    out = {}
    cases = [("euler1", "hll3", "weno2", (24, 1, 1)), ("burgers", "godunov", "eno3", (21, 1, 1)),
             ("euler2", "hll3", "weno2", (14, 11, 1)), ("euler2", "hll", "eno2", (12, 10, 1)),
             ("euler3", "hll3", "weno2", (8, 7, 6))]
    for eq, fl, rc, n in cases:
        g = workloads.ghost_cells(rc)
        dim = workloads.dimension(n)
        t = padded_shape(n, g)
        U = workloads.smooth_random_state(eq, t, rng)
        o0 = rng.uniform(-1, 1, U.shape)
        regions = [([g if d < dim else 0 for d in range(3)], [-g if d < dim else 0 for d in range(3)])]
        for d in range(dim):
            # ConservedSystem's strips (ConservedSystem.cpp:67-96), in interior coordinates
            hi = [0, 0, 0]
            hi[d] = -n[d] + g
            regions.append(([0, 0, 0], hi))
            lo = [0, 0, 0]
            lo[d] = n[d] - g
            regions.append((lo, [0, 0, 0]))
        regions.append(([1 if d < dim else 0 for d in range(3)], [-2 if d < dim else 0 for d in range(3)]))
        regions.append(([0, 0, 0], [0, 0, 0]))
        case = f"{eq}_{fl}_{rc}"
        out[case + "_U"] = U
        out[case + "_out0"] = o0
        out[case + "_n"] = np.array(n)
        out[case + "_regions"] = np.array(len(regions))
        for k, (lo, hi) in enumerate(regions):
            o = o0.copy()
            ws = (D * 3)()
            check(R.ref_compute_flux_region(eq.encode(), fl.encode(), rc.encode(), i3(n), D(1.4), P(U), P(o), ws,
                                            i3(lo), i3(hi)))
            key = f"{case}_{k}"
            out[key + "_out"] = o
            out[key + "_ws"] = np.array(list(ws))
            out[key + "_start"] = np.array(lo)
            out[key + "_end"] = np.array(hi)
    np.savez_compressed(os.path.join(HERE, "flux_region.npz"), **out)


def extra_flux_combinations():
    """(equation, flux, reconstruction) pairs beyond the base set: the extra
    fluxes with every reconstruction, the limiters with every base flux."""
    out = []
    for eq in ("euler1", "euler2", "euler3", "burgers"):
        extra_rc = workloads.LIMITER_RECONSTRUCTIONS + (workloads.EULER_RECONSTRUCTIONS if eq != "burgers" else [])
        for fl in workloads.EXTRA_FLUXES[eq]:
            for rc in workloads.RECONSTRUCTIONS + extra_rc:
                out.append((eq, fl, rc))
        for fl in workloads.BASE_FLUXES[eq]:
            for rc in extra_rc:
                out.append((eq, fl, rc))
    return out


def flux_extra_cases():
    rng = np.random.default_rng(20240602)
    out = {}
    grids = {"euler1": (24, 1, 1), "euler2": (10, 9, 1), "euler3": (9, 8, 8), "burgers": (24, 1, 1)}
    for eq, fl, rc in extra_flux_combinations():
        n = grids[eq]
        g = workloads.ghost_cells(rc)
        t = padded_shape(n, g)
        U = workloads.smooth_random_state(eq, t, rng)
        o = np.zeros_like(U)
        ws = (D * 3)()
        check(R.ref_compute_flux(eq.encode(), fl.encode(), rc.encode(), i3(n), D(1.4), P(U), P(o), ws))
        key = f"{eq}_{fl}_{rc}"
        out[key + "_U"] = U
        out[key + "_L"] = o
        out[key + "_ws"] = np.array(list(ws))
    np.savez_compressed(os.path.join(HERE, "flux_extra.npz"), **out)


STRUCTURE_CASES = {
    # name: (equation, boundary, n, ghosts, number_of_h, p)
    "burgers_periodic_p2": ("burgers", "periodic", (20, 1, 1), 2, 6, 2.0),
    "euler1_neumann_p1": ("euler1", "neumann", (16, 1, 1), 3, 5, 1.0),
    "euler2_periodic_p3": ("euler2", "periodic", (12, 10, 1), 2, 5, 3.0),
    "euler2_neumann_p2_5": ("euler2", "neumann", (9, 11, 1), 1, 4, 2.5),
    "euler3_periodic_p2": ("euler3", "periodic", (6, 5, 4), 2, 4, 2.0),
    "burgers2d_neumann_p4": ("burgers", "neumann", (8, 7, 1), 2, 5, 4.0),
}


def functional_cases():
    rng = np.random.default_rng(20241203)
    out = {}
    for name, (fn, eq, bc, n, g, lo, hi, prm, w) in workloads.FUNCTIONAL_CASES.items():
        t = padded_shape(n, g)
        U = workloads.smooth_random_state(eq, t, rng)
        nv = workloads.NVAR[eq]
        size = (ctypes.c_int * 3)()
        o = np.zeros(nv * int(np.prod(n)) + nv * 64)
        check(R.ref_functional(fn.encode(), eq.encode(), bc.encode(), i3(n), g, d3(lo), d3(hi),
                               int(prm.get("degree", 0)), D(prm.get("min_value", 0.0)),
                               D(prm.get("max_value", 1.0)), prm.get("variables", "").encode(),
                               D(prm.get("gamma", 1.4)), D(prm.get("p", 1.0)), int(prm.get("number_of_h", 1)),
                               D(w), P(U), P(o), size))
        cells = size[0] * size[1] * size[2]
        out[name + "_U"] = U
        out[name + "_out"] = o[:nv * cells].reshape(nv, cells)
        out[name + "_size"] = np.array(list(size))
    for name, (eq, n, g, d, p) in workloads.BV_DIRECTION_CASES.items():
        t = padded_shape(n, g)
        U = workloads.smooth_random_state(eq, t, rng)
        nv = workloads.NVAR[eq]
        o = np.zeros(nv)
        check(R.ref_total_variation_direction(eq.encode(), i3(n), g, d, p, P(U), P(o)))
        out["bvdir_" + name + "_U"] = U
        out["bvdir_" + name + "_out"] = o
    np.savez_compressed(os.path.join(HERE, "functional.npz"), **out)


def structure_basic_cases():
    rng = np.random.default_rng(20241204)
    out = {}
    for name, (eq, bc, n, g, H, p, d) in workloads.STRUCTURE_BASIC_CASES.items():
        t = padded_shape(n, g)
        U = workloads.smooth_random_state(eq, t, rng)
        nv = workloads.NVAR[eq]
        o = np.zeros((nv, H))
        check(R.ref_structure_basic(eq.encode(), bc.encode(), i3(n), g, H, D(p), d, P(U), P(o)))
        out[name + "_U"] = U
        out[name + "_S"] = o
    np.savez_compressed(os.path.join(HERE, "structure_basic.npz"), **out)


def structure_cases():
    rng = np.random.default_rng(20240603)
    out = {}
    for name, (eq, bc, n, g, H, p) in STRUCTURE_CASES.items():
        t = padded_shape(n, g)
        U = workloads.smooth_random_state(eq, t, rng)
        nv = workloads.NVAR[eq]
        o = np.zeros((nv, H))
        check(R.ref_structure_cube(eq.encode(), bc.encode(), i3(n), g, H, D(p), P(U), P(o)))
        out[name + "_U"] = U
        out[name + "_S"] = o
    np.savez_compressed(os.path.join(HERE, "structure.npz"), **out)


def boundary_cases():
    out = {}
    for bc in ("neumann", "periodic"):
        for n in ((7, 1, 1), (6, 5, 1), (5, 6, 4)):
            for g in (1, 2, 3, 4):
                t = padded_shape(n, g)
                if any(t[d] < 2 * g for d in range(3) if n[d] > 1):
                    continue
                tot = t[0] * t[1] * t[2]
                U = np.arange(tot, dtype=np.float64).reshape(1, tot) + 0.25
                check(R.ref_boundary(bc.encode(), i3(n), g, 1, P(U)))
                out[f"{bc}_{n[0]}x{n[1]}x{n[2]}_g{g}"] = U
    np.savez_compressed(os.path.join(HERE, "boundary.npz"), **out)


def generator_cases():
    out = {}
    for s in range(6):
        a = np.zeros(40)
        check(R.ref_uniform(40, s, D(0.0), D(1.0), P(a)))
        out[f"uniform40_s{s}"] = a
    np.savez_compressed(os.path.join(HERE, "generator.npz"), **out)


# (dims per parameter in name order, lowers, uppers, first sample, samples):
# the Runner's draws on a fresh process-wide engine, as one rank sees them
SEQUENCE_CASES = {
    "kh40_from0": ([40], [0.0], [1.0], 0, 5),
    "two_from0": ([3, 7], [0.0, 0.0], [1.0, 1.0], 0, 4),
    "two_from5": ([3, 7], [0.0, 0.0], [1.0, 1.0], 5, 3),
    "three_from2": ([10, 1, 4], [-1.0, 0.0, 2.0], [1.0, 5.0, 3.0], 2, 3),
}


def _sequence_case(name, path):
    dims, lo, hi, start, n = SEQUENCE_CASES[name]
    out = np.zeros((n, sum(dims)))
    di = (ctypes.c_int * len(dims))(*dims)
    check(R.ref_generate_sequence(len(dims), di, P(np.array(lo)), P(np.array(hi)), ctypes.c_longlong(start),
                                  ctypes.c_longlong(n), P(out)))
    np.save(path, out)


def generator_sequence_cases():
    import subprocess
    import tempfile
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (dims, lo, hi, start, n) in SEQUENCE_CASES.items():
            path = os.path.join(tmp, name + ".npy")
            # a fresh process per case: the reference's engine is process-wide
            subprocess.run([sys.executable, os.path.abspath(__file__), "--sequence", name, path], check=True,
                           timeout=300)
            out[name] = np.load(path)
            out[name + "_dims"] = np.array(dims)
            out[name + "_lower"] = np.array(lo)
            out[name + "_upper"] = np.array(hi)
            out[name + "_start"] = np.array([start])
    np.savez_compressed(os.path.join(HERE, "generator_sequence.npz"), **out)


def meanvar_cases():
    rng = np.random.default_rng(7)
    n, g = (8, 6, 1), 2
    tot = 12 * 10
    S = [rng.uniform(0.5, 2.0, (4, tot)) for _ in range(9)]
    arr = (ctypes.c_void_p * len(S))(*[P(s) for s in S])
    m = np.zeros((4, tot))
    v = np.zeros((4, tot))
    check(R.ref_meanvar(b"euler2", i3(n), g, len(S), arr, P(m), P(v)))
    np.savez_compressed(os.path.join(HERE, "meanvar.npz"), samples=np.array(S), mean=m, var=v)


def run_cases():
    out = {}
    for name, case in workloads.GOLDEN_RUNS.items():
        prim = case["prim"]()
        g = workloads.ghost_cells(case["recon"])
        t = padded_shape(case["n"], g)
        nv = workloads.NVAR[case["equation"]]
        U = np.zeros((nv, t[0] * t[1] * t[2]))
        tt = D()
        st = ctypes.c_int()
        check(R.ref_run(case["equation"].encode(), case["flux"].encode(), case["recon"].encode(),
                        case["integrator"].encode(), case["boundary"].encode(), i3(case["n"]),
                        d3(case["lower"]), d3(case["upper"]), D(case["gamma"]), D(case["cfl"]),
                        D(case["end_time"]), case["number_of_saves"], case["max_steps"], P(prim), P(U),
                        ctypes.byref(tt), ctypes.byref(st), None, 0))
        out[name + "_prim"] = prim
        out[name + "_U"] = U
        out[name + "_t"] = np.array([tt.value])
        out[name + "_steps"] = np.array([st.value])
    np.savez_compressed(os.path.join(HERE, "runs.npz"), **out)


if __name__ == "__main__" and len(sys.argv) == 4 and sys.argv[1] == "--sequence":
    _sequence_case(sys.argv[2], sys.argv[3])
elif __name__ == "__main__":
    R.ref_set_threads(4)
    generator_cases()
    generator_sequence_cases()
    flux_cases()
    region_cases()
    flux_extra_cases()
    structure_cases()
    structure_basic_cases()
    functional_cases()
    boundary_cases()
    meanvar_cases()
    run_cases()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
