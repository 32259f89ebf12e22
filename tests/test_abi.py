"""The C-ABI library loads, exports every entry point include/gbfv.h declares,
and its host-only entry points behave; no GPU needed."""
import os
import re

import numpy as np
import pytest

from alsvinn_gb300 import lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "gbfv.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\*)\s+(gbfv_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_function():
    L = lib.load()
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert names == lib.exported_names()


def test_ghost_cells_and_variables():
    assert [lib.ghost_cells(r) for r in ("none", "weno2", "eno2", "eno3", "eno4", "mc", "mm")] == \
        [1, 2, 2, 3, 4, 2, 2]
    assert [lib.num_variables(e) for e in ("burgers", "euler1", "euler2", "euler3")] == [1, 3, 4, 5]
    with pytest.raises(lib.GbfvError):
        lib.ghost_cells("weno9")


def test_generator_matches_reference_fixture():
    z = np.load(os.path.join(ROOT, "tests", "golden", "generator.npz"))
    for s in range(6):
        assert np.array_equal(lib.uniform(40, s), z["uniform40_s%d" % s])


@pytest.mark.parametrize("name", ("kh40_from0", "two_from0", "two_from5", "three_from2"))
def test_stateful_generator_matches_reference_fixture(name):
    """gbfv_generator driven in the Runner's order reproduces the reference's
    parameter draws bit for bit (host code: no GPU needed)."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "generator_sequence.npz"))
    dims, lo, hi = z[name + "_dims"], z[name + "_lower"], z[name + "_upper"]
    start, want = int(z[name + "_start"][0]), z[name]
    g = lib.Generator()
    got = []
    for s in range(start, start + want.shape[0]):
        row = []
        for p, d in enumerate(dims):
            row += [g.uniform(d, c, s, lo[p], hi[p]) for c in range(d)]
        got.append(row)
    g.close()
    assert np.array_equal(np.array(got), want)


def test_stateful_generator_rejects_bad_components():
    g = lib.Generator()
    with pytest.raises(lib.GbfvError):
        g.uniform(3, 3, 0)
    g.close()


def test_generator_scaling():
    a = lib.uniform(10, 3, 0.0, 1.0)
    b = lib.uniform(10, 3, -2.0, 5.0)
    assert np.array_equal(b, a * 7.0 + -2.0)


@pytest.mark.parametrize("field,value", [("equation", "euler4"), ("flux", "tecno1"), ("reconstruction", "weno9"),
                                         ("integrator", "rungekutta4"), ("boundary", "reflective")])
def test_create_rejects_unknown_names(field, value):
    kw = dict(equation="euler2", flux="hll3", reconstruction="weno2", integrator="rungekutta3",
              boundary="periodic", n=(8, 8, 1), lower=(0, 0, 0), upper=(1, 1, 0))
    kw[field] = value
    with pytest.raises(lib.GbfvError) as e:
        lib.Solver(**kw)
    assert e.value.code == lib.ERR_ARGUMENT


def test_create_rejects_mismatched_combinations():
    with pytest.raises(lib.GbfvError) as e:
        lib.Solver("burgers", "hll3", "weno2", "rungekutta3", "periodic", (8, 1, 1), (0, 0, 0), (1, 1, 1))
    assert e.value.code == lib.ERR_UNSUPPORTED
    with pytest.raises(lib.GbfvError) as e:
        lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (8, 1, 1), (0, 0, 0), (1, 1, 1))
    assert e.value.code == lib.ERR_UNSUPPORTED
    with pytest.raises(lib.GbfvError) as e:
        lib.Solver("euler1", "hll3", "eno4", "rungekutta3", "periodic", (3, 1, 1), (0, 0, 0), (1, 1, 1))
    assert e.value.code == lib.ERR_UNSUPPORTED
    # rusanov and roe are Burgers fluxes (numerical_flux_list.hpp)
    for flux in ("rusanov", "roe"):
        with pytest.raises(lib.GbfvError) as e:
            lib.Solver("euler1", flux, "mc", "rungekutta3", "periodic", (8, 1, 1), (0, 0, 0), (1, 1, 1))
        assert e.value.code == lib.ERR_UNSUPPORTED


def test_initial_data_matches_the_workload_formulas():
    """The library's initial data equal the formulas evaluated with Python's
    math module (the same C library), bit for bit."""
    import math

    import workloads
    assert np.array_equal(lib.init_sod(64), workloads.sod_prim(64))
    for s in (0, 3):
        assert np.array_equal(lib.init_kelvin_helmholtz(48, sample=s), workloads.kh_prim(48, lib.uniform(40, s)))
    assert np.array_equal(lib.init_taylor_green(6), workloads.tg_prim(6))
    assert np.array_equal(lib.init_burgers_sine(50, -0.37), workloads.burgers_prim(50, -0.37))
    assert math.pi == 3.141592653589793
