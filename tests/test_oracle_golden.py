"""The CPU oracle against fixtures generated from the reference's own CPU
implementation (tests/golden/make_golden.py): every comparison is bit-exact."""
import os

import numpy as np
import pytest

import workloads
from oracle import fvoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name))


FLUX_GRIDS = {"euler1": (24, 1, 1), "euler2": (10, 9, 1), "euler3": (9, 8, 8), "burgers": (24, 1, 1)}


def flux_keys():
    """(fixture file, equation_flux_reconstruction) pairs: the base schemes
    and the extra fluxes / limiter reconstructions."""
    out = []
    for name in ("flux.npz", "flux_extra.npz"):
        z = load(name)
        out += [(name, k) for k in sorted({k.rsplit("_", 1)[0] for k in z.files})]
    return out


@pytest.mark.parametrize("name,key", flux_keys())
def test_flux_matches_reference(name, key):
    z = load(name)
    eq, fl, rc = key.split("_")
    out, ws = fvoracle.compute_flux(eq, fl, rc, FLUX_GRIDS[eq], 1.4, z[key + "_U"])
    assert np.isfinite(out).all()
    assert np.array_equal(out, z[key + "_L"])
    assert ws == list(z[key + "_ws"])


def test_boundary_matches_reference():
    z = load("boundary.npz")
    for key in z.files:
        bc, dims, g = key.split("_")
        n = tuple(int(v) for v in dims.split("x"))
        g = int(g[1:])
        t = workloads.padded_shape(n, g)
        tot = t[0] * t[1] * t[2]
        U = np.arange(tot, dtype=np.float64).reshape(1, tot) + 0.25
        assert np.array_equal(fvoracle.boundary(bc, n, g, U), z[key]), key


def test_generator_matches_reference():
    z = load("generator.npz")
    for s in range(6):
        assert np.array_equal(fvoracle.uniform(40, s), z["uniform40_s%d" % s])


def test_meanvar_matches_reference():
    z = load("meanvar.npz")
    m, v = fvoracle.meanvar(list(z["samples"]))
    assert np.array_equal(m, z["mean"])
    assert np.array_equal(v, z["var"])


@pytest.mark.parametrize("name", sorted(workloads.GOLDEN_RUNS))
def test_run_matches_reference(name):
    z = load("runs.npz")
    case = workloads.GOLDEN_RUNS[name]
    g = workloads.ghost_cells(case["recon"])
    rc, U, t, steps = fvoracle.run(case["equation"], case["flux"], case["recon"], case["integrator"],
                                   case["boundary"], case["n"], case["lower"], case["upper"], case["gamma"],
                                   case["cfl"], case["end_time"], case["number_of_saves"], case["max_steps"],
                                   z[name + "_prim"], g, workloads.NVAR[case["equation"]])
    assert rc == 0
    assert steps == int(z[name + "_steps"][0])
    assert t == float(z[name + "_t"][0])
    assert np.array_equal(U, z[name + "_U"])


def test_fixture_initial_data_is_reproducible():
    """The stored initial data equal the workload formulas evaluated here."""
    z = load("runs.npz")
    for name, case in workloads.GOLDEN_RUNS.items():
        assert np.array_equal(case["prim"](), z[name + "_prim"]), name


def test_constraint_violation_is_reported():
    n = (16, 1, 1)
    prim = workloads.sod_prim(16)
    prim[2, 7] = -1.0  # negative pressure
    rc, U, t, steps = fvoracle.run("euler1", "hll3", "weno2", "rungekutta3", "neumann", n, (-5, 0, 0), (5, 1, 1),
                                   1.4, 0.475, 1.0, 0, 5, prim, 2, 3)
    assert rc == -2
    assert steps == 1


SEQUENCE_CASES = ("kh40_from0", "two_from0", "two_from5", "three_from2")


@pytest.mark.parametrize("name", SEQUENCE_CASES)
def test_generator_sequence_matches_reference(name):
    """The Runner's stateful draws (several parameters on one engine, a rank
    starting mid-way) from the oracle equal the reference's."""
    z = load("generator_sequence.npz")
    out = fvoracle.generate_sequence(z[name + "_dims"], int(z[name + "_start"][0]), z[name].shape[0],
                                     z[name + "_lower"], z[name + "_upper"])
    assert np.array_equal(out, z[name])


STRUCTURE_CASES = {
    # name: (equation, boundary, n, ghosts, number_of_h, p), as tests/golden/make_golden.py
    "burgers_periodic_p2": ("burgers", "periodic", (20, 1, 1), 2, 6, 2.0),
    "euler1_neumann_p1": ("euler1", "neumann", (16, 1, 1), 3, 5, 1.0),
    "euler2_periodic_p3": ("euler2", "periodic", (12, 10, 1), 2, 5, 3.0),
    "euler2_neumann_p2_5": ("euler2", "neumann", (9, 11, 1), 1, 4, 2.5),
    "euler3_periodic_p2": ("euler3", "periodic", (6, 5, 4), 2, 4, 2.0),
    "burgers2d_neumann_p4": ("burgers", "neumann", (8, 7, 1), 2, 5, 4.0),
}


@pytest.mark.parametrize("name", sorted(STRUCTURE_CASES))
def test_structure_cube_matches_reference(name):
    z = load("structure.npz")
    eq, bc, n, g, H, p = STRUCTURE_CASES[name]
    out = fvoracle.structure_cube(eq, bc, n, g, H, p, z[name + "_U"])
    assert np.array_equal(out, z[name + "_S"])


# ---------------------------------------------------------------- functionals

FUNCTIONAL_CASES = workloads.FUNCTIONAL_CASES
BV_DIRECTION_CASES = workloads.BV_DIRECTION_CASES


@pytest.mark.parametrize("name", sorted(FUNCTIONAL_CASES))
def test_oracle_functionals_match_the_reference(name):
    """The CPU functionals (Identity, Moment, LegendrePointWise, LogEntropy,
    BoundedVariation, StructureCube) of the reference's own build."""
    z = np.load(os.path.join(GOLDEN, "functional.npz"))
    fn, eq, bc, n, g, lo, hi, prm, w = FUNCTIONAL_CASES[name]
    got, size = fvoracle.functional(fn, eq, bc, n, g, lo, hi, z[name + "_U"], weight=w, **prm)
    assert tuple(z[name + "_size"]) == size
    # the reference's operations in its loop order, the same libm: bit for bit
    assert np.array_equal(got, z[name + "_out"]), np.abs(got - z[name + "_out"]).max()


@pytest.mark.parametrize("name", sorted(BV_DIRECTION_CASES))
def test_oracle_total_variation_per_direction(name):
    z = np.load(os.path.join(GOLDEN, "functional.npz"))
    eq, n, g, d, p = BV_DIRECTION_CASES[name]
    got, _ = fvoracle.functional("bv_direction", eq, "periodic", n, g, (0, 0, 0), (1, 1, 1),
                                 z["bvdir_" + name + "_U"], degree=p, direction=d)
    assert np.array_equal(got[:, 0], z["bvdir_" + name + "_out"])


@pytest.mark.parametrize("name", sorted(workloads.STRUCTURE_BASIC_CASES))
def test_oracle_structure_basic_matches_the_reference(name):
    """StructureBasic (alsuq/src/stats/StructureBasic.cpp) of the reference's own build."""
    z = np.load(os.path.join(GOLDEN, "structure_basic.npz"))
    eq, bc, n, g, H, p, d = workloads.STRUCTURE_BASIC_CASES[name]
    got = fvoracle.structure_basic(eq, bc, n, g, H, p, d, z[name + "_U"])
    assert np.array_equal(got, z[name + "_S"]), np.abs(got - z[name + "_S"]).max()
