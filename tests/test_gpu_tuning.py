"""Stage kernel candidates, TMA halo staging and the autotuner on the GPU.

Every candidate of a scheme (tile shape, cells per thread, TMA or per-thread
halo loads) computes each cell with the same arithmetic in the same order, so
its states must be bit-identical to candidate 0's; candidate 0 of the exact
variant is itself bit-identical to the oracle (test_gpu_parity), which makes
every exact candidate bit-identical to the oracle. Grids include ragged sizes
(tiles hanging over the upper edge, where the TMA box reads past the padded
array) and sizes whose padded rows break the TMA alignment rule.
"""
import numpy as np
import pytest

import workloads
from alsvinn_gb300 import lib
from oracle import fvoracle

pytestmark = pytest.mark.gpu

KH_X = np.random.default_rng(7).uniform(0.0, 1.0, 40)


def smooth_prim(eq, n, seed=3):
    """Interior primitive variables (rho, u..., p) or (u) on grid n: smooth
    waves in every direction plus 1% noise (positive density and pressure)."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    wave = np.sin(0.41 * x + 0.2) + np.cos(0.33 * y + 0.5) + np.sin(0.29 * z + 1.1)
    nv = workloads.NVAR[eq]
    if eq == "burgers":
        return (0.3 * wave + rng.uniform(-0.01, 0.01, x.size))[None, :]
    prim = np.zeros((nv, x.size))
    prim[0] = 1.5 + 0.15 * wave + rng.uniform(0, 0.01, x.size)
    for k in range(nv - 2):
        prim[1 + k] = 0.2 * np.sin(0.37 * x + 0.23 * y + 0.7 * k) + rng.uniform(-0.01, 0.01, x.size)
    prim[-1] = 1.5 + 0.15 * np.cos(0.23 * x + 0.31 * y + 0.17 * z) + rng.uniform(0, 0.01, x.size)
    return prim


# (equation, flux, integrator, boundary, n, lower, upper, primitive data)
CASES = {
    "kh2d": ("euler2", "hll3", "rungekutta3", "periodic", (96, 96, 1), (0, 0, 0), (1, 1, 0),
             lambda n: workloads.kh_prim(n[0], KH_X)),
    "ragged2d": ("euler2", "hll3", "rungekutta3", "neumann", (100, 70, 1), (0, 0, 0), (1, 0.7, 0),
                 lambda n: smooth_prim("euler2", n)),
    "sod1d": ("euler1", "hll3", "rungekutta3", "neumann", (500, 1, 1), (-5, 0, 0), (5, 1, 1),
              lambda n: workloads.sod_prim(n[0])),
    "ragged3d": ("euler3", "hll3", "rungekutta3", "periodic", (20, 24, 12), (0, 0, 0), (1, 1.2, 0.6),
                 lambda n: smooth_prim("euler3", n)),
    "burgers1d_rk2": ("burgers", "godunov", "rungekutta2", "periodic", (1000, 1, 1), (0, 0, 0), (1, 1, 1),
                      lambda n: workloads.burgers_prim(n[0], 0.3)),
}
PRECISIONS = {"fp64": lib.FP64, "fp64_exact": lib.FP64_EXACT, "fp32": lib.FP32}
STEPS = 6


def _solver(case, precision):
    eq, flux, integ, bc, n, lo, hi, prim = CASES[case]
    s = lib.Solver(eq, flux, "weno2", integ, bc, n, lo, hi, cfl=0.4, precision=precision)
    s.set_primitive(np.asarray(prim(n), dtype=np.float64).reshape(s.nvar, -1))
    return s


def _run(case, precision, cand):
    s = _solver(case, precision)
    try:
        s.select_candidate(cand)
        s.advance(1e9, 0, STEPS)
        assert s.current_candidate() == cand
        t, steps, _ = s.time()
        assert steps == STEPS
        return s.get_state(), t
    finally:
        s.close()


@pytest.mark.parametrize("precision", sorted(PRECISIONS) + ["fp64_df"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_every_candidate_is_bit_identical(cuda_device, case, precision):
    if precision == "fp64_df" and case not in ("kh2d", "ragged2d"):
        pytest.skip("the double-float variant has tuning candidates for 2D only")
    prec = lib.FP64_DF if precision == "fp64_df" else PRECISIONS[precision]
    s = _solver(case, prec)
    cands = s.candidates()
    s.close()
    assert len(cands) > 1, "the tuned schemes have several candidates"
    # TMA staging copies the storage type: not for the double-float variant
    assert cands[0][2] is False and (any(c[2] for c in cands[1:]) == (precision != "fp64_df"))
    ref, t_ref = _run(case, prec, 0)
    for i in range(1, len(cands)):
        got, t = _run(case, prec, i)
        assert t == t_ref, (case, precision, cands[i])
        assert np.array_equal(got, ref), (case, precision, cands[i])


@pytest.mark.parametrize("case", ["ragged2d", "ragged3d"])
def test_exact_candidates_match_the_oracle(cuda_device, case):
    """Ragged grids with every exact candidate against the oracle run (tiles
    over the upper edge: the zero-filled part of a TMA box must not leak)."""
    eq, flux, integ, bc, n, lo, hi, prim = CASES[case]
    nv = workloads.NVAR[eq]
    p = np.asarray(prim(n), dtype=np.float64).reshape(nv, -1)
    rc, U, t, steps = fvoracle.run(eq, flux, "weno2", integ, bc, n, lo, hi, 1.4, 0.4, 1e9, 0, STEPS, p, 2, nv)
    assert rc == 0 and steps == STEPS
    s = _solver(case, lib.FP64_EXACT)
    k = len(s.candidates())
    s.close()
    for i in range(k):
        got, tt = _run(case, lib.FP64_EXACT, i)
        assert tt == t
        assert np.array_equal(got, U.reshape(got.shape)), i


def test_tma_needs_aligned_rows(cuda_device):
    """FP32 with 101 cells per row: padded rows of 105 * 4 bytes break the
    16-byte rule, so TMA candidates are refused and the autotuner skips them."""
    s = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (101, 40, 1), (0, 0, 0), (1, 1, 0),
                   cfl=0.4, precision=lib.FP32)
    try:
        s.set_primitive(smooth_prim("euler2", (101, 40, 1)))
        cands = s.candidates()
        for i, c in enumerate(cands):
            if c[2]:
                with pytest.raises(lib.GbfvError):
                    s.select_candidate(i)
        chosen, ms = s.autotune()
        assert chosen == 0
        assert ms[0] > 0 and all(m == -1 for m, c in zip(ms, cands) if c[2])
        s.advance(1e9, 0, 2)
    finally:
        s.close()


def test_autotuner_times_every_eligible_candidate(cuda_device):
    s = _solver("kh2d", lib.FP64)
    try:
        assert s.current_candidate() == -1
        chosen, ms = s.autotune()
        assert 0 <= chosen < len(ms)
        assert all(m > 0 for m in ms)
        assert ms[chosen] == min(ms)
        assert s.current_candidate() == chosen
        s.advance(1e9, 0, 2)
        # a second solver of the same scheme and grid reuses the cached choice
        s2 = _solver("kh2d", lib.FP64)
        s2.advance(1e9, 0, 1)
        assert s2.current_candidate() == chosen
        s2.close()
    finally:
        s.close()


@pytest.mark.parametrize("precision", [lib.FP64, lib.FP32])
def test_autotuning_leaves_the_solve_untouched(cuda_device, precision):
    """The tuner's launches write only scratch (L, V, a scratch step state):
    tuning first and then stepping equals stepping with the chosen
    candidate pinned from the start."""
    s = _solver("kh2d", precision)
    try:
        chosen, _ = s.autotune()
        s.advance(1e9, 0, STEPS)
        tuned = s.get_state()
    finally:
        s.close()
    s = _solver("kh2d", precision)
    try:
        s.select_candidate(chosen)
        s.advance(1e9, 0, STEPS)
        assert np.array_equal(s.get_state(), tuned)
    finally:
        s.close()


def _ensemble(precision, sizes, cand):
    b = lib.Batch("euler2", "hll3", "weno2", "rungekutta3", "periodic", 256 << 20, len(sizes), cfl=0.4,
                  precision=precision)
    try:
        if cand is not None:
            b.select_candidate(cand)
        slots = []
        for k, m in enumerate(sizes):
            n = (m, m, 1)
            X = np.random.default_rng(100 + k).uniform(0.0, 1.0, 40)
            slots.append(b.add(n, (0, 0, 0), (1, 1, 0), np.asarray(workloads.kh_prim(m, X)).reshape(4, -1)))
        b.advance(0.01, 0, STEPS)
        cur = b.current_candidate()
        out = []
        for sl, m in zip(slots, sizes):
            total = (m + 4) * (m + 4)
            out.append((b.member_time(sl), b.member_state(sl, total)))
        return cur, out
    finally:
        b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp64_df"])
def test_ensemble_candidates_are_bit_identical(cuda_device, precision):
    prec = lib.FP64_DF if precision == "fp64_df" else PRECISIONS[precision]
    # 62: FP32 padded rows of 66 * 4 bytes break the TMA rule; that member
    # keeps per-thread loads inside a TMA candidate
    sizes = [64, 96, 40, 62] if precision == "fp32" else [64, 96, 40]
    s = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (64, 64, 1), (0, 0, 0), (1, 1, 0),
                   precision=prec)
    cands = s.candidates()
    s.close()
    (c0, _), ref = _ensemble(prec, sizes, 0)
    assert c0 == 0
    for i in range(1, len(cands)):
        (ci, tma_members), got = _ensemble(prec, sizes, i)
        assert ci == i
        if cands[i][2]:
            assert tma_members == len(sizes) - (1 if precision == "fp32" else 0)
        for (tg, sg), (tr, sr) in zip(got, ref):
            assert tg == tr, (i, cands[i])
            assert np.array_equal(sg, sr), (i, cands[i])


@pytest.mark.parametrize("case,integ", [("kh2d", None), ("burgers1d_rk2", None), ("sod1d", "forwardeuler")])
def test_step_graph_replay_matches_direct_launches(cuda_device, case, integ):
    """Advances of 16 steps and more replay a captured graph of 16 steps;
    with profiling on, every kernel is launched directly. Both must give
    the same bits, the same time and step count, whether the advance stops
    on a step limit or inside a replayed group at its end time."""
    eq, flux, integ0, bc, n, lo, hi, prim = CASES[case]
    integ = integ or integ0
    out = []
    for direct in (False, True):
        s = lib.Solver(eq, flux, "weno2", integ, bc, n, lo, hi, cfl=0.4, precision=lib.FP64)
        try:
            s.set_primitive(np.asarray(prim(n), dtype=np.float64).reshape(s.nvar, -1))
            s.profile(direct)
            s.advance(1e9, 0, 100)
            t1, steps1, _ = s.time()
            assert steps1 == 100
            # an end time 37.5 steps further on: the advance ends inside a group
            s.advance(t1 + 37.5 * (t1 / steps1), 0, 0)
            out.append((s.get_state(), s.time()[:2], t1))
        finally:
            s.close()
    (a, ta, t1a), (b, tb, t1b) = out
    assert t1a == t1b and ta == tb
    assert np.array_equal(a, b)


def test_small_grids_keep_the_default_without_tuning(cuda_device):
    """Below 4096 interior cells the first advance keeps candidate 0 and
    launches no tuning kernels (a few CTAs per stage time alike): the same
    kernel launches as a solve with candidate 0 pinned. An explicit
    gbfv_autotune still tunes."""
    launches = []
    for pin in (False, True):
        s = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (32, 32, 1), (0, 0, 0), (1, 1, 0),
                       cfl=0.4, precision=lib.FP64)
        try:
            s.set_primitive(workloads.kh_prim(32, lib.uniform(40, 0)))
            if pin:
                s.select_candidate(0)
            s.profile(True)
            _, _, k0 = s.profile_read()
            s.advance(1e9, 0, 5)
            _, _, k1 = s.profile_read()
            assert s.current_candidate() == 0
            launches.append(k1 - k0)
            if not pin:
                chosen, ms = s.autotune()
                assert all(m > 0 for m in ms)
        finally:
            s.close()
    assert launches[0] == launches[1], launches
