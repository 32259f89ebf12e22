"""The operator-level boundary on the reference's own Volume layout (one
device array per conserved variable), through the C ABI:

- region computeFlux (NumericalFlux::computeFlux with start / end) against
  the reference's own region calls (tests/golden/flux_region.npz, made by
  oracle/refbuild from the unmodified reference): the exact variant
  bit-identical on every cell and wave speed, the fast FP64 variant within
  1e-10 relative L1 on the region, cells outside the region untouched;
- ConservedSystem's split of a stage into the interior and 2 x dim side
  strips equals the whole-domain operator;
- the per-variable reconstruction / boundary / constraint / cell-map calls
  equal the block calls and the oracle;
- the device Memory arithmetic (Memory<real>'s operators, makeZero,
  addLinearCombination, addPower, subtractPower, getTotalVariation)
  against numpy restatements of the reference's HostMemory loops;
- one SSP-RK3 step driven the way the reference's RungeKutta3 and
  Simulator drive it (operator calls + Memory arithmetic + boundary) equals
  the fused device step bit for bit in the exact variant.
"""
import os

import numpy as np
import pytest

import workloads
from alsvinn_gb300 import lib
from conftest import interior
from oracle import fvoracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "flux_region.npz")
CASES = ["euler1_hll3_weno2", "burgers_godunov_eno3", "euler2_hll3_weno2", "euler2_hll_eno2", "euler3_hll3_weno2"]
DTYPE = {lib.FP64: np.float64, lib.FP64_EXACT: np.float64, lib.FP32: np.float32, lib.FP64_DF: np.float64}


def to_dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), device="cuda")


def var_tensors(U, dtype=np.float64):
    """One separate device array per variable (not one block)."""
    return [to_dev(np.asarray(U[k], dtype=dtype)) for k in range(U.shape[0])]


def ptrs(ts):
    return [t.data_ptr() for t in ts]


def host(ts):
    import torch
    torch.cuda.synchronize()
    return np.stack([t.cpu().numpy().astype(np.float64) for t in ts])


def solver(eq, fl, rc, n, precision=lib.FP64, boundary="periodic"):
    lower, upper = (0, 0, 0), (1, 1, 1)
    return lib.Solver(eq, fl, rc, "rungekutta3", boundary, n, lower, upper, gamma=1.4, cfl=0.4, precision=precision)


@pytest.mark.parametrize("precision", [lib.FP64_EXACT, lib.FP64])
@pytest.mark.parametrize("case", CASES)
def test_region_flux_matches_reference_region_calls(cuda_device, case, precision):
    import torch
    d = np.load(GOLDEN)
    eq, fl, rc = case.split("_")
    n = tuple(int(v) for v in d[case + "_n"])
    U, out0 = d[case + "_U"], d[case + "_out0"]
    g = workloads.ghost_cells(rc)
    with solver(eq, fl, rc, n, precision) as s:
        for k in range(int(d[case + "_regions"])):
            key = "%s_%d" % (case, k)
            start, end = [int(v) for v in d[key + "_start"]], [int(v) for v in d[key + "_end"]]
            ref, ws_ref = d[key + "_out"], d[key + "_ws"]
            uin, out = var_tensors(U), var_tensors(out0)
            torch.cuda.synchronize()
            ws = s.compute_flux_region(ptrs(uin), ptrs(out), start, end)
            got = host(out)
            if precision == lib.FP64_EXACT:
                assert np.array_equal(got, ref), key
                assert list(ws) == list(ws_ref), (key, ws, ws_ref)
            else:
                # only the region's cells change, as in the reference
                mask = ref != out0
                assert np.array_equal(got[~mask], out0[~mask]), key
                a = interior(got, n, g).reshape(got.shape[0], -1)
                b = interior(ref, n, g).reshape(ref.shape[0], -1)
                den = np.abs(b).sum(axis=1)
                err = np.abs(a - b).sum(axis=1) / np.where(den > 0, den, 1)
                assert (err <= 1e-10).all(), (key, err)
                assert np.allclose(ws, ws_ref, rtol=1e-12, atol=0), (key, ws, ws_ref)


def conserved_system_regions(n, g, dim):
    """The region calls of ConservedSystem::operator() (alsfvm/src/simulator/
    ConservedSystem.cpp:59-96) in interior coordinates: the interior, then
    per dimension the bottom and top strips."""
    regions = [([g if d < dim else 0 for d in range(3)], [-g if d < dim else 0 for d in range(3)])]
    for d in range(dim):
        hi = [0, 0, 0]
        hi[d] = -n[d] + g
        regions.append(([0, 0, 0], hi))
        lo = [0, 0, 0]
        lo[d] = n[d] - g
        regions.append((lo, [0, 0, 0]))
    return regions


@pytest.mark.parametrize("precision", [lib.FP64, lib.FP64_EXACT, lib.FP32, lib.FP64_DF])
@pytest.mark.parametrize("eq,n", [("euler1", (200, 1, 1)), ("euler2", (70, 45, 1)), ("euler3", (20, 18, 22))])
def test_conserved_system_split_equals_whole_domain(cuda_device, eq, n, precision):
    import torch
    rng = np.random.default_rng(7)
    g = 2
    t = workloads.padded_shape(n, g)
    U = workloads.smooth_random_state(eq, t, rng)
    dt = DTYPE[precision]
    with solver(eq, "hll3", "weno2", n, precision) as s:
        block = to_dev(U.astype(dt))
        full = torch.zeros_like(block)
        torch.cuda.synchronize()
        ws_full = s.compute_flux(block.data_ptr(), full.data_ptr())
        uin = var_tensors(U, dt)
        out = [torch.zeros_like(v) for v in uin]
        ws = [0.0, 0.0, 0.0]
        dim = workloads.dimension(n)
        for lo, hi in conserved_system_regions(n, g, dim):
            w = s.compute_flux_region(ptrs(uin), ptrs(out), lo, hi)
            ws = [max(a, b) for a, b in zip(ws, w)]
        torch.cuda.synchronize()
        got = interior(host(out), n, g)
        ref = interior(full.cpu().numpy().astype(np.float64), n, g)
    assert np.array_equal(got, ref)
    assert ws == list(ws_full)


def test_region_arguments_are_checked(cuda_device):
    import torch
    n = (32, 32, 1)
    U = workloads.smooth_random_state("euler2", workloads.padded_shape(n, 2), np.random.default_rng(1))
    with solver("euler2", "hll3", "weno2", n) as s:
        uin, out = var_tensors(U), var_tensors(U)
        torch.cuda.synchronize()
        for lo, hi in (([-1, 0, 0], [0, 0, 0]), ([0, 0, 0], [1, 0, 0]), ([0, 0, 1], [0, 0, 0])):
            with pytest.raises(lib.GbfvError) as e:
                s.compute_flux_region(ptrs(uin), ptrs(out), lo, hi)
            assert e.value.code == lib.ERR_ARGUMENT
        # an empty region computes nothing
        before = host(out)
        assert s.compute_flux_region(ptrs(uin), ptrs(out), [5, 0, 0], [-27, 0, 0]) == [0.0, 0.0, 0.0]
        assert np.array_equal(host(out), before)


@pytest.mark.parametrize("rc", ["weno2", "eno3", "none"])
def test_per_variable_calls_equal_block_calls(cuda_device, rc):
    import torch
    rng = np.random.default_rng(11)
    n = (40, 33, 1)
    g = workloads.ghost_cells(rc)
    t = workloads.padded_shape(n, g)
    U = workloads.smooth_random_state("euler2", t, rng)
    fill = rng.uniform(-1, 1, U.shape)
    with solver("euler2", "hll3", rc, n, boundary="neumann") as s:
        for direction in (0, 1):
            block = to_dev(U)
            bl, br = to_dev(fill), to_dev(fill)
            torch.cuda.synchronize()
            s.reconstruct(direction, block.data_ptr(), bl.data_ptr(), br.data_ptr())
            uin, l, r = var_tensors(U), var_tensors(fill), var_tensors(fill)
            torch.cuda.synchronize()
            s.reconstruct_vars(direction, ptrs(uin), ptrs(l), ptrs(r))
            assert np.array_equal(host(l), bl.cpu().numpy()) and np.array_equal(host(r), br.cpu().numpy())
            # a shifted range writes only its cells (NoReconstruction ignores the range)
            l2, r2 = var_tensors(fill), var_tensors(fill)
            torch.cuda.synchronize()
            s.reconstruct_vars(direction, ptrs(uin), ptrs(l2), ptrs(r2), [1, 2, 0], [-3, -1, 0])
            got = host(l2)
            if rc != "none":
                full = host(l)
                assert ((got == fill) | (got == full)).all()
                assert (got == fill).sum() > (full == fill).sum()
        # boundary and constraints
        block = to_dev(U)
        torch.cuda.synchronize()
        s.apply_boundary(block.data_ptr())
        vs = var_tensors(U)
        torch.cuda.synchronize()
        s.apply_boundary_vars(ptrs(vs))
        assert np.array_equal(host(vs), block.cpu().numpy())
        assert s.obeys_constraints_vars(ptrs(vs)) == s.obeys_constraints(block.data_ptr()) is True
        bad = U.copy()
        bad[0, t[0] * 5 + 7] = -1.0
        vb = var_tensors(bad)
        torch.cuda.synchronize()
        assert s.obeys_constraints_vars(ptrs(vb)) is False


@pytest.mark.parametrize("eq", ["euler1", "euler2", "euler3", "burgers"])
def test_cell_maps(cuda_device, eq):
    import torch
    rng = np.random.default_rng(5)
    n = {"euler1": (30, 1, 1), "euler2": (20, 17, 1), "euler3": (9, 8, 7), "burgers": (30, 1, 1)}[eq]
    g = 2
    t = workloads.padded_shape(n, g)
    nv = workloads.NVAR[eq]
    U = workloads.smooth_random_state(eq, t, rng)
    total = U.shape[1]
    with solver(eq, "godunov" if eq == "burgers" else "hll3", "weno2", n) as s:
        # conserved -> primitive on the host, then back on the device: the
        # oracle's computeFromPrimitive gives the bits
        if eq == "burgers":
            prim = U.copy()
        else:
            nsd = nv - 2
            u = U[1:1 + nsd] / U[0]
            p = 0.4 * (U[-1] - 0.5 * (U[1:1 + nsd] ** 2).sum(0) / U[0])
            prim = np.concatenate([U[:1], u, p[None]])
        pin, cout = var_tensors(prim), var_tensors(np.zeros_like(U))
        torch.cuda.synchronize()
        s.prim_to_cons_vars(ptrs(pin), ptrs(cout))
        ref = fvoracle.prim_to_cons(eq, n, g, 1.4, prim)
        assert np.array_equal(host(cout), ref)
        cin = var_tensors(U)
        torch.cuda.synchronize()
        if eq == "burgers":
            s.extra_variables_vars(ptrs(cin), [])
            for d in range(workloads.dimension(n)):
                assert s.max_wave_speed_vars(ptrs(cin), d) == np.abs(U[0]).max()
            return
        nsd = nv - 2
        extra = var_tensors(np.zeros((nsd + 1, total)))
        torch.cuda.synchronize()
        s.extra_variables_vars(ptrs(cin), ptrs(extra))
        E = host(extra)
        dot = U[1] * U[1]
        for k in range(2, 1 + nsd):
            dot = dot + U[k] * U[k]
        p = (1.4 - 1.0) * (U[-1] - 0.5 * dot / U[0])  # Euler::computeExtra, (gamma - 1) * ie
        assert np.array_equal(E[0], p)
        for k in range(nsd):
            assert np.array_equal(E[1 + k], U[1 + k] / U[0])
        for d in range(3):
            ud = U[1 + d] / U[0] if d < nsd else np.zeros(total)
            w = np.abs(ud) + np.sqrt(1.4 * p / U[0])
            assert s.max_wave_speed_vars(ptrs(cin), d) == pytest.approx(w.max(), rel=1e-15)


@pytest.mark.parametrize("precision", [lib.FP64, lib.FP32])
def test_memory_arithmetic(cuda_device, precision):
    import torch
    rng = np.random.default_rng(3)
    dt = np.float64 if precision == lib.FP64 else np.float32
    m = 10007
    a0 = rng.uniform(0.5, 2.0, m).astype(dt)
    b0 = rng.uniform(0.5, 2.0, m).astype(dt)
    for op, f in ((lib.MEMORY_ADD, np.add), (lib.MEMORY_SUBTRACT, np.subtract), (lib.MEMORY_MULTIPLY, np.multiply),
                  (lib.MEMORY_DIVIDE, np.divide)):
        a, b = to_dev(a0), to_dev(b0)
        torch.cuda.synchronize()
        lib.memory_op(op, a.data_ptr(), b.data_ptr(), m, precision)
        assert np.array_equal(host([a])[0], f(a0, b0).astype(np.float64)), op
        a = to_dev(a0)
        torch.cuda.synchronize()
        lib.memory_op_scalar(op, a.data_ptr(), 0.3, m, precision)
        # a double scalar: float elements are widened, operated on, rounded
        assert np.array_equal(host([a])[0], f(a0.astype(np.float64), 0.3).astype(dt).astype(np.float64)), op
    a = to_dev(a0)
    torch.cuda.synchronize()
    lib.memory_make_zero(a.data_ptr(), m, precision)
    assert not host([a]).any()
    # v1 = a1 v1 + a2 v2 + ... left to right, coefficients in the element type
    vs = [rng.uniform(-1, 1, m).astype(dt) for _ in range(5)]
    c = [dt(x) for x in (0.75, 0.25, -1.5, 2.0, 1.0 / 3.0)]
    ts = [to_dev(v) for v in vs]
    torch.cuda.synchronize()
    lib.memory_add_linear_combination(ts[0].data_ptr(), c[0], c[1], ts[1].data_ptr(), c[2], ts[2].data_ptr(), c[3],
                                      ts[3].data_ptr(), c[4], ts[4].data_ptr(), m, precision)
    ref = c[0] * vs[0] + c[1] * vs[1] + c[2] * vs[2] + c[3] * vs[3] + c[4] * vs[4]
    assert np.array_equal(host([ts[0]])[0], ref.astype(np.float64))
    # addPower / subtractPower with power 2 (MeanVariance) exact; power 3 to CUDA's pow bound
    for power, exact in ((2.0, True), (1.0, True), (3.0, False)):
        a, b = to_dev(a0), to_dev(b0)
        torch.cuda.synchronize()
        lib.memory_add_power(a.data_ptr(), b.data_ptr(), power, m, factor=0.5, precision=precision)
        ref = (a0.astype(np.float64) + 0.5 * np.power(b0.astype(np.float64), power)).astype(dt)
        got = host([a])[0]
        if exact:
            assert np.array_equal(got, ref.astype(np.float64)), power
        else:
            assert np.allclose(got, ref, rtol=4 * np.finfo(dt).eps, atol=0), power
        a = to_dev(a0)
        torch.cuda.synchronize()
        lib.memory_subtract_power(a.data_ptr(), b.data_ptr(), power, m, precision=precision)
        ref = (a0.astype(np.float64) - np.power(b0.astype(np.float64), power)).astype(dt)
        got = host([a])[0]
        if exact:
            assert np.array_equal(got, ref.astype(np.float64)), power
        else:
            assert np.allclose(got, ref, rtol=4 * np.finfo(dt).eps, atol=1e-12), power


def tv_reference(u, ext, p, direction, start, end):
    """HostMemory::getTotalVariation (alsfvm/src/memory/HostMemory.cpp:
    323-392) as loops: the isotropic form (direction -1, 1D / 2D) and the
    one-direction form."""
    nx, ny, nz = ext
    v = u.reshape(nz, ny, nx)
    s = 0.0
    if direction < 0:
        for z in range(0, end[2]):
            for y in range(start[1] + (1 if ny > 1 else 0), end[1]):
                for x in range(start[0] + 1, end[0]):
                    yb = y - 1 if ny > 1 else 0
                    dy = v[z, y, x] - v[z, yb, x]
                    dx = v[z, y, x] - v[z, y, x - 1]
                    s += (np.sqrt(dy ** 2 + dx ** 2)) ** p
        return s
    e = [0, 0, 0]
    e[direction] = 1
    for z in range(start[2] + e[2], end[2]):
        for y in range(start[1] + e[1], end[1]):
            for x in range(start[0] + e[0], end[0]):
                s += abs(v[z, y, x] - v[z - e[2], y - e[1], x - e[0]]) ** p
    return s


def test_memory_total_variation(cuda_device):
    import torch
    rng = np.random.default_rng(9)
    ext = (23, 19, 1)
    u = rng.uniform(-1, 1, ext[0] * ext[1])
    a = to_dev(u)
    torch.cuda.synchronize()
    for p in (1, 2, 3):
        for direction in (-1, 0, 1):
            start, end = (2, 2, 0), (21, 17, 1)
            got = lib.memory_total_variation(a.data_ptr(), ext, p, direction, start, end)
            ref = tv_reference(u, ext, p, direction, start, end)
            assert got == pytest.approx(ref, rel=1e-13), (p, direction)
    with pytest.raises(lib.GbfvError):
        lib.memory_total_variation(a.data_ptr(), (4, 4, 4), 1, -1, (0, 0, 0), (4, 4, 4))


@pytest.mark.parametrize("eq,n", [("euler2", (48, 48, 1)), ("euler3", (16, 16, 16))])
def test_reference_rk3_step_through_the_boundary_equals_the_fused_step(cuda_device, eq, n):
    """One SSP-RK3 step as the reference's Simulator and RungeKutta3 take it
    (alsfvm/src/simulator/Simulator.cpp:191-214, alsfvm/src/integrator/
    RungeKutta3.cpp:49-86, Integrator::computeTimestep Integrator.cpp:20-46):
    per stage the operator through ConservedSystem's region calls, then
    output *= dt / dx.x; output += U_s; the stage combinations; the boundary.
    In the exact variant this equals gbfv_advance's fused step bit for bit."""
    import torch
    g = 2
    if eq == "euler2":
        prim = lib.init_kelvin_helmholtz(n[0], sample=3)
        lower, upper = (0, 0, 0), (1, 1, 0)
    else:
        prim = lib.init_taylor_green(n[0])
        lower, upper = (0, 0, 0), (2 * np.pi,) * 3
    cfl = 0.4
    with lib.Solver(eq, "hll3", "weno2", "rungekutta3", "periodic", n, lower, upper, cfl=cfl,
                    precision=lib.FP64_EXACT) as s:
        s.set_primitive(prim)
        U0 = s.get_state()
        s.advance(1.0, 0, 1)
        fused = s.get_state()
        t_fused, _, dt_fused = s.time()
        nv, total = U0.shape
        cell_lengths = [(upper[d] - lower[d]) / n[d] if n[d] > 1 else 1.0 for d in range(3)]
        dim = workloads.dimension(n)
        regions = conserved_system_regions(n, g, dim)
        U = [var_tensors(U0)] + [[torch.zeros(total, dtype=torch.float64, device="cuda") for _ in range(nv)]
                                 for _ in range(3)]
        torch.cuda.synchronize()

        def operator(src, out):
            ws = [0.0, 0.0, 0.0]
            for lo, hi in regions:
                w = s.compute_flux_region(ptrs(src), ptrs(out), lo, hi)
                ws = [max(a, b) for a, b in zip(ws, w)]
            return ws

        dt = None
        for stage in range(3):
            out = U[stage + 1]
            ws = operator(U[stage], out)
            if stage == 0:
                total_ws = 0.0
                for d in range(3):
                    if cell_lengths[d] != 0:
                        total_ws += ws[d] / cell_lengths[d]
                dt = cfl / total_ws
            scale = dt / cell_lengths[0]
            for k in range(nv):
                o, us, u0 = out[k].data_ptr(), U[stage][k].data_ptr(), U[0][k].data_ptr()
                lib.memory_op_scalar(lib.MEMORY_MULTIPLY, o, scale, total)
                lib.memory_op(lib.MEMORY_ADD, o, us, total)
                if stage == 1:
                    lib.memory_op_scalar(lib.MEMORY_MULTIPLY, o, 1.0 / 3.0, total)
                    lib.memory_op(lib.MEMORY_ADD, o, u0, total)
                    lib.memory_op_scalar(lib.MEMORY_MULTIPLY, o, 3.0 / 4.0, total)
                elif stage == 2:
                    lib.memory_op_scalar(lib.MEMORY_MULTIPLY, o, 2.0, total)
                    lib.memory_op(lib.MEMORY_ADD, o, u0, total)
                    lib.memory_op_scalar(lib.MEMORY_MULTIPLY, o, 1.0 / 3.0, total)
            torch.cuda.synchronize()
            s.apply_boundary_vars(ptrs(out))
        stepped = host(U[3])
        assert s.obeys_constraints_vars(ptrs(U[3])) is True
    assert dt == dt_fused
    assert np.array_equal(stepped, fused)
