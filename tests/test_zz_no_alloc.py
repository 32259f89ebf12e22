"""gbfv_advance_noalloc, the entry point for callers that cannot call
cudaMalloc (memory owned by a pool or arena they do not expose, plug-ins that
may not allocate after start-up, fixed memory budgets). It must give the same
states as gbfv_advance through a solver, bit for bit (both run the same
default stage kernels), call after call, with its scratch in the library's
static device array, and a call must leave the device's free memory as it
found it. This file is collected last on purpose."""
import numpy as np
import pytest

import workloads
from alsvinn_gb300 import lib

pytestmark = pytest.mark.gpu

CASES = {
    # name: (equation, flux, recon, integrator, boundary, n, lower, upper, cfl)
    "kh64_rk3": ("euler2", "hll3", "weno2", "rungekutta3", "periodic", (64, 64, 1), (0, 0, 0), (1, 1, 0), 0.4),
    "sod256_rk2_eno3": ("euler1", "hll", "eno3", "rungekutta2", "neumann", (256, 1, 1), (-5, 0, 0), (5, 1, 1),
                        0.475),
    "burgers2d_fe": ("burgers", "godunov", "eno2", "forwardeuler", "periodic", (48, 40, 1), (0, 0, 0),
                     (1, 1, 1), 0.4),
}


def prim_for(name, n):
    if name.startswith("kh"):
        return workloads.kh_prim(n[0], lib.uniform(40, 2))
    if name.startswith("sod"):
        return workloads.sod_prim(n[0])
    return np.sin(np.arange(n[0] * n[1]) * 0.07).reshape(1, -1) * 0.5


@pytest.mark.parametrize("precision", [lib.FP64, lib.FP32])
@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_solver_on_consecutive_calls(cuda_device, name, precision):
    import torch

    eq, fl, rc, integ, bc, n, lo, hi, cfl = CASES[name]
    prim = prim_for(name, n)
    with lib.Solver(eq, fl, rc, integ, bc, n, lo, hi, cfl=cfl, precision=precision) as s:
        s.set_primitive(prim)
        U0 = s.get_state()
        expected = []
        for _ in range(2):
            s.advance(2.0, 0, 4)
            t, steps, _ = s.time()
            expected.append((s.get_state(), t, steps))

    desc, keep = lib.make_desc(eq, fl, rc, integ, bc, n, lo, hi, cfl=cfl, precision=precision)
    dtype = torch.float64 if precision == lib.FP64 else torch.float32
    state = torch.from_numpy(U0.copy()).to(dtype).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    t, steps = 0.0, 0
    for call, (want, t_want, steps_want) in enumerate(expected):
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        t, steps = lib.advance_noalloc(desc, state.data_ptr(), t, steps, 2.0, 0, 4, stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        got = state.cpu().numpy().astype(np.float64)
        assert steps == steps_want
        assert t == t_want
        # the same default stage kernels as the solver: the same bits
        assert np.array_equal(got, want)
        if call > 0:
            # once the library's kernels are loaded (the first call), a call
            # takes no device memory
            assert free_after == free_before


def test_noalloc_rejects_grids_beyond_its_scratch(cuda_device):
    import torch

    n = (1024, 1024, 1)  # two 4-variable FP64 states need ~68 MB > 32 MiB
    desc, keep = lib.make_desc("euler2", "hll3", "weno2", "rungekutta3", "periodic", n, (0, 0, 0), (1, 1, 0))
    state = torch.zeros(8, device="cuda", dtype=torch.float64)
    with pytest.raises(lib.GbfvError) as e:
        lib.advance_noalloc(desc, state.data_ptr(), 0.0, 0, 1.0, 0, 1, None)
    assert e.value.code == lib.ERR_UNSUPPORTED
    assert "scratch" in str(e.value)
