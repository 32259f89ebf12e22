"""Device functionals against the oracle (which the CPU suite pins to the
reference's own functionals, tests/golden/functional.npz): the pointwise
ones bit for bit, the sums (log entropy, total variation) and pow-based ones
to rounding, in FP64 and from FP32 states."""
import numpy as np
import pytest

import workloads
from alsvinn_gb300 import lib
from oracle import fvoracle

pytestmark = pytest.mark.gpu

def _golden():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "functional.npz"))


def _device(torch, U, precision):
    dt = torch.float32 if precision == lib.FP32 else torch.float64
    return torch.tensor(U, dtype=dt, device="cuda").contiguous()


@pytest.mark.parametrize("name", sorted(workloads.FUNCTIONAL_CASES))
def test_functional_matches_the_oracle(cuda_device, name):
    import torch
    z = _golden()
    fn, eq, bc, n, g, lo, hi, prm, w = workloads.FUNCTIONAL_CASES[name]
    U = z[name + "_U"]
    want = z[name + "_out"]
    f = lib.Functional(fn, eq, bc, n, g, lo, hi, **prm)
    try:
        assert f.size == tuple(z[name + "_size"])
        d = _device(torch, U, lib.FP64)
        f.apply(d.data_ptr(), lib.FP64, w)
        got = f.result()
        if fn in ("identity", "legendre_pointwise"):
            assert np.array_equal(got, want)
        else:
            np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-15)
        # accumulation: a second application adds (structure_cube replaces)
        f.apply(d.data_ptr(), lib.FP64, w)
        twice = f.result()
        np.testing.assert_allclose(twice, want if fn == "structure_cube" else 2 * want, rtol=1e-13, atol=1e-15)
        f.reset()
        assert not f.result().any()
        # an FP32 state: the functional of the rounded state, in FP64
        U32 = U.astype(np.float32)
        want32, _ = fvoracle.functional(fn, eq, bc, n, g, lo, hi, U32.astype(np.float64), weight=w, **prm)
        f.apply(_device(torch, U32, lib.FP32).data_ptr(), lib.FP32, w)
        np.testing.assert_allclose(f.result(), want32, rtol=1e-12, atol=1e-14)
    finally:
        f.close()


@pytest.mark.parametrize("name", sorted(workloads.BV_DIRECTION_CASES))
def test_total_variation_per_direction(cuda_device, name):
    import torch
    z = _golden()
    eq, n, g, d, p = workloads.BV_DIRECTION_CASES[name]
    f = lib.Functional("bv_direction", eq, "periodic", n, g, (0, 0, 0), (1, 1, 1), degree=p, direction=d)
    try:
        f.apply(_device(torch, z["bvdir_" + name + "_U"], lib.FP64).data_ptr())
        np.testing.assert_allclose(f.result()[:, 0], z["bvdir_" + name + "_out"], rtol=1e-13)
    finally:
        f.close()


def test_functional_errors_follow_the_reference(cuda_device):
    import torch
    with pytest.raises(lib.GbfvError):
        lib.Functional("tecno_entropy", "euler2", "periodic", (8, 8, 1), 2, (0, 0, 0), (1, 1, 0))
    # Legendre is 2D only; log entropy needs Euler; bv is 1D / 2D
    with pytest.raises(lib.GbfvError):
        lib.Functional("legendre_pointwise", "burgers", "periodic", (16, 1, 1), 2, (0, 0, 0), (1, 1, 1), degree=2)
    with pytest.raises(lib.GbfvError):
        lib.Functional("log_entropy", "burgers", "periodic", (16, 1, 1), 2, (0, 0, 0), (1, 1, 1))
    with pytest.raises(lib.GbfvError):
        lib.Functional("bv", "euler3", "periodic", (4, 4, 4), 2, (0, 0, 0), (1, 1, 1), degree=1)
    with pytest.raises(lib.GbfvError):
        lib.Functional("legendre_pointwise", "euler2", "periodic", (4, 4, 1), 2, (0, 0, 0), (1, 1, 0),
                       variables="rho pressure")
    # values outside [minValue, maxValue]: the reference's Boost domain error
    f = lib.Functional("legendre_pointwise", "euler2", "periodic", (4, 4, 1), 2, (0, 0, 0), (1, 1, 0), degree=2,
                       min_value=0.0, max_value=0.5)
    try:
        U = workloads.smooth_random_state("euler2", (8, 8, 1), np.random.default_rng(1))
        with pytest.raises(lib.GbfvError):
            f.apply(_device(torch, U, lib.FP64).data_ptr())
    finally:
        f.close()
