"""Cube structure functions on the GPU (gbfv_structure_*) against the
reference's own StructureCube kernel (golden fixtures from the reference
build): one sample, the mean of two samples, FP32 states."""
import os

import numpy as np
import pytest

from alsvinn_gb300 import lib
from test_oracle_golden import STRUCTURE_CASES

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def dev(a, dtype=np.float64):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


@pytest.mark.parametrize("name", sorted(STRUCTURE_CASES))
def test_structure_cube_matches_reference(cuda_device, name):
    z = np.load(os.path.join(GOLDEN, "structure.npz"))
    eq, bc, n, g, H, p = STRUCTURE_CASES[name]
    U, want = z[name + "_U"], z[name + "_S"]
    st = lib.Structure(bc, n, g, U.shape[0], H, p)
    u = dev(U)
    st.add_device(u.data_ptr(), lib.FP64)
    got, count = st.result()
    assert count == 1
    # the reference sums term by term in cell order; the device sums per
    # cell, then per block, then the blocks in order
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)
    # a second sample: the mean of the two
    st.add_device(dev(2.0 * U).data_ptr(), lib.FP64)
    got2, count = st.result()
    assert count == 2
    np.testing.assert_allclose(got2, want * (1 + 2.0 ** p) / 2, rtol=1e-12, atol=1e-15)
    n_, sums = st.export()
    assert n_ == 2
    np.testing.assert_allclose(sums, want * (1 + 2.0 ** p), rtol=1e-12, atol=1e-15)
    st.close()


def test_structure_cube_of_fp32_states(cuda_device):
    z = np.load(os.path.join(GOLDEN, "structure.npz"))
    name = "euler2_periodic_p3"
    eq, bc, n, g, H, p = STRUCTURE_CASES[name]
    U = z[name + "_U"].astype(np.float32)
    st = lib.Structure(bc, n, g, U.shape[0], H, p)
    st.add_device(dev(U, np.float32).data_ptr(), lib.FP32)
    got, _ = st.result()
    np.testing.assert_allclose(got, z[name + "_S"], rtol=1e-5, atol=1e-7)
    st.close()


def test_structure_arguments_are_checked():
    with pytest.raises(lib.GbfvError):
        lib.Structure("reflective", (8, 8, 1), 2, 4, 4, 2.0)
    with pytest.raises(lib.GbfvError):
        lib.Structure("periodic", (8, 8, 1), 2, 4, 0, 2.0)
