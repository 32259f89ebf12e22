"""The error path of the bounded TMA halo wait, made to run out without any
fault: gbfv_test_tma_wait_limit makes the solver's TMA stage launches
announce more bytes on their halo barrier than the copies deliver, so every
wait reaches its time limit. The kernels record status 2 and return without
writing, the advance reports GBFV_ERR_CUDA, the state stays the one before
the step, and the context stays usable: the same solver, reset, and a new
one step on with the reference's bits."""
import numpy as np
import pytest

from alsvinn_gb300 import lib

pytestmark = pytest.mark.gpu

N = 64


def kh_solver():
    s = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0), (1, 1, 0), cfl=0.4,
                   precision=lib.FP64)
    s.set_primitive(lib.init_kelvin_helmholtz(N, sample=4))
    return s


def tma_candidate(s):
    for i, (tile, threads, tma) in enumerate(s.candidates()):
        if tma:
            return i
    pytest.skip("no TMA candidate for this scheme")


def test_halo_wait_runs_out_reports_and_leaves_the_context_usable(cuda_device):
    with kh_solver() as ref:
        ref.advance(1.0, 0, 3)
        expected = ref.get_state()
        t_expected = ref.time()[0]
    with kh_solver() as s:
        s.select_candidate(tma_candidate(s))
        s.advance(1.0, 0, 2)
        before = s.get_state()
        s.test_tma_wait_limit(16)
        with pytest.raises(lib.GbfvError) as e:
            s.advance(1.0, 0, 1)
        assert e.value.code == lib.ERR_CUDA
        assert "time limit" in str(e.value)
        # the timed-out stages wrote nothing
        assert np.array_equal(s.get_state(), before)
        # restored: from the state before the failed step, the step gives the reference's bits
        s.test_tma_wait_limit(0)
        s.set_state(before)
        s.advance(1.0, 0, 1)
        assert np.array_equal(s.get_state(), expected)
    # a new solver on the same context
    with kh_solver() as s2:
        s2.advance(1.0, 0, 3)
        assert np.array_equal(s2.get_state(), expected)
        assert s2.time()[0] == t_expected
