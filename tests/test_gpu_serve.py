"""The continuous-batching request loop (gbfv_server_*): requests that arrive
while others run are admitted into the running ensembles, each result is the
same alone and in the mix (bit for bit: the per-member arithmetic does not
depend on the other members), every request ends at its own end time,
admission respects the memory budget, every final state lands in its group's
statistics, and a request that fails leaves without stopping the others."""
import numpy as np
import pytest

from alsvinn_gb300 import lib

pytestmark = pytest.mark.gpu

B, KH = lib.REQUEST_BURGERS, lib.REQUEST_KELVIN_HELMHOLTZ
T_B, T_K = 0.1, 0.02


def size_of(kind, n):
    return n + 4 if kind == B else 4 * (n + 4) ** 2


def test_result_is_the_same_alone_and_in_the_mix(cuda_device):
    with lib.Server(2 << 30, precision=lib.FP32, max_slots=64) as s:
        xk = s.submit(KH, 96, T_K, sample=7, keep=True)
        xb = s.submit(B, 2048, T_B, phase=0.3, keep=True)
        s.run(8)
        alone_k = s.final_state(xk, size_of(KH, 96))
        alone_b = s.final_state(xb, size_of(B, 2048))
    with lib.Server(2 << 30, precision=lib.FP32, max_slots=64) as s:
        others = [s.submit(KH, n, T_K, sample=20 + i, arrival=0.0) for i, n in enumerate((64, 128, 64, 160))]
        others += [s.submit(B, n, T_B, phase=-0.5 + 0.1 * i, arrival=0.0) for i, n in enumerate((1024, 4096, 8192))]
        # x arrives while the others are in flight
        xk = s.submit(KH, 96, T_K, sample=7, arrival=0.05, keep=True)
        xb = s.submit(B, 2048, T_B, phase=0.3, arrival=0.05, keep=True)
        s.run(8)
        mixed_k = s.final_state(xk, size_of(KH, 96))
        mixed_b = s.final_state(xb, size_of(B, 2048))
        results = [s.result(i) for i in others + [xk, xb]]
    assert all(r["status"] == 2 for r in results)
    assert np.array_equal(alone_k, mixed_k)
    assert np.array_equal(alone_b, mixed_b)


def test_admission_waits_for_memory(cuda_device):
    # room for a single 256^2 KH member at a time: requests queue and run one
    # after another, all complete, none starts before the previous one ends
    b = lib.Batch("euler2", "hll3", "weno2", "rungekutta3", "periodic", 1 << 20, 1, precision=lib.FP32)
    per = b.member_bytes((256, 256, 1))
    b.close()
    # the 1D ensemble takes max(budget / 64, 16 MiB); the 2D one the rest
    budget = int(per * 1.5) + (16 << 20)
    with lib.Server(budget, precision=lib.FP32, max_slots=16) as s:
        ids = [s.submit(KH, 256, T_K, sample=i, arrival=0.0) for i in range(3)]
        s.run(8)
        res = [s.result(i) for i in ids]
    assert all(r["status"] == 2 for r in res)
    order = sorted(res, key=lambda r: r["admit"])
    for a, b2 in zip(order, order[1:]):
        assert b2["admit"] >= a["finish"] - 1e-6


def test_statistics_receive_every_request(cuda_device):
    with lib.Server(1 << 30, precision=lib.FP32, max_slots=32) as s:
        for i in range(5):
            s.submit(KH, 64, T_K, sample=i, arrival=0.01 * i)
        for i in range(3):
            s.submit(B, 1024, T_B, phase=0.2 * i - 0.2, arrival=0.0)
        s.run(8)
        _, _, ck = s.stats(KH, 64, size_of(KH, 64))
        mb, vb, cb = s.stats(B, 1024, size_of(B, 1024))
    assert ck == 5 and cb == 3
    assert np.isfinite(mb).all() and (vb >= 0).all()


def served_alone(kind, n, end_time, **kw):
    with lib.Server(1 << 30, precision=lib.FP32, max_slots=8) as s:
        i = s.submit(kind, n, end_time, keep=True, **kw)
        s.run(8)
        r = s.result(i)
        return s.final_state(i, size_of(kind, n)), r


def test_requests_have_their_own_end_times(cuda_device):
    # one grid per kind, several end times, all in flight together: each
    # request stops at its own end time with the bits it has alone
    kh = [(64, T_K, 3), (64, 0.5 * T_K, 4), (64, 1.5 * T_K, 5), (96, 0.75 * T_K, 6)]
    bu = [(1024, T_B, 0.2), (1024, 0.3 * T_B, -0.4), (2048, 0.6 * T_B, 0.7)]
    with lib.Server(2 << 30, precision=lib.FP32, max_slots=32) as s:
        ik = [s.submit(KH, n, T, sample=sm, arrival=0.01 * k, keep=True) for k, (n, T, sm) in enumerate(kh)]
        ib = [s.submit(B, n, T, phase=ph, arrival=0.01 * k, keep=True) for k, (n, T, ph) in enumerate(bu)]
        s.run(8)
        mixed = [(s.final_state(i, size_of(KH, n)), s.result(i)) for i, (n, _, _) in zip(ik, kh)]
        mixed += [(s.final_state(i, size_of(B, n)), s.result(i)) for i, (n, _, _) in zip(ib, bu)]
        # statistics groups are (kind, grid, end time)
        for n, T, _ in kh:
            assert s.stats(KH, n, size_of(KH, n), end_time=T)[2] == 1
        with pytest.raises(lib.GbfvError):
            s.stats(KH, 64, size_of(KH, 64))  # three end times share this grid
    alone = [served_alone(KH, n, T, sample=sm) for (n, T, sm) in kh]
    alone += [served_alone(B, n, T, phase=ph) for (n, T, ph) in bu]
    for (u_mix, r_mix), (u_alone, r_alone) in zip(mixed, alone):
        assert r_mix["status"] == r_alone["status"] == 2
        assert r_mix["steps"] == r_alone["steps"]
        assert np.array_equal(u_mix, u_alone)
    # the end time is the request's: a single-grid FP32 solve to it gives the bits
    n, T, sm = kh[1]
    with lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (n, n, 1), (0, 0, 0), (1, 1, 0),
                    cfl=0.4, precision=lib.FP32) as sv:
        sv.set_primitive(lib.init_kelvin_helmholtz(n, sample=sm))
        sv.advance(T, 1)
        t, steps, _ = sv.time()
        assert t == T and steps == mixed[1][1]["steps"]
        assert np.array_equal(sv.get_state().ravel(), mixed[1][0])


def test_a_failing_request_leaves_without_stopping_the_server(cuda_device):
    # a KH request whose initial pressure is negative in a patch breaks the
    # constraint check in its first step; it fails alone, the others finish
    # with the bits they have alone and only they enter the statistics
    n = 64
    bad = lib.init_kelvin_helmholtz(n, sample=9).reshape(4, n, n).copy()
    bad[3, 20:30, 20:30] = -1.0
    with lib.Server(2 << 30, precision=lib.FP32, max_slots=16) as s:
        good = [s.submit(KH, n, T_K, sample=k, arrival=0.0, keep=True) for k in range(3)]
        ib = s.submit(KH, n, T_K, arrival=0.0, initial=bad.ravel())
        later = s.submit(KH, n, T_K, sample=5, arrival=0.05, keep=True)
        burg = s.submit(B, 1024, T_B, phase=0.1, arrival=0.0, keep=True)
        s.run(8)
        res_bad = s.result(ib)
        states = [s.final_state(i, size_of(KH, n)) for i in good + [later]]
        res = [s.result(i) for i in good + [later, burg]]
        _, _, count = s.stats(KH, n, size_of(KH, n))
    assert res_bad["status"] == 3
    assert res_bad["steps"] <= 1
    assert all(r["status"] == 2 for r in res)
    assert count == 4
    for k, u in zip([0, 1, 2, 5], states):
        assert np.array_equal(u, served_alone(KH, n, T_K, sample=k)[0])
