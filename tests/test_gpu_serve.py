"""The continuous-batching request loop (gbfv_server_*): requests that arrive
while others run are admitted into the running ensembles, each result is the
same alone and in the mix (bit for bit: the per-member arithmetic does not
depend on the other members), admission respects the memory budget, and every
final state lands in its group's statistics."""
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


def test_requests_of_one_kind_share_the_end_time(cuda_device):
    with lib.Server(1 << 30, precision=lib.FP32, max_slots=8) as s:
        s.submit(KH, 64, T_K)
        with pytest.raises(lib.GbfvError) as e:
            s.submit(KH, 64, 2 * T_K)
        assert e.value.code == lib.ERR_UNSUPPORTED
