"""Sample sharding of an ensemble over ranks and the cross-rank statistics
merge (alsvinn_gb300.uq), run as two gloo ranks on the CPU. The merged mean
and variance must equal the oracle's MeanVariance over all samples
(alsuq/src/stats/MeanVariance.cpp:30-67 with
alsuq/src/stats/StatisticsHelper.cpp:35-79), and every rank must hold the
same bits."""
import os
import socket

import numpy as np
import pytest

from alsvinn_gb300 import uq
from oracle import fvoracle


def _samples(count, cells, seed=11):
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, cells)
    out = []
    for _ in range(count):
        a, b, c = rng.uniform(-1, 1, 3)
        out.append(np.stack([1.0 + 0.1 * a * np.sin(2 * np.pi * (x + b)),
                             0.5 * c * np.cos(2 * np.pi * x),
                             2.5 + 0.05 * a * b * np.ones(cells)]))
    return out


def test_equal_blocks_follow_the_reference_balancer():
    assert uq.sample_blocks(12, 3) == [(0, 4), (4, 8), (8, 12)]
    assert uq.sample_blocks(0, 2) == [(0, 0), (0, 0)]
    with pytest.raises(ValueError):
        uq.sample_blocks(10, 3)


def test_cost_blocks_are_contiguous_and_balanced():
    rng = np.random.default_rng(3)
    sizes = rng.choice([128, 256, 512], size=101)
    costs = sizes.astype(np.float64) ** 3  # cells x steps, steps ~ n
    for world in (1, 2, 3, 4, 8):
        blocks = uq.sample_blocks(len(costs), world, costs)
        assert blocks[0][0] == 0 and blocks[-1][1] == len(costs)
        assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
        loads = [costs[s:e].sum() for s, e in blocks]
        assert max(loads) - costs.sum() / world <= costs.max()


def test_chan_merge_equals_one_pass():
    xs = np.stack([s.ravel() for s in _samples(9, 50)])
    whole = uq.welford(xs)
    parts = [uq.welford(xs[:2]), uq.welford(xs[2:7]), uq.welford(xs[7:])]
    merged = (0, np.zeros(xs.shape[1]), np.zeros(xs.shape[1]))
    for p in parts:
        merged = uq.chan_merge(merged, p)
    assert merged[0] == 9
    np.testing.assert_allclose(merged[1], whole[1], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(merged[2], whole[2], rtol=1e-12, atol=1e-15)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir, count, use_costs):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        samples = _samples(count, 64)
        costs = np.arange(1, count + 1, dtype=np.float64) if use_costs else None
        s, e = uq.sample_blocks(count, world, costs)[rank]
        local = np.stack([x.ravel() for x in samples[s:e]]) if e > s else np.zeros((0, samples[0].size))
        n, m, q = uq.welford(local) if e > s else (0, np.zeros(samples[0].size), np.zeros(samples[0].size))
        n, mean, var = uq.combine_statistics(n, m, q)
        np.savez(os.path.join(outdir, "rank%d.npz" % rank), n=n, mean=mean, var=var, block=(s, e))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("use_costs", [False, True])
def test_two_ranks_merge_to_the_oracle(tmp_path, use_costs):
    import torch.multiprocessing as mp
    count = 10
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path), count, use_costs), nprocs=2, join=True)
    r0 = np.load(tmp_path / "rank0.npz")
    r1 = np.load(tmp_path / "rank1.npz")
    assert int(r0["n"]) == int(r1["n"]) == count
    assert tuple(r0["block"])[1] == tuple(r1["block"])[0]
    # every rank holds the same bits
    assert np.array_equal(r0["mean"], r1["mean"]) and np.array_equal(r0["var"], r1["var"])
    m, v = fvoracle.meanvar([s.ravel() for s in _samples(count, 64)])
    np.testing.assert_allclose(r0["mean"], m, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(r0["var"], v, rtol=1e-9, atol=1e-15)
