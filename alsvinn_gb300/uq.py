"""Sample sharding and the cross-rank statistics merge of an ensemble run.

An ensemble shards by samples: every rank (one GPU each) runs a contiguous
block of sample indices through its own `Batch`, accumulates FP64 Welford
triples (count, mean, M2) per grid size, and the triples of all ranks are
combined once at the end. No state crosses ranks during the run.

Reference counterparts:
  * alsuq/src/mpi/SimpleLoadBalancer.cpp:63-97 - contiguous blocks of
    totalNumberOfSamples / processes sample indices per statistical rank; the
    count must divide evenly (alsuq/src/mpi/SimpleLoadBalancer.cpp:44-60).
  * alsuq/src/stats/StatisticsHelper.cpp:35-79 - MPI_Reduce(SUM) of the
    per-rank sums u and u^2 to rank 0, then division by the sample count.
    Here the per-rank Welford triples are all-gathered and folded with Chan et
    al.'s pairwise update in rank order, so every rank ends with the same,
    bit-identical result and no cancellation-prone sum of squares.
"""
import numpy as np


def sample_blocks(num_samples, world_size, costs=None):
    """Contiguous [start, end) sample blocks, one per rank.

    Without `costs` the blocks have equal counts and `num_samples` must be a
    multiple of `world_size`, as in the reference load balancer. With `costs`
    (one positive number per sample, e.g. cells x steps) the cut points follow
    the prefix sums so that each block carries about 1/world_size of the
    total cost; blocks stay contiguous and in sample order.
    """
    if world_size < 1:
        raise ValueError("world_size must be positive")
    if num_samples < 0:
        raise ValueError("num_samples must be non-negative")
    if costs is None:
        if num_samples % world_size != 0:
            raise ValueError("the number of samples (%d) must be a multiple of the number of ranks (%d)"
                             % (num_samples, world_size))
        per = num_samples // world_size
        return [(r * per, (r + 1) * per) for r in range(world_size)]
    c = np.asarray(costs, dtype=np.float64)
    if c.shape != (num_samples,):
        raise ValueError("costs needs one entry per sample")
    if num_samples and not (c > 0).all():
        raise ValueError("costs must be positive")
    prefix = np.concatenate(([0.0], np.cumsum(c)))
    total = prefix[-1]
    cuts = [0]
    for r in range(1, world_size):
        target = total * r / world_size
        # first boundary whose prefix reaches the target, nearer side wins
        k = int(np.searchsorted(prefix, target))
        if 0 < k <= num_samples and target - prefix[k - 1] < prefix[k] - target:
            k -= 1
        cuts.append(min(max(k, cuts[-1]), num_samples))
    cuts.append(num_samples)
    return [(cuts[r], cuts[r + 1]) for r in range(world_size)]


def welford(samples):
    """(count, mean, M2) of the rows of `samples` (shape (count, cells)) by
    Welford's update in row order; a host-side triple for tests and for
    statistics gathered on the host."""
    x = np.asarray(samples, dtype=np.float64)
    mean = np.zeros(x.shape[1:])
    m2 = np.zeros(x.shape[1:])
    for i, v in enumerate(x, start=1):
        d = v - mean
        mean = mean + d / i
        m2 = m2 + d * (v - mean)
    return x.shape[0], mean, m2


def chan_merge(a, b):
    """Pairwise merge of two Welford triples (Chan, Golub, LeVeque 1979):
    n = na + nb, delta = mean_b - mean_a, mean = mean_a + delta nb / n,
    M2 = M2_a + M2_b + delta^2 na nb / n. An empty side returns the other."""
    na, ma, qa = a
    nb, mb, qb = b
    if nb == 0:
        return na, ma, qa
    if na == 0:
        return nb, mb, qb
    n = na + nb
    delta = mb - ma
    return n, ma + delta * (nb / n), qa + qb + delta * delta * (na * nb / n)


def combine_statistics(count, mean, m2, group=None):
    """All-gather every rank's Welford triple over torch.distributed and fold
    them in rank order. Returns (count, mean, population variance), identical
    on every rank. With no initialised process group the local triple is the
    result."""
    import torch
    import torch.distributed as dist

    mean = np.ascontiguousarray(mean, dtype=np.float64)
    m2 = np.ascontiguousarray(m2, dtype=np.float64)
    if not (dist.is_available() and dist.is_initialized()):
        n, m, q = count, mean, m2
    else:
        world = dist.get_world_size(group)
        backend = dist.get_backend(group)
        dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
        counts = [torch.zeros(1, dtype=torch.float64, device=dev) for _ in range(world)]
        dist.all_gather(counts, torch.tensor([float(count)], dtype=torch.float64, device=dev), group=group)
        packed = torch.from_numpy(np.stack([mean.ravel(), m2.ravel()])).to(dev)
        parts = [torch.empty_like(packed) for _ in range(world)]
        dist.all_gather(parts, packed, group=group)
        n, m, q = 0, np.zeros_like(mean), np.zeros_like(m2)
        for c, p in zip(counts, parts):
            p = p.cpu().numpy()
            n, m, q = chan_merge((n, m, q), (int(c.item()), p[0].reshape(mean.shape), p[1].reshape(m2.shape)))
    var = q / n if n else np.zeros_like(q)
    return n, m, var


def combine_sums(count, sums, group=None):
    """All-gather every rank's (count, sums) and add them in rank order;
    returns (total count, total sums / total count): the rank reduction of
    sum-type statistics such as the structure functions
    (StatisticsHelper::combineStatistics, MPI_Reduce(SUM) then division by the
    sample count)."""
    import torch
    import torch.distributed as dist

    sums = np.ascontiguousarray(sums, dtype=np.float64)
    if not (dist.is_available() and dist.is_initialized()):
        n, total = count, sums
    else:
        world = dist.get_world_size(group)
        backend = dist.get_backend(group)
        dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
        packed = torch.from_numpy(np.concatenate(([float(count)], sums.ravel()))).to(dev)
        parts = [torch.empty_like(packed) for _ in range(world)]
        dist.all_gather(parts, packed, group=group)
        n, total = 0, np.zeros_like(sums)
        for part in parts:
            a = part.cpu().numpy()
            n += int(a[0])
            total = total + a[1:].reshape(sums.shape)
    return n, (total / n if n else np.zeros_like(total))
