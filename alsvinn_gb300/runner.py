"""The UQ ensemble run of alsuqcli: sample parameters, one finite-volume run
per sample, mean / variance statistics, written by rank 0.

Follows alsuq's Setup::makeRunner and Runner::run
(alsuq/src/config/Setup.cpp:69-126, alsuq/src/run/Runner.cpp:39-90):
  * samples sampleStart .. sampleStart + samples - 1, split into contiguous
    equal blocks over the ranks (SimpleLoadBalancer);
  * per sample, ascending, the parameters in name order (std::map), each
    component drawn through the run's one stateful generator
    (lib.Generator: STLMersenne + Uniform, or Uniform1D's midpoints), then
    the initial data program evaluated with them;
  * statistics at the FixedIntervalStatistics save times, combined over
    ranks and written by rank 0: meanvar over the whole padded state
    (<basename>_mean, <basename>_variance) and structure_cube
    (<basename>_structure_cube_<p>, one value per distance h;
    alsuq/src/stats/StructureCube.cpp).

Two engines run the samples:
  * "batch" - the ensemble engine (lib.Batch): every sample of a wave is a
    member of one persistent launch per RK stage, each with its own dt; the
    statistics are folded on the device as members reach their save times.
    An fvm writer is the member's second save clamp: the wave advances to
    each writer save, where every member stops exactly, and the host writes
    the members' states (Runner::run attaches the writers to every sample's
    simulator, alsuq/src/run/Runner.cpp:55-73). Used for mean / variance
    statistics without an initial-time save and without fvm functionals.
  * "serial" - one lib.Solver reused sample after sample with the writer and
    statistics save clamps (any schedule).
Both give each sample the reference's trajectory; the statistics are FP64
Welford accumulators (population variance, as MeanVariance).
"""
import time

import numpy as np

from . import initdata, lib, uq
from .config import ConfigError
from .simulator import Simulator, interior
from .writers import NetCDFWriter, NumpyWriter, make_writer


class _FunctionalAccumulator:
    """Sum-type statistics built on device functionals (weight 1 per sample):
    functional (FunctionalStatistics), onepointmoment (OnePointMoment:
    addPower, the "moment" functional), bv (BoundedVariation), bv_direction
    (BoundedVariationDirection, one functional per direction). `assign`
    keeps only the latest sample, as BoundedVariationDirection assigns its
    snapshot instead of adding to it (alsuq/src/stats/
    BoundedVariationDirection.cpp:40-60); StatisticsHelper::
    combineStatistics then sums over ranks and divides by the sample count
    for all of them (StatisticsHelper.cpp:35-79)."""

    def __init__(self, functionals, assign=False):
        self.functionals = functionals
        self.assign = assign
        self.count = 0

    def add_device(self, ptr, precision):
        for f in self.functionals:
            if self.assign:
                f.reset()
            f.apply(ptr, precision, 1.0)
        self.count += 1

    def export(self):
        return self.count, np.stack([f.result() for f in self.functionals])

    def close(self):
        for f in self.functionals:
            f.close()


def make_statistic_accumulator(st, fvm, ghosts, nvar):
    """The device accumulator of one save of statistic `st` on grid `fvm`."""
    n, lo, hi = fvm.dimension, fvm.lower, fvm.upper
    if st.name == "meanvar":
        return lib.Stats(nvar * int(np.prod([n[d] + 2 * ghosts if d < fvm.dim else n[d] for d in range(3)])))
    if st.name == "structure_cube":
        return lib.Structure(fvm.boundary, n, ghosts, nvar, st.number_of_h, st.p)
    if st.name == "structure_basic":
        return lib.Structure(fvm.boundary, n, ghosts, nvar, st.number_of_h, st.p, direction=st.direction)
    if st.name == "onepointmoment":
        fs = [lib.Functional("moment", fvm.equation, fvm.boundary, n, ghosts, lo, hi, degree=int(st.p))]
    elif st.name == "bv":
        fs = [lib.Functional("bv", fvm.equation, fvm.boundary, n, ghosts, lo, hi, degree=int(st.p))]
    elif st.name == "bv_direction":
        fs = [lib.Functional("bv_direction", fvm.equation, fvm.boundary, n, ghosts, lo, hi, degree=int(st.p),
                             direction=d) for d in range(fvm.dim)]
        return _FunctionalAccumulator(fs, assign=True)
    else:
        f = st.functional
        fs = [lib.Functional(f.name, fvm.equation, fvm.boundary, n, ghosts, lo, hi, **f.params())]
    return _FunctionalAccumulator(fs)


def sample_parameters(uqc, samples, generator=None):
    """{sample: {name: [values]}} for the given ascending samples, drawn in
    the Runner's order on one generator."""
    gen = generator or lib.Generator()
    out = {}
    for s in samples:
        params = {}
        for p in sorted(uqc.parameters, key=lambda q: q.name):
            if p.type == "uniform":
                params[p.name] = [gen.uniform(p.length, c, s, p.lower, p.upper) for c in range(p.length)]
            elif p.type == "uniform1d":
                if p.length != 1:
                    raise ConfigError("With Uniform1D we only support 1 dimension")
                params[p.name] = [p.a + (p.b - p.a) / uqc.samples * (s + 0.5)]
            else:
                raise ConfigError("Unknown distribution %s" % p.type)
        out[s] = params
    return out


class Runner:
    def __init__(self, config, precision=lib.FP64, rank=0, world_size=1, output_dir=".", engine="auto",
                 hbm_budget_bytes=None):
        if config.uq is None:
            raise ConfigError("Missing configuration node: uq")
        self.config = config
        self.fvm = config.fvm
        self.uqc = config.uq
        self.precision = precision
        self.rank = rank
        self.world_size = world_size
        self.output_dir = output_dir
        self.hbm_budget = hbm_budget_bytes
        s0, s1 = uq.sample_blocks(self.uqc.samples, world_size)[rank]
        self.samples = list(range(self.uqc.sample_start + s0, self.uqc.sample_start + s1))
        stats = self.uqc.stats
        intervals = {st.save_interval(self.fvm.end_time) for st in stats}
        if len(intervals) > 1:
            raise ConfigError("statistics with different numberOfSaves in one run are not supported")
        self.stats_interval = intervals.pop() if intervals else 0.0
        self.stats_saves = stats[0].number_of_saves if stats else 0
        self.stats_initial = bool(stats and stats[0].write_initial_timestep)
        batch_ok = (not self.fvm.functionals
                    and not self.stats_initial and all(st.name == "meanvar" for st in stats)
                    and self.fvm.integrator in ("rungekutta2", "rungekutta3"))
        if engine == "auto":
            engine = "batch" if batch_ok else "serial"
        if engine == "batch" and not batch_ok:
            raise ConfigError("the batch engine needs rungekutta2/3, mean/variance statistics (no initial-time "
                              "statistics) and no fvm functionals; use the serial engine")
        self.engine = engine
        self.timesteps = 0
        self.wall_s = 0.0

    def _prim(self, params):
        p = dict(self.fvm.init_parameters)
        p.update(params)
        return initdata.evaluate(self.fvm.python_program, self.fvm.equation, self.fvm.lower, self.fvm.upper,
                                 self.fvm.dimension, p)

    def run(self):
        """Runs this rank's samples and combines the statistics over the
        ranks (identical on every rank); rank 0 writes them. self.statistics
        holds, per configured statistic, one entry per save: (count, mean,
        variance) for meanvar (padded states (nvar, total) flattened), (count,
        structure function (nvar, numberOfH)) for structure_cube, (count,
        mean (outputs, nvar, output cells)) for the functional-based ones
        (functional, onepointmoment, bv: one output; bv_direction: one per
        grid direction). Returns the first meanvar statistic's entries."""
        t0 = time.perf_counter()
        params = sample_parameters(self.uqc, self.samples)
        if self.engine == "batch":
            raw = self._run_batch(params)
        else:
            raw = self._run_serial(params)
        self.statistics = []
        for st, saves in zip(self.uqc.stats, raw):
            if st.name == "meanvar":
                self.statistics.append([uq.combine_statistics(*t) for t in saves])
            else:
                self.statistics.append([uq.combine_sums(*t) for t in saves])
        self.wall_s = time.perf_counter() - t0
        if self.rank == 0:
            self._write_statistics()
        for st, res in zip(self.uqc.stats, self.statistics):
            if st.name == "meanvar":
                return res
        return []

    # -- engines -----------------------------------------------------------

    def _run_serial(self, params):
        sim = Simulator(self.fvm, self.precision, num_samples=self.uqc.samples, output_dir=self.output_dir,
                        statistics_interval=self.stats_interval, statistics_initial=self.stats_initial)
        nsave = self.stats_saves + (1 if self.stats_initial else 0)
        g = lib.ghost_cells(self.fvm.reconstruction)
        acc = []  # per statistic, per save
        for st in self.uqc.stats:
            acc.append([make_statistic_accumulator(st, self.fvm, g, sim.solver.nvar) for _ in range(nsave)])
        prec = self.precision if self.precision == lib.FP32 else lib.FP64

        def on_statistics(s, k):
            ptr = s.solver.state_device()
            for per_save in acc:
                per_save[k].add_device(ptr, prec)

        sim.on_statistics = on_statistics
        try:
            for s in self.samples:
                sim.sample = s
                sim.set_initial_value(self._prim(params[s]))
                sim.call_writers()
                sim.run()
                self.timesteps += sim.get_number_of_timesteps()
            sim.finalize()
            raw = [[a.export() for a in per_save] for per_save in acc]
        finally:
            for per_save in acc:
                for a in per_save:
                    a.close()
            sim.close()
        return raw

    def _run_batch(self, params):
        f = self.fvm
        b = lib.Batch(f.equation, f.flux, f.reconstruction, f.integrator, f.boundary, 1 << 20, 1, gamma=f.gamma,
                      cfl=f.cfl, precision=self.precision)
        per = b.member_bytes(f.dimension)
        b.close()
        budget = self.hbm_budget
        if budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            budget = int(free * 0.8)
        wave = max(1, min(len(self.samples), int(budget // per)))
        pool = wave * per + (16 << 20)
        b = lib.Batch(f.equation, f.flux, f.reconstruction, f.integrator, f.boundary, pool, wave, gamma=f.gamma,
                      cfl=f.cfl, precision=self.precision)
        # statistics at each of the numberOfSaves save times, folded on the
        # device as every member's save clamp stops it there
        saves = max(1, self.stats_saves)
        per_save = []
        writer = None
        if f.writer is not None:
            writer = make_writer(f.writer, f.equation, f.lower, f.upper, f.dimension, self.uqc.samples,
                                 self.output_dir)
        g = lib.ghost_cells(f.reconstruction)
        try:
            b.set_statistics_saves(saves)
            for i in range(0, len(self.samples), wave):
                chunk = self.samples[i:i + wave]
                slots = [b.add(f.dimension, f.lower, f.upper, self._prim(params[s]), group=0) for s in chunk]
                if writer is None:
                    b.advance(f.end_time, saves if self.stats_saves > 0 else 1, 0)
                else:
                    self._advance_with_writer(b, writer, slots, chunk, saves, g)
                for sl in slots:
                    self.timesteps += b.member_time(sl)[1]
                    b.remove(sl)
            if writer is not None:
                writer.finalize()
            nv = lib.num_variables(f.equation)
            dim = f.dim
            total = int(np.prod([f.dimension[d] + 2 * g if d < dim else f.dimension[d] for d in range(3)]))
            for k in range(saves):
                if self.samples:
                    n, m, q = b.stats_export(0, total, save=k)
                else:
                    n, m, q = 0, np.zeros((nv, total)), np.zeros((nv, total))
                per_save.append((n, m.reshape(-1), q.reshape(-1)))
        finally:
            b.close()
        return [list(per_save) for _ in self.uqc.stats]

    def _advance_with_writer(self, b, writer, slots, samples, saves, g):
        """A wave with the fvm writer: each member's own end time with the
        statistics clamp (interval endTime / saves) and the writer's clamp
        (endTime / numberOfSaves); the wave advances to each writer save
        k * interval, where every member stops exactly, and the host writes
        the members' states (snapshot 0 at t = 0 with writeInitialTimestep),
        as the serial engine's simulator does between its advances."""
        f = self.fvm
        W = f.save_interval()
        nvar = lib.num_variables(f.equation)
        total = int(np.prod([f.dimension[d] + 2 * g if d < f.dim else f.dimension[d] for d in range(3)]))
        for sl in slots:
            b.set_member_end(sl, f.end_time, saves)
            b.set_member_write_interval(sl, W)

        def write_all(snapshot):
            for sl, s in zip(slots, samples):
                U = b.member_state(sl, total)
                t, _ = b.member_time(sl)
                writer.write(interior(U.reshape(nvar, total), f.dimension, g), s, snapshot, time=t)

        snapshot = 0
        if f.writer.write_initial_timestep:
            write_all(snapshot)
            snapshot += 1
        for k in range(1, f.writer.number_of_saves + 1):
            b.advance(k * W, 0, 0)
            write_all(snapshot)
            snapshot += 1
        # the end time itself (k * interval may fall an ulp short of it)
        b.advance(f.end_time, 0, 0)

    # -- output ------------------------------------------------------------

    def _functional_size(self, st):
        """Output extents of a functional-based statistic."""
        if st.name in ("bv", "bv_direction"):
            return (1, 1, 1)
        if st.name == "onepointmoment":
            return tuple(self.fvm.dimension)
        fc = st.functional
        if fc.name in ("log_entropy", "bv"):
            return (1, 1, 1)
        if fc.name == "structure_cube":
            return (fc.number_of_h, 1, 1)
        return tuple(self.fvm.dimension)

    def _write_statistics(self):
        f = self.fvm
        nv = lib.num_variables(f.equation)
        g = lib.ghost_cells(f.reconstruction)
        from .simulator import interior
        for st, results in zip(self.uqc.stats, self.statistics):
            w = st.writer
            if st.name == "meanvar":
                outputs = [(name, [interior(np.asarray(r[idx]).reshape(nv, -1), f.dimension, g) for r in results],
                            (f.lower, f.upper, f.dimension))
                           for name, idx in (("mean", 1), ("variance", 2))]
            elif st.name in ("structure_cube", "structure_basic"):
                # one value per distance h: x runs over h = 0 .. numberOfH - 1
                H = st.number_of_h
                outputs = [(st.output_names()[0], [np.asarray(r[1]).reshape(nv, 1, 1, H) for r in results],
                            ((-0.5, 0.0, 0.0), (H - 0.5, 1.0, 1.0), (H, 1, 1)))]
            else:
                outputs = []
                for k, name in enumerate(st.output_names()):
                    size = self._functional_size(st)
                    if st.name == "bv_direction" and k >= f.dim:
                        # a direction the grid does not have: its snapshot is never assigned
                        arrays = [np.zeros((nv, 1, 1, 1)) for _ in results]
                    else:
                        arrays = [np.asarray(r[1])[k].reshape(nv, size[2], size[1], size[0]) for r in results]
                    grid = ((f.lower, f.upper, f.dimension) if tuple(size) == tuple(f.dimension)
                            else (f.lower, f.upper, tuple(size)))
                    outputs.append((name, arrays, grid))
            for name, arrays, (lo, hi, dims) in outputs:
                base = "%s/%s_%s" % (self.output_dir, w.basename, name)
                if w.type == "netcdf":
                    writer = NetCDFWriter(base, f.equation, lo, hi, dims, 1, w.save_fractions())
                else:
                    writer = NumpyWriter(base, f.equation)
                for k, a in enumerate(arrays):
                    writer.write(a, 0, k)
                writer.finalize()
