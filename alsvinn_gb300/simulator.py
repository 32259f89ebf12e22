"""One configured finite-volume run on the GPU: the counterpart of
alsfvm::simulator::Simulator as SimulatorSetup builds it
(alsfvm/src/config/SimulatorSetup.cpp:102-230) and alsvinncli drives it
(alsvinncli/src/main.cpp:195-235): set the initial value, call the writers
once, step until the end time, finalize.

The time loop runs on the device (lib.Solver.advance_schedule); the host
wakes up only at save times. The writer's FixedIntervalWriter and the
statistics' FixedIntervalStatistics clamp dt on the device exactly as the
reference's timestep adjusters do, so the trajectory is the reference's.
"""
from . import lib
from .config import ConfigError
from .writers import NetCDFWriter, NumpyWriter, make_writer

PRECISIONS = {"fp64": lib.FP64, "fp64-exact": lib.FP64_EXACT, "fp32": lib.FP32, "fp64-df": lib.FP64_DF}


def interior(U, n, g):
    """Interior cells (nvar, nz, ny, nx) of a padded state (nvar, total)."""
    dim = 3 if n[2] > 1 else (2 if n[1] > 1 else 1)
    t = [n[d] + 2 * g if d < dim else n[d] for d in range(3)]
    V = U.reshape(U.shape[0], t[2], t[1], t[0])
    gz, gy = (g if dim > 2 else 0), (g if dim > 1 else 0)
    return V[:, gz:gz + n[2], gy:gy + n[1], g:g + n[0]]


class Simulator:
    """fvm: a config.FvmConfig. statistics_interval > 0 adds the statistics
    save clamp (alsuq's FixedIntervalStatistics) and calls on_statistics(sim,
    snapshot) after each statistics save; the fvm writer (if configured)
    writes member `sample` of a file sized for num_samples members."""

    def __init__(self, fvm, precision=lib.FP64, sample=0, num_samples=1, output_dir=".",
                 statistics_interval=0.0, statistics_initial=False, on_statistics=None, writer=None):
        self.fvm = fvm
        self.precision = precision
        self.sample = sample
        self.solver = lib.Solver(fvm.equation, fvm.flux, fvm.reconstruction, fvm.integrator, fvm.boundary,
                                 fvm.dimension, fvm.lower, fvm.upper, gamma=fvm.gamma, cfl=fvm.cfl,
                                 precision=precision)
        self.ghosts = lib.ghost_cells(fvm.reconstruction)
        if writer is not None:
            self.writer = writer
        elif fvm.writer is not None:
            self.writer = make_writer(fvm.writer, fvm.equation, fvm.lower, fvm.upper, fvm.dimension, num_samples,
                                      output_dir)
        else:
            self.writer = None
        self.write_interval = fvm.save_interval()
        self.statistics_interval = statistics_interval
        self.statistics_initial = statistics_initial
        self.on_statistics = on_statistics
        self.snapshot = 0
        self.statistics_snapshot = 0
        self._setup_functionals(num_samples, output_dir)

    def _setup_functionals(self, num_samples, output_dir):
        """<functionals>: each an IntervalFunctionalWriter inside a
        FixedIntervalWriter of interval endTime / numberOfSaves that writes the
        initial state too (its writeInitialTimestep defaults to true,
        SimulatorSetup.cpp:626-640, FixedIntervalWriter.hpp:41-43). The
        FixedIntervalWriter is also a timestep adjuster; its save times share
        the device's two save clamps with the writer's and the statistics'
        (equal intervals share a clamp; more than two distinct intervals are
        refused). The output file's time axis holds the initial write plus
        numberOfSaves entries."""
        import os
        f = self.fvm
        self.functionals = []  # [functional, writer, clamp slot, snapshot]
        intervals = [self.write_interval if self.writer is not None else 0.0, self.statistics_interval]
        for fc in f.functionals:
            interval = f.end_time / fc.number_of_saves
            if interval in intervals:
                slot = intervals.index(interval)
            elif 0.0 in intervals:
                slot = intervals.index(0.0)
                intervals[slot] = interval
            else:
                raise ConfigError("more than two distinct save intervals (writer, statistics, functionals) are not "
                                  "supported")
            fn = lib.Functional(fc.name, f.equation, f.boundary, f.dimension, self.ghosts, f.lower, f.upper,
                                **fc.params())
            size = fn.size
            path = os.path.join(output_dir, fc.writer.basename)
            if fc.writer.type == "netcdf":
                times = [0.0] + [(k + 1) / fc.number_of_saves for k in range(fc.number_of_saves)]
                w = NetCDFWriter(path, f.equation, f.lower, f.upper, size, num_samples, times)
            else:
                w = NumpyWriter(path, f.equation)
            self.functionals.append([fn, w, slot, 0])
        self.clamp_intervals = intervals

    def close(self):
        for fn in self.functionals:
            fn[0].close()
        self.solver.close()

    def _write_functionals(self, mask=None):
        prec = self.precision if self.precision == lib.FP32 else lib.FP64
        for entry in self.functionals:
            fn, w, slot, snap = entry
            if mask is not None and not (mask >> slot) & 1:
                continue
            fn.reset()
            fn.apply(self.solver.state_device(), prec, 1.0)
            size = fn.size
            w.write(fn.result().reshape(fn.nvar, size[2], size[1], size[0]), self.sample, snap,
                    time=self.get_current_time())
            entry[3] = snap + 1

    def set_initial_value(self, prim):
        """Interior primitive variables (nvar, nz, ny, nx); resets the time,
        the step count and the save counters."""
        self.solver.set_primitive(prim)
        self.snapshot = 0
        self.statistics_snapshot = 0
        for entry in getattr(self, "functionals", []):
            entry[3] = 0

    def conserved_interior(self):
        return interior(self.solver.get_state(), self.fvm.dimension, self.ghosts)

    def _write(self):
        self.writer.write(self.conserved_interior(), self.sample, self.snapshot, time=self.get_current_time())
        self.snapshot += 1

    def _statistics(self):
        if self.on_statistics is not None:
            self.on_statistics(self, self.statistics_snapshot)
        self.statistics_snapshot += 1

    def call_writers(self):
        """The writers' calls at t = 0 (Simulator::callWriters): a write only
        with writeInitialTimestep, as FixedIntervalWriter starts its counter
        at 1 otherwise."""
        if self.writer is not None and self.fvm.writer.write_initial_timestep:
            self._write()
        if self.functionals:
            self._write_functionals()
        if self.statistics_interval > 0 and self.statistics_initial:
            self._statistics()

    def _advance(self, max_steps):
        mask = self.solver.advance_schedule(self.fvm.end_time, tuple(self.clamp_intervals), max_steps=max_steps,
                                            stop_at_save=True)
        if mask & 1 and self.writer is not None:
            self._write()
        if self.functionals and mask:
            self._write_functionals(mask)
        if mask & 2 and self.statistics_interval > 0:
            self._statistics()
        return mask

    def perform_step(self):
        """One time step (Simulator::performStep), then the due writes."""
        self._advance(1)

    def run(self):
        """Steps until the end time (the alsvinncli loop); the host is
        involved only at save times."""
        while not self.at_end():
            self._advance(0)

    def finalize(self):
        if self.writer is not None:
            self.writer.finalize()
        for fn in self.functionals:
            fn[1].finalize()

    def at_end(self):
        return self.get_current_time() >= self.fvm.end_time

    def get_current_time(self):
        return self.solver.time()[0]

    def get_number_of_timesteps(self):
        return self.solver.time()[1]

    def get_end_time(self):
        return self.fvm.end_time

    def get_name(self):
        return self.fvm.name

