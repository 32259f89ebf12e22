"""Benchmark of the GB300 finite-volume step.

Workload: 2D Kelvin-Helmholtz, compressible Euler (gamma 1.4) on a periodic
1024x1024 grid over [0,1]^2, WENO2 reconstruction, HLL3 flux, SSP-RK3, CFL 0.4,
FP64 state and arithmetic (the drop-in path). Initial data are the seeded
interface perturbation evaluated at cell midpoints (sample 0 of the
reference's generator). One "step" is one SSP-RK3 time step of the whole grid.

Metric: cell-updates/s = interior cells x time steps / time (RK stages are
not counted separately). `value` is measured with the state resident in HBM;
the L2 (129 MB) is flushed by a 512 MiB memset on the solver's stream before
every timed step, outside the step's events. `e2e` is the same metric through
gbfv_advance_host with the state in pinned host memory: every step copies the
padded state host->device, advances one step and copies it back.

The roofline uses the algorithmic bytes of an SSP-RK3 step, 8 * nvar * 8 bytes
per interior cell (stage 0 reads U0 and writes L0, stages 1 and 2 read two
state arrays and write one), against the measured HBM copy bandwidth in
MEASURED_PEAKS.json. The stage kernel's per-launch time comes from CUDA events
the library records around every stage launch on its stream.

--impl reference times the reference's CPU algorithm (the oracle restatement,
bit-identical to the reference CPU path) on all host cores for the same
workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

N = 1024
NVAR = 4
BYTES_PER_CELL_STEP = 8 * NVAR * 8  # SSP-RK3, FP64
WORKLOAD = "kh2d_1024x1024_euler2_weno2_hll3_rk3_fp64"
METRIC = "cell-updates/s"
FLUSH_BYTES = 512 << 20


def kh_initial_primitives(n, sample=0):
    import workloads
    from alsvinn_gb300 import lib
    return workloads.kh_prim(n, lib.uniform(40, sample))


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per stage launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(steps):
    """The oracle (reference CPU algorithm) on all host cores, bounded sample."""
    from oracle import fvoracle
    import workloads  # noqa: F401
    prim = kh_initial_primitives(N)
    threads = os.cpu_count() or 1
    fvoracle.set_threads(threads)
    t0 = time.perf_counter()
    rc, _, _, done = fvoracle.run("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0),
                                  (1, 1, 0), 1.4, 0.4, 2.0, 0, steps, prim, 2, NVAR)
    dt = time.perf_counter() - t0
    if rc != 0 or done != steps:
        raise RuntimeError("oracle run failed")
    return {"value": N * N * steps / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "KH 1024x1024 WENO2/HLL3/RK3 FP64, %d steps from t=0 on %d threads (incl. setup)"
                      % (steps, threads)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import fvoracle
    prim = kh_initial_primitives(N)
    threads = os.cpu_count() or 1
    fvoracle.set_threads(threads)
    # warm-up steps are run untimed; then K single-step samples are timed
    fvoracle.run("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0), (1, 1, 0), 1.4,
                 0.4, 2.0, 0, max(args.warmup, 1), prim, 2, NVAR)
    t0 = time.perf_counter()
    rc, _, _, done = fvoracle.run("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0),
                                  (1, 1, 0), 1.4, 0.4, 2.0, 0, args.steps, prim, 2, NVAR)
    dt = time.perf_counter() - t0
    value = N * N * done / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded KH interface perturbation)",
            "config": {"workload": WORKLOAD, "grid": [N, N], "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": "%d SSP-RK3 steps of KH 1024x1024 from t=0 (incl. setup) on %d threads"
                                       % (done, threads)},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from alsvinn_gb300 import lib

    prim = kh_initial_primitives(N, sample=rank)
    s = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0), (1, 1, 0),
                   gamma=1.4, cfl=0.4, precision=lib.FP64)
    s.set_primitive(prim)
    stream = torch.cuda.ExternalStream(s.stream())
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    # warm-up
    s.advance(2.0, 0, args.warmup)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    s.profile(True)
    s.profile_read()
    _, _, launches0 = s.profile_read()
    barrier()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xFF)  # L2 flush, outside the timed events
                starts[i].record(stream)
            s.advance(2.0, 0, 1)
            with torch.cuda.stream(stream):
                ends[i].record(stream)
        barrier()
    stage_ms, stage_launches, launches1 = s.profile_read()
    s.profile(False)
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = sum(step_ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    t_sim, steps_done, _ = s.time()
    cells = N * N
    value = world * cells * args.steps / (total_ms * 1e-3)

    # end to end through host buffers (pinned), one step per call
    host = torch.empty((NVAR, s.total), dtype=torch.float64).pin_memory()
    host_np = host.numpy()
    host_np[...] = s.get_state()
    e2e_steps = max(1, min(args.steps, 10))
    s.advance_host(host_np, 2.0, 0, 1)  # warm path
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.advance_host(host_np, 2.0, 0, 1)
    barrier()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    state_bytes = NVAR * s.total * 8
    e2e = {"value": world * cells * e2e_steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "steps": e2e_steps}

    peak, peak_kind = measured_peaks()
    per_launch_ms = stage_ms / max(stage_launches, 1)
    alg_bytes_per_launch = cells * BYTES_PER_CELL_STEP / 3.0
    achieved = alg_bytes_per_launch / (per_launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profile_traffic(), "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "kernel": "stage_kernel<double,euler2,hll3,weno2,2D>", "launch_ms": per_launch_ms,
                "alg_bytes_per_launch": alg_bytes_per_launch,
                "note": "FP64 arithmetic on GB300 issues at ~1/64 of the FP32 rate; this step is FP64-compute "
                        "bound, not HBM bound"}
    clk = clocks.summary()
    line = None
    if rank == 0:
        base = cpu_baseline(args.cpu_steps) if world == 1 else None
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded KH interface perturbation, sample = rank)",
                "config": {"workload": WORKLOAD, "grid": [N, N], "equation": "euler2", "reconstruction": "weno2",
                           "flux": "hll3", "integrator": "rungekutta3", "precision": "fp64",
                           "l2": "flushed before every timed step (512 MiB memset, outside the events)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": roofline, "cpu_baseline": base, "e2e": e2e, "clocks": clk,
                "gpu_launches": int(launches1 - launches0),
                "sim": {"t": t_sim, "steps": steps_done}}
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=60)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
