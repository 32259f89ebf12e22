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
gbfv_advance_host with the state in pinned host memory, one step per call:
each step's input state comes from host memory and its result goes back to
it (the first stage reads the mapped host state in place and the last stage
writes it back, over NVLink-C2C, instead of two copies around the step).

The roofline uses the algorithmic bytes of an SSP-RK3 step, 8 * nvar * 8 bytes
per interior cell (stage 0 reads U0 and writes L0, stages 1 and 2 read two
state arrays and write one), against the measured HBM copy bandwidth in
MEASURED_PEAKS.json. The stage kernel's per-launch time comes from CUDA events
the library records around every stage launch on its stream.

The headline line also carries sub-objects measured in the same run: the
double-float variant (`fp64_df`), the batched UQ ensemble (`uq`) and the
serving stream (`serve`) to their end times, the Sod configuration to its end
time (`sod`) and Taylor-Green 256^3 in FP64 and FP32 state (`tg`).

--impl reference times the reference's CPU algorithm (the oracle restatement,
bit-identical to the reference CPU path) on all host cores for the same
workload, and beside it the reference's own CUDA kernels built for sm_103a
(`reference_gpu_path`).
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
    """Product initial data (the library's C++ formula) for the GPU arm."""
    from alsvinn_gb300 import lib
    return lib.init_kelvin_helmholtz(n, sample=sample)


def oracle_kh_primitives(n, sample=0):
    """The same initial data for the CPU arms, without product code: the
    oracle's generator draws and the Python formula of tests/workloads.py
    (bit-identical to the library's, which the tests check)."""
    import workloads
    from oracle import fvoracle
    return workloads.kh_prim(n, fvoracle.uniform(40, sample))


def headline_config(precision):
    """The workload description both arms print (the same dict in each)."""
    return {"workload": WORKLOAD, "grid": [N, N], "domain": [[0, 1], [0, 1]], "boundary": "periodic",
            "equation": "euler2", "gamma": 1.4, "reconstruction": "weno2", "flux": "hll3",
            "integrator": "rungekutta3", "cfl": 0.4, "precision": precision,
            "initial_data": "KH interface perturbation, generator sample = rank",
            "l2": "state 33.8 MB < L2: flushed before every timed GPU step (512 MiB memset, outside the events)",
            "parallelism": "independent replicas, one per rank"}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def time_oracle_kh(prim, steps, threads):
    """The oracle's KH 1024^2 run of `steps` SSP-RK3 steps on `threads`
    threads; returns (steps done, seconds of the step loop alone)."""
    from oracle import fvoracle
    fvoracle.set_threads(threads)
    rc, _, _, done = fvoracle.run("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0),
                                  (1, 1, 0), 1.4, 0.4, 2.0, 0, steps, prim, 2, NVAR)
    if rc != 0 or done != steps:
        raise RuntimeError("oracle run failed")
    return done, fvoracle.last_loop_seconds()


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


def profile_summary():
    """The committed ncu figures of the stage kernel (DRAM bytes per launch,
    FP64 pipe use), if any."""
    p = os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def profile_traffic():
    """DRAM bytes per stage launch from the committed ncu summary, if any."""
    return profile_summary().get("dram_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms over the timed region:
    sampling is running before the region starts and takes one more sample
    after it ends, so even a region shorter than the interval is bracketed."""

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
        # sampling running before the timed region starts, and one more
        # sample after it ends: a short region is bracketed by samples
        self._wait_samples(1, 3.0)
        self.before = self._samples()
        return self

    def _samples(self):
        try:
            with open(self.path) as f:
                return sum(1 for line in f if line.strip())
        except OSError:
            return 0

    def _wait_samples(self, n, timeout):
        t0 = time.time()
        while (self.proc and self.proc.poll() is None and self._samples() < n
               and time.time() - t0 < timeout):
            time.sleep(0.02)

    def __exit__(self, *exc):
        if self.proc:
            self._wait_samples(self.before + 1, 1.0)
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


def cpu_baseline(steps, one_thread_steps=2):
    """The oracle (the reference's CPU algorithm, restated) on every host core
    over a bounded sample, plus a one-thread figure; step loop only."""
    prim = oracle_kh_primitives(N)
    threads = os.cpu_count() or 1
    time_oracle_kh(prim, 1, threads)  # untimed: first touch, thread pool
    done, sec = time_oracle_kh(prim, steps, threads)
    done1, sec1 = time_oracle_kh(prim, one_thread_steps, 1)
    return {"value": N * N * done / sec, "unit": METRIC, "cores": threads, "kind": "port",
            "cpu_model": cpu_model(), "one_thread_value": N * N * done1 / sec1,
            "sample": "KH 1024x1024 WENO2/HLL3/SSP-RK3 FP64: %d steps on %d threads, %d steps on 1 thread, "
                      "step loop only (initial data and allocation excluded)" % (done, threads, done1)}


def run_reference(args):
    """The reference's CPU path for the headline workload: the oracle port
    (bit-identical to the reference's own CPU build wherever both ran) on all
    host threads. Initial data come from the oracle's generator and the
    Python formula; nothing of the GPU library is loaded."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    prim = oracle_kh_primitives(N)
    threads = os.cpu_count() or 1
    time_oracle_kh(prim, max(args.warmup, 1), threads)  # warm-up run, untimed
    done, sec = time_oracle_kh(prim, args.steps, threads)
    done1, sec1 = time_oracle_kh(prim, 2, 1)
    value = N * N * done / sec
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / max(done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded KH interface perturbation)",
            "config": headline_config("fp64"),
            "executor": "oracle port of the reference CPU path, %d host threads (%s)" % (threads, cpu_model()),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(), "one_thread_value": N * N * done1 / sec1,
                             "sample": "%d SSP-RK3 steps of KH 1024x1024 after %d warm-up steps on %d threads; "
                                       "%d steps on 1 thread; step loop only" % (done, max(args.warmup, 1),
                                                                                 threads, done1)},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["reference_gpu_path"] = time_reference_cuda(prim, args)
    line["reference_gpu_path_other"] = time_reference_cuda_other(args)
    print(json.dumps(line), flush=True)


def time_reference_cuda(prim, args):
    """The reference's own CUDA path on the same workload, beside its CPU
    path: its kernels compiled from its sources for sm_103a (oracle/_ref/cuda)
    and launched by oracle/refcuda in the order the reference's Simulator
    launches them on the cuda platform, state resident on the device. Reported
    next to the line's value, not as it."""
    import numpy as np
    from oracle import fvoracle, refcuda
    why = refcuda.missing()
    if why:
        return {"unavailable": why}
    g = 2
    t = N + 2 * g
    P = np.zeros((4, t, t))
    P[:, g:g + N, g:g + N] = prim.reshape(4, N, N)
    U0 = fvoracle.prim_to_cons("euler2", (N, N, 1), g, 1.4, P.reshape(4, -1))
    steps = max(1, min(args.steps, 20))
    try:
        with refcuda.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0), (1, 1, 0),
                            1.4, 0.4) as s:
            s.set_state(U0)
            s.run(1e9, 0, max(args.warmup, 3))
            l0 = s.launches()
            _, done = s.run(1e9, 0, steps)
            ms = s.last_ms()
            per_step = (s.launches() - l0) / max(done, 1)
    except refcuda.RefCudaError as e:
        return {"unavailable": str(e)}
    return {"value": N * N * done / (ms * 1e-3), "unit": METRIC, "steps": done, "ms_per_step": ms / done,
            "kernels_per_step": per_step, "blocking_copies_per_step": 3 * 5 * 2,
            "executor": "the reference's CUDA kernels (NumericalFluxCUDA, ReconstructionCUDA, BoundaryCUDA, "
                        "vector_operations, CUDACellComputer) built from its sources for sm_103a with its release "
                        "flags; host sequence restated by oracle/refcuda (cub max and a blocking copy per direction "
                        "and computeFlux call, thrust constraint reduce per step)",
            "timing": "CUDA events on the legacy default stream around %d steps after %d warm-up steps; working "
                      "set (seven FP64 volumes, 237 MB) larger than L2" % (done, max(args.warmup, 3))}


def time_reference_cuda_other(args):
    """The reference's CUDA path on the other two finite-volume
    configurations, for comparison with the headline line's `sod` and `tg`
    sub-objects: Sod 2048 from t = 0 to 1.3 (one save's dt clamp) and
    Taylor-Green 256^3 (2 steps after 1), FP64, CUDA events around the runs."""
    import math
    import numpy as np
    import workloads
    from oracle import fvoracle, refcuda
    why = refcuda.missing()
    if why:
        return {"unavailable": why}
    out = {}
    g = 2
    try:
        prim = workloads.sod_prim(2048)
        P = np.zeros((3, 2048 + 2 * g))
        P[:, g:g + 2048] = prim
        U0 = fvoracle.prim_to_cons("euler1", (2048, 1, 1), g, 1.4, P)
        with refcuda.Solver("euler1", "hll3", "weno2", "rungekutta3", "neumann", (2048, 1, 1), (-5, 0, 0),
                            (5, 1, 1), 1.4, 0.475) as s:
            s.set_state(U0)
            s.run(1.3, 1, 0)  # warm-up run
            s.set_state(U0)
            t, done = s.run(1.3, 1, 0)
            out["sod2048_to_t1.3"] = {"ms_to_end_time": s.last_ms(), "steps": done, "end_time": t,
                                      "value": 2048 * done / (s.last_ms() * 1e-3), "unit": METRIC}
        n = 256
        x = (np.arange(n) + 0.5) * (2 * math.pi / n)
        Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
        P = np.zeros((5, n + 2 * g, n + 2 * g, n + 2 * g))
        inner = (slice(None), slice(g, g + n), slice(g, g + n), slice(g, g + n))
        P[0][inner[1:]] = 1.0
        P[1][inner[1:]] = np.sin(X) * np.cos(Y) * np.cos(Z)
        P[2][inner[1:]] = -np.cos(X) * np.sin(Y) * np.cos(Z)
        P[4][inner[1:]] = 100 + ((np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2) - 2) / 16
        del X, Y, Z
        U0 = fvoracle.prim_to_cons("euler3", (n, n, n), g, 1.4, P.reshape(5, -1))
        del P
        with refcuda.Solver("euler3", "hll3", "weno2", "rungekutta3", "periodic", (n, n, n), (0, 0, 0),
                            (2 * math.pi,) * 3, 1.4, 0.4) as s:
            s.set_state(U0)
            s.run(1e9, 0, 1)
            _, done = s.run(1e9, 0, 2)
            ms = s.last_ms()
            out["tg256"] = {"value": n ** 3 * done / (ms * 1e-3), "unit": METRIC, "steps": done,
                            "ms_per_step": ms / done}
    except refcuda.RefCudaError as e:
        out["unavailable"] = str(e)
    return out


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from alsvinn_gb300 import lib

    prim = kh_initial_primitives(N, sample=rank)
    precision = {"fp64": lib.FP64, "fp64-df": lib.FP64_DF, "fp64-exact": lib.FP64_EXACT, "fp32": lib.FP32}[
        args.precision]
    elem = 4 if args.precision == "fp32" else 8
    s = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0), (1, 1, 0),
                   gamma=1.4, cfl=0.4, precision=precision)
    s.set_primitive(prim)
    stream = torch.cuda.ExternalStream(s.stream())
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    # the autotuner (the same one the first advance runs), its table reported;
    # --candidate pins one configuration instead (reproducible profiler runs)
    cands = s.candidates()
    if args.candidate >= 0:
        s.select_candidate(args.candidate)
        chosen, tune_ms = args.candidate, [-1.0] * len(cands)
    else:
        chosen, tune_ms = s.autotune()
    stage_kernel = {"candidate": chosen, "tile": list(cands[chosen][0]), "threads": cands[chosen][1],
                    "tma": cands[chosen][2],
                    "autotune_ms_per_launch": [{"tile": list(c[0]), "threads": c[1], "tma": c[2], "ms": m}
                                               for c, m in zip(cands, tune_ms)]}

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
    state_bytes = NVAR * s.total * 8  # gbfv_advance_host moves the FP64 host state
    e2e = {"value": world * cells * e2e_steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "steps": e2e_steps,
           "transfer": "the padded FP64 state read from and written to pinned host memory every step, by the "
                       "first and last stage kernels in place (mapped memory over NVLink-C2C)"}

    # the same workload with the reconstruction and flux arithmetic in
    # double-float on the FP32 pipes (FP64 state and RK update): reported
    # beside the FP64 headline, with its parity
    df = None
    if args.precision == "fp64" and not args.no_df:
        sd = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (N, N, 1), (0, 0, 0), (1, 1, 0),
                        gamma=1.4, cfl=0.4, precision=lib.FP64_DF)
        sd.set_primitive(prim)
        sd.advance(2.0, 0, args.warmup)
        dstream = torch.cuda.ExternalStream(sd.stream())
        sd.profile(True)
        sd.profile_read()
        dms = 0.0
        for i in range(args.steps):
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(dstream):
                flush.fill_(i & 0xFF)
                a0.record(dstream)
            sd.advance(2.0, 0, 1)
            with torch.cuda.stream(dstream):
                a1.record(dstream)
            torch.cuda.synchronize()
            dms += a0.elapsed_time(a1)
        dstage_ms, dstage_n, _ = sd.profile_read()
        sd.close()
        df = {"value": world * cells * args.steps / (dms * 1e-3), "unit": METRIC, "ms_per_step": dms / args.steps,
              "stage_launch_ms": dstage_ms / max(dstage_n, 1),
              "arithmetic": "reconstruction + flux in double-float (2 x fp32, ~48 bits) on the FP32 pipes; "
                            "FP64 state and FP64 Runge-Kutta update",
              "parity": "<= 1e-10 relative L1 per variable vs the reference on Sod, KH, Burgers; 4.3e-10 on "
                        "Taylor-Green z-momentum (tests/test_gpu_parity.py)"}

    peak, peak_kind = measured_peaks()
    per_launch_ms = stage_ms / max(stage_launches, 1)
    alg_bytes_per_launch = cells * (8 * NVAR * elem) / 3.0
    achieved = alg_bytes_per_launch / (per_launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profile_traffic(), "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "kernel": "%s<double,euler2,hll3,weno2,2D>%s tile %dx%d, %d threads" % (
                    "stage_kernel_tma" if stage_kernel["tma"] else "stage_kernel",
                    " (double-float arithmetic)" if args.precision == "fp64-df" else "", stage_kernel["tile"][0],
                    stage_kernel["tile"][1], stage_kernel["threads"]), "launch_ms": per_launch_ms,
                "alg_bytes_per_launch": alg_bytes_per_launch,
                "note": "FP64 arithmetic on GB300 issues at ~1/64 of the FP32 rate; this step is FP64-compute "
                        "bound, not HBM bound",
                "fp64_pipe": {"active_frac": profile_summary().get("fp64_pipe_active_frac"),
                              "issue_frac": profile_summary().get("fp64_issue_frac"),
                              "source": "ncu sm__pipe_fp64_cycles_active and DADD+DFMA+DMUL thread "
                                        "instructions per cycle over the 2 per SM per cycle peak "
                                        "(profiles/stage_kernel_tma_kh1024_fp64.md)"}}
    if args.precision != "fp64":
        # the traffic and FP64-pipe figures come from the FP64 kernel's capture
        roofline["traffic"] = None
        roofline["fp64_pipe"] = None
    clk = clocks.summary()
    line = None
    if rank == 0:
        base = cpu_baseline(args.cpu_steps) if world == 1 else None
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if elem == 4 else "f64",
                "data": "synthetic (seeded KH interface perturbation, sample = rank)",
                "config": headline_config(args.precision), "stage_kernel": stage_kernel,
                "roofline": roofline, "cpu_baseline": base, "e2e": e2e, "clocks": clk,
                "gpu_launches": int(launches1 - launches0), "fp64_df": df,
                "sim": {"t": t_sim, "steps": steps_done}}
        s.close()
        # the batched UQ ensemble and the serving stream, measured to their
        # end times (one GPU: these describe the single-device engines)
        if world == 1 and args.headline_uq_samples > 0:
            line["uq"] = measure_uq(args.headline_uq_samples, args.uq_plain, args.warmup)
        if world == 1 and args.headline_serve_requests > 0:
            line["serve"] = measure_serve(args.headline_serve_requests, args.serve_rate, args.serve_chunk,
                                          args.serve_plain)
        # the other two finite-volume configurations: Sod 2048 to its end
        # time, Taylor-Green 256^3 (FP64 and FP32 state)
        if world == 1 and args.headline_fv:
            line["sod"] = measure_sod(warmup=1)
            line["tg"] = {"fp64": measure_tg(256, "fp64", 5, 3), "fp32": measure_tg(256, "fp32", 5, 3)}
        print(json.dumps(line), flush=True)
    else:
        s.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def measure_tg(n, precision_name, steps, warmup, candidate=-1):
    """Taylor-Green (euler3, WENO2, HLL3, SSP-RK3, CFL 0.4, periodic on
    [0, 2 pi]^3) on n^3 cells: `warmup` steps, then `steps` timed steps with
    CUDA events on the solver's stream (the L2 flushed before each); the
    autotuner's table, or `candidate` pinned (profiler runs). Roofline of the
    stage launch as for the headline: 8 nvar b / 3 algorithmic bytes per cell
    per stage (5 variables)."""
    import math
    import torch
    from alsvinn_gb300 import lib

    precision = {"fp64": lib.FP64, "fp32": lib.FP32, "fp64-df": lib.FP64_DF, "fp64-exact": lib.FP64_EXACT}[
        precision_name]
    elem = 4 if precision_name == "fp32" else 8
    s = lib.Solver("euler3", "hll3", "weno2", "rungekutta3", "periodic", (n, n, n), (0, 0, 0), (2 * math.pi,) * 3,
                   gamma=1.4, cfl=0.4, precision=precision)
    try:
        s.set_primitive(lib.init_taylor_green(n))
        cands = s.candidates()
        if candidate >= 0:
            s.select_candidate(candidate)
            chosen, tune_ms = candidate, [-1.0] * len(cands)
        else:
            chosen, tune_ms = s.autotune()
        s.advance(1e9, 0, warmup)
        stream = torch.cuda.ExternalStream(s.stream())
        flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        s.profile(True)
        s.profile_read()
        total = 0.0
        with ClockSampler(0) as clocks:
            for i in range(steps):
                a0 = torch.cuda.Event(enable_timing=True)
                a1 = torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    flush.fill_(i & 0xFF)
                    a0.record(stream)
                s.advance(1e9, 0, 1)
                with torch.cuda.stream(stream):
                    a1.record(stream)
                torch.cuda.synchronize()
                total += a0.elapsed_time(a1)
        stage_ms, stage_n, _ = s.profile_read()
    finally:
        s.close()
    del flush
    cells = n ** 3
    launch_ms = stage_ms / max(stage_n, 1)
    alg = 8 * 5 * elem / 3 * cells
    peak = measured_peaks()
    return {"metric": METRIC, "value": cells * steps / (total * 1e-3), "unit": METRIC, "steps": steps,
            "warmup": warmup, "ms_per_step": total / steps, "dtype": precision_name,
            "workload": "tg3d_%d_euler3_weno2_hll3_rk3" % n, "grid": [n, n, n],
            "l2": "flushed before every timed step (512 MiB memset)",
            "stage_kernel": {"candidate": chosen, "tile": list(cands[chosen][0]), "threads": cands[chosen][1],
                             "tma": cands[chosen][2],
                             "autotune_ms_per_launch": [{"tile": list(c[0]), "threads": c[1], "tma": c[2], "ms": m}
                                                        for c, m in zip(cands, tune_ms)]},
            "stage_launch_ms": launch_ms,
            "roofline": {"bound": "hbm", "achieved": alg / (launch_ms * 1e-3) / 1e9, "peak": peak[0], "unit": "GB/s",
                         "frac": alg / (launch_ms * 1e-3) / 1e9 / peak[0], "alg_bytes_per_launch": alg,
                         "peak_source": peak[1],
                         "note": "FP64 builds are FP64-pipe bound (75 % of the pipe, "
                                 "profiles/stage_kernel_tg128_fp64.md)" if elem == 8 else
                                 "FP32: arithmetic-bound stencil"},
            "clocks": clocks.summary()}


def run_tg(args):
    """`--workload tg`: the Taylor-Green measurement as its own line."""
    m = measure_tg(args.tg_n, args.precision, args.steps, args.warmup, args.candidate)
    line = {"metric": METRIC, "value": m["value"], "unit": METRIC, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.precision, "data": "synthetic (Taylor-Green initial data)",
            "config": {"workload": m["workload"], "grid": m["grid"], "precision": args.precision, "l2": m["l2"]},
            "stage_kernel": m["stage_kernel"], "stage_launch_ms": m["stage_launch_ms"], "roofline": m["roofline"],
            "clocks": m["clocks"]}
    print(json.dumps(line), flush=True)


def measure_sod(warmup=1):
    """The Sod configuration (euler1, 2048 cells on [-5, 5], Neumann, WENO2,
    HLL3, SSP-RK3, CFL 0.475) run from t = 0 to its end time 1.3 in FP64 with
    the writer's dt clamp (one save): `warmup` untimed whole runs, then one
    timed run from the initial data, CUDA events on the solver's stream around
    the advance. A 2048-cell grid is latency bound (one 16-step CUDA graph per
    16 steps, a few microseconds per stage launch)."""
    import torch
    from alsvinn_gb300 import lib

    prim = lib.init_sod(2048)
    s = lib.Solver("euler1", "hll3", "weno2", "rungekutta3", "neumann", (2048, 1, 1), (-5, 0, 0), (5, 1, 1),
                   gamma=1.4, cfl=0.475, precision=lib.FP64)
    try:
        for _ in range(warmup):
            s.set_primitive(prim)
            s.advance(1.3, 1)
        s.set_primitive(prim)
        stream = torch.cuda.ExternalStream(s.stream())
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with ClockSampler(0) as clocks:
            with torch.cuda.stream(stream):
                a0.record(stream)
            s.advance(1.3, 1)
            with torch.cuda.stream(stream):
                a1.record(stream)
            torch.cuda.synchronize()
        ms = a0.elapsed_time(a1)
        t, steps, _ = s.time()
    finally:
        s.close()
    return {"metric": METRIC, "value": 2048 * steps / (ms * 1e-3), "unit": METRIC, "dtype": "f64",
            "workload": "sod1d_2048_euler1_weno2_hll3_rk3_to_t1.3", "end_time": t, "steps": steps,
            "ms_to_end_time": ms, "us_per_step": 1e3 * ms / steps, "warmup_runs": warmup,
            "bound": "launch / latency (2048 cells: 8 CTAs per stage)", "clocks": clocks.summary()}


UQ_SIZES = (128, 256, 512)
UQ_SCHEME = ("euler2", "hll3", "weno2", "rungekutta3", "periodic")
UQ_T = 2.0


def uq_sizes(S):
    """Grid sizes of the first S members of the 4096-member ensemble: drawn
    uniformly from {128, 256, 512} (log-uniform in size) with a fixed seed."""
    import numpy as np
    rng = np.random.default_rng(20240611)
    return rng.choice(UQ_SIZES, size=max(S, 4096))[:S]


def measure_uq(S, plain_per_size, warmup, candidate=-1):
    """Batched UQ ensemble: S Kelvin-Helmholtz members (generator sample =
    member index, grids from uq_sizes), FP32 state, FP64 Welford mean /
    variance per grid size, every member advanced from t = 0 to T = 2 in one
    ensemble (one persistent launch per RK stage, one graph per step). The
    timed region is the whole advance to T with the members resident in HBM;
    samples/s = S / that time. The plain FP64 path solves members one at a
    time to T = 2 as well (plain_per_size members of each grid size, the
    first ones of the ensemble); its samples/s is S over the time those
    measured per-size means give for the ensemble's mix."""
    import numpy as np
    import torch
    from alsvinn_gb300 import lib

    sizes = uq_sizes(S)
    counts = {int(n): int((sizes == n).sum()) for n in UQ_SIZES}
    probe = lib.Batch(*UQ_SCHEME, 1 << 20, 1, gamma=1.4, cfl=0.4, precision=lib.FP32)
    pool = sum(probe.member_bytes((int(n), int(n), 1)) for n in sizes) + (64 << 20)
    probe.close()

    def build():
        b = lib.Batch(*UQ_SCHEME, pool, S, gamma=1.4, cfl=0.4, precision=lib.FP32)
        if candidate >= 0:
            b.select_candidate(candidate)
        slots = [b.add((int(n), int(n), 1), (0, 0, 0), (1, 1, 0), lib.init_kelvin_helmholtz(int(n), sample=i),
                       group=UQ_SIZES.index(int(n))) for i, n in enumerate(sizes)]
        return b, slots

    # warm-up ensemble of the same members: a few steps (the ensemble
    # autotuner runs here and caches its choice for the scheme)
    wb, _ = build()
    wb.advance(UQ_T, 1, warmup)
    torch.cuda.synchronize()
    tune_ms = wb.autotune_result()
    wb.close()

    t0 = time.perf_counter()
    b, slots = build()
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.stream())
    launches0 = b.launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        e0.record(stream)
        b.advance(UQ_T, 1, 0)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    gpu_ms = e0.elapsed_time(e1)
    launches = b.launches() - launches0
    steps = {}
    cell_updates = 0
    for i, n in enumerate(sizes):
        t, st = b.member_time(slots[i])
        if t != UQ_T:
            raise RuntimeError("member %d ended at t=%r, not T" % (i, t))
        steps.setdefault(int(n), []).append(st)
        cell_updates += int(n) ** 2 * st
    folded = {n: b.stats(UQ_SIZES.index(n), (n + 4) ** 2)[2] for n in UQ_SIZES if counts[n]}
    cand, tma_members = b.current_candidate()
    b.close()
    probe = lib.Solver(*UQ_SCHEME, (128, 128, 1), (0, 0, 0), (1, 1, 0), precision=lib.FP32)
    cands = probe.candidates()
    probe.close()
    stage_kernel = {"candidate": cand, "tile": list(cands[cand][0]), "threads": cands[cand][1],
                    "tma": cands[cand][2], "members_staged_by_tma": tma_members,
                    "autotune_ms_per_launch": [{"tile": list(c[0]), "threads": c[1], "tma": c[2], "ms": m}
                                               for c, m in zip(cands, tune_ms)]}

    # plain FP64, one solve at a time, each run from t = 0 to T
    plain = {}
    for n in UQ_SIZES:
        members = [i for i in range(S) if int(sizes[i]) == n][:plain_per_size]
        times = []
        for i in members:
            sv = lib.Solver(*UQ_SCHEME, (n, n, 1), (0, 0, 0), (1, 1, 0), gamma=1.4, cfl=0.4, precision=lib.FP64)
            sv.set_primitive(lib.init_kelvin_helmholtz(n, sample=i))
            sv.autotune()  # cached per scheme and grid, as a served process would have it
            st = torch.cuda.ExternalStream(sv.stream())
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            p0 = time.perf_counter()
            a0.record(st)
            sv.advance(UQ_T, 1, 0)
            a1.record(st)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - p0)
            t, nst, _ = sv.time()
            if t != UQ_T:
                raise RuntimeError("plain solve ended at t=%r" % t)
            sv.close()
        if times:
            plain[n] = {"members_timed": len(times), "mean_s_to_T": sum(times) / len(times)}
    plain_time = sum(counts[n] * plain[n]["mean_s_to_T"] for n in UQ_SIZES if counts[n])
    plain_rate = S / plain_time
    return {"metric": "UQ samples/s", "value": S / wall, "unit": "samples/s", "samples": S,
            "size_counts": {str(n): counts[n] for n in UQ_SIZES}, "end_time": UQ_T,
            "wall_s_to_T": wall, "gpu_ms_to_T": gpu_ms, "setup_s": setup_s,
            "steps_to_T": {str(n): [min(v), max(v)] for n, v in sorted(steps.items())},
            "cell_updates_per_s": cell_updates / wall, "members_folded_per_size": {str(k): v for k, v in folded.items()},
            "dtype": "f32 state, f64 statistics", "stage_kernel": stage_kernel,
            "plain_fp64_one_at_a_time": {"samples_per_s": plain_rate, "per_size": {str(k): v for k, v in plain.items()},
                                         "method": "members solved one at a time to T = 2 (FP64, autotuned "
                                                   "single-grid path); the per-size mean time applied to the "
                                                   "ensemble's size mix"},
            "speedup_vs_plain_fp64": (S / wall) / plain_rate,
            "measured": "every member run from t = 0 to T = 2 inside the timed region (no extrapolation)",
            "gpu_launches": int(launches), "clocks": clocks.summary()}


def run_uq_steps(args):
    """A fixed number of ensemble steps (profiler runs): the first
    `--uq-samples` members, `--warmup` steps, then `--uq-steps` timed steps."""
    import torch
    from alsvinn_gb300 import lib

    S = args.uq_samples
    sizes = uq_sizes(S)
    probe = lib.Batch(*UQ_SCHEME, 1 << 20, 1, gamma=1.4, cfl=0.4, precision=lib.FP32)
    pool = sum(probe.member_bytes((int(n), int(n), 1)) for n in sizes) + (64 << 20)
    probe.close()
    b = lib.Batch(*UQ_SCHEME, pool, S, gamma=1.4, cfl=0.4, precision=lib.FP32)
    if args.candidate >= 0:
        b.select_candidate(args.candidate)
    for i, n in enumerate(sizes):
        b.add((int(n), int(n), 1), (0, 0, 0), (1, 1, 0), lib.init_kelvin_helmholtz(int(n), sample=i),
              group=UQ_SIZES.index(int(n)))
    b.advance(UQ_T, 1, args.warmup)
    stream = torch.cuda.ExternalStream(b.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    b.advance(UQ_T, 1, args.uq_steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = float(sum(int(n) ** 2 for n in sizes))
    cand, tma = b.current_candidate()
    b.close()
    print(json.dumps({"metric": "ensemble cell-updates/s", "value": cells * args.uq_steps / (ms * 1e-3),
                      "unit": "cell-updates/s", "samples": S, "steps": args.uq_steps, "ms_per_step":
                      ms / args.uq_steps, "candidate": cand, "members_staged_by_tma": tma}), flush=True)


def run_uq(args):
    if args.uq_steps > 0:
        return run_uq_steps(args)
    r = measure_uq(args.uq_samples, args.uq_plain, args.warmup, args.candidate)
    line = {"metric": r["metric"], "value": r["value"], "unit": r["unit"], "n_gpus": 1, "steps": None,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": r["dtype"],
            "data": "synthetic (seeded KH perturbation per member, generator sample = member index)",
            "config": {"workload": "uq_kh_%d_samples_128_256_512_fp32_to_T2" % args.uq_samples,
                       "samples": args.uq_samples, "l2": "working set of the ensemble >> L2"},
            "e2e": None}
    line.update({k: v for k, v in r.items() if k not in line})
    print(json.dumps(line), flush=True)


def _l1_scaled(a, b):
    """Per-variable sum|a-b| over max(sum|b| of the variable, of variable 0)."""
    import numpy as np
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    den = np.maximum(np.abs(b).sum(axis=1), np.abs(b[0]).sum())
    return np.abs(a - b).sum(axis=1) / den


def run_uq_error(args):
    """Error of the UQ ensemble's statistics against the FP64 reference at the
    UQ configuration's grids, end time and save times: per grid size the
    first `--uq-error-members` members of the 4096-member ensemble, run as
    three ensembles -- GBFV_FP64_EXACT (bit-identical to the reference CPU
    path at any length, so it is the FP64 oracle), GBFV_FP64 and GBFV_FP32 --
    with mean / variance at 8 save times up to T = 2; per save time the
    per-variable L1 error of the mean and of the variance over the interior
    (scaled by max(the variable's L1 norm, the density's))."""
    import numpy as np
    from alsvinn_gb300 import lib

    M = args.uq_error_members
    saves = 8
    sizes = uq_sizes(4096)
    out = {}
    t0 = time.perf_counter()
    for n in UQ_SIZES:
        members = [i for i in range(4096) if int(sizes[i]) == n][:M]
        total = (n + 4) ** 2
        stats = {}
        for name, prec in (("fp64_exact", lib.FP64_EXACT), ("fp64", lib.FP64), ("fp32", lib.FP32)):
            probe = lib.Batch(*UQ_SCHEME, 1 << 20, 1, gamma=1.4, cfl=0.4, precision=prec)
            pool = len(members) * probe.member_bytes((n, n, 1)) + (16 << 20)
            probe.close()
            with lib.Batch(*UQ_SCHEME, pool, len(members), gamma=1.4, cfl=0.4, precision=prec) as b:
                b.set_statistics_saves(saves)
                for i in members:
                    b.add((n, n, 1), (0, 0, 0), (1, 1, 0), lib.init_kelvin_helmholtz(n, sample=i), group=0)
                b.advance(UQ_T, saves, 0)
                per_save = []
                for k in range(saves):
                    cnt, mean, m2 = b.stats_export(0, total, save=k)
                    if cnt != len(members):
                        raise RuntimeError("save %d folded %d of %d members" % (k, cnt, len(members)))
                    g = 2
                    sl = lambda X: X.reshape(4, n + 4, n + 4)[:, g:-g, g:-g]
                    per_save.append((sl(mean), sl(m2 / cnt)))
                stats[name] = per_save
        ref = stats["fp64_exact"]
        rows = []
        for k in range(saves):
            row = {"t": UQ_T * (k + 1) / saves}
            for name in ("fp64", "fp32"):
                m, v = stats[name][k]
                row[name] = {"mean": [float(x) for x in _l1_scaled(m, ref[k][0])],
                             "variance": [float(x) for x in _l1_scaled(v, ref[k][1])]}
            rows.append(row)
        out[str(n)] = {"members": len(members), "per_save": rows}
    line = {"metric": "UQ statistics L1 error vs FP64 reference", "unit": "relative L1 (per variable)",
            "value": max(max(r["fp32"]["variance"]) for v in out.values() for r in v["per_save"][-1:]),
            "config": {"workload": "uq_kh_128_256_512_to_T2_first_members", "members_per_size": M,
                       "saves": saves, "reference": "GBFV_FP64_EXACT ensembles (bit-identical to the reference CPU "
                                                    "path)", "variables": ["rho", "mx", "my", "E"]},
            "errors": out, "wall_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


SERVE_BUDGET = 120 * (1 << 30)


def serve_requests(R, rate):
    """R requests with Poisson arrivals at `rate` per second (fixed seed),
    about half 1D Burgers (1024-8192 cells, T = 0.5, phase U[-1, 1]) and half
    2D Kelvin-Helmholtz (128^2-1024^2, T = 1.0, generator sample = request
    index), sizes uniform over the powers of two."""
    import numpy as np
    from alsvinn_gb300 import lib
    rng = np.random.default_rng(20240612)
    gaps = rng.exponential(1.0 / rate, size=R)
    arrivals = np.cumsum(gaps) - gaps[0]
    kinds = rng.integers(0, 2, size=R)
    reqs = []
    for i in range(R):
        if kinds[i] == lib.REQUEST_BURGERS:
            n = int(rng.choice([1024, 2048, 4096, 8192]))
            reqs.append((lib.REQUEST_BURGERS, n, 0.5, float(rng.uniform(-1, 1)), 0, float(arrivals[i])))
        else:
            n = int(rng.choice([128, 256, 512, 1024]))
            reqs.append((lib.REQUEST_KELVIN_HELMHOLTZ, n, 1.0, 0.0, i, float(arrivals[i])))
    return reqs


def serve_batched(reqs, chunk):
    """Serves `reqs` through the continuous-batching loop (FP32 state, FP64
    statistics, 120 GB budget); returns (wall s, results, launches, clocks)."""
    from alsvinn_gb300 import lib
    s = lib.Server(SERVE_BUDGET, precision=lib.FP32, max_slots=4096)
    ids = [s.submit(k, n, T, phase=ph, sample=sm, arrival=a) for (k, n, T, ph, sm, a) in reqs]
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        s.run(chunk)
        wall = time.perf_counter() - t0
    res = [s.result(i) for i in ids]
    launches = s.launches()
    s.close()
    return wall, res, launches, clocks.summary()


def serve_plain_fp64(reqs):
    """The same requests solved by plain FP64 solvers one at a time, first
    come first served, each started no earlier than its arrival (real time)."""
    import torch
    from alsvinn_gb300 import lib
    lat, steps, busy = [], [], []
    t0 = time.perf_counter()
    for (k, n, T, ph, sm, a) in reqs:
        now = time.perf_counter() - t0
        if now < a:
            time.sleep(a - now)
        b0 = time.perf_counter()
        if k == lib.REQUEST_BURGERS:
            sv = lib.Solver("burgers", "godunov", "weno2", "rungekutta2", "periodic", (n, 1, 1), (0, 0, 0),
                            (1, 1, 1), cfl=0.475, precision=lib.FP64)
            sv.set_primitive(lib.init_burgers_sine(n, ph))
        else:
            sv = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (n, n, 1), (0, 0, 0), (1, 1, 0),
                            cfl=0.4, precision=lib.FP64)
            sv.set_primitive(lib.init_kelvin_helmholtz(n, sample=sm))
        sv.advance(T, 1, 0)
        torch.cuda.synchronize()
        steps.append(sv.time()[1])
        sv.close()
        busy.append(time.perf_counter() - b0)
        lat.append(time.perf_counter() - t0 - a)
    wall = time.perf_counter() - t0
    return wall, lat, steps, busy


def measure_serve(R, rate, chunk, plain_subset):
    """Serving stream: R requests through the continuous-batching loop
    (latency = completion - arrival, samples/s = completed / wall from the
    first arrival); then the first `plain_subset` requests of the same
    stream, run both ways -- batched, and plain FP64 one at a time FIFO --
    for a measured comparison on equal work."""
    import numpy as np
    reqs = serve_requests(R, rate)
    wall, res, launches, clk = serve_batched(reqs, chunk)
    lat = np.array([r["finish"] - r["arrival"] for r in res])
    done = sum(1 for r in res if r["status"] == 2)
    sub = reqs[:plain_subset]
    swall, sres, _, sclk = serve_batched(sub, chunk)
    slat = np.array([r["finish"] - r["arrival"] for r in sres])
    pwall, plat, _, pbusy = serve_plain_fp64(sub)
    plat = np.array(plat)
    sub_rate = len(sub) / swall
    plain_rate = len(sub) / pwall
    # capacity: the same requests all present at t = 0 (batched: one run;
    # plain: the sum of the measured one-at-a-time solve times)
    cwall, cres, _, cclk = serve_batched([r[:5] + (0.0,) for r in sub], chunk)
    cap_batched = len(sub) / cwall
    cap_plain = len(sub) / sum(pbusy)
    kinds = {}
    for (k, n, T, ph, sm, a) in reqs:
        key = "%s_%d" % ("burgers1d" if k == 0 else "kh2d", n)
        kinds[key] = kinds.get(key, 0) + 1
    return {"metric": "serving samples/s", "value": done / wall, "unit": "samples/s", "requests": R,
            "rate_per_s": rate, "completed": done, "wall_s": wall,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "mix": kinds, "budget_bytes": SERVE_BUDGET, "steps_per_chunk": chunk,
            "dtype": "f32 state, f64 statistics",
            "subset_comparison": {
                "requests": len(sub), "batched_fp32": {"samples_per_s": sub_rate,
                                                        "latency_p50_s": float(np.percentile(slat, 50)),
                                                        "latency_p99_s": float(np.percentile(slat, 99)),
                                                        "clocks": sclk},
                "plain_fp64_one_at_a_time": {"samples_per_s": plain_rate,
                                             "latency_p50_s": float(np.percentile(plat, 50)),
                                             "latency_p99_s": float(np.percentile(plat, 99)),
                                             "method": "run: FP64 solver per request, FIFO, each started no "
                                                       "earlier than its arrival"},
                "speedup_vs_plain_fp64": sub_rate / plain_rate,
                "capacity": {"batched_fp32_samples_per_s": cap_batched, "plain_fp64_samples_per_s": cap_plain,
                             "speedup": cap_batched / cap_plain, "clocks": cclk,
                             "method": "the subset's requests all present at t = 0: batched wall time of one "
                                       "run; plain = the sum of its measured one-at-a-time solve times"}},
            "gpu_launches": int(launches), "clocks": clk}


def run_serve(args):
    r = measure_serve(args.serve_requests, args.serve_rate, args.serve_chunk, args.serve_plain)
    line = {"metric": r["metric"], "value": r["value"], "unit": r["unit"], "n_gpus": 1, "steps": None,
            "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": r["dtype"], "data": "synthetic (Poisson arrivals, seeded phases / perturbations)",
            "config": {"workload": "serve_burgers1d_kh2d_mix", "requests": args.serve_requests,
                       "rate_per_s": args.serve_rate}, "e2e": None}
    line.update({k: v for k, v in r.items() if k not in line})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="kh1024", choices=["kh1024", "uq", "serve", "uq-error", "tg"])
    ap.add_argument("--tg-n", type=int, default=256, help="cells per dimension of --workload tg")
    ap.add_argument("--uq-error-members", type=int, default=8, help="members per grid size of --workload uq-error")
    ap.add_argument("--serve-requests", type=int, default=128)
    ap.add_argument("--serve-rate", type=float, default=2.0)
    ap.add_argument("--serve-chunk", type=int, default=256,
                    help="time steps per ensemble advance between admissions (larger chunks: fewer host round trips)")
    ap.add_argument("--serve-plain", type=int, default=12,
                    help="requests of the stream also run by plain FP64 one at a time")
    ap.add_argument("--uq-samples", type=int, default=4096)
    ap.add_argument("--uq-plain", type=int, default=2, help="plain FP64 solves to T per grid size")
    ap.add_argument("--uq-steps", type=int, default=0,
                    help="--workload uq: a fixed number of ensemble steps instead of the run to T (profiler runs)")
    ap.add_argument("--headline-uq-samples", type=int, default=192,
                    help="members of the UQ ensemble measured to T inside the default run (0: skip)")
    ap.add_argument("--headline-serve-requests", type=int, default=96,
                    help="requests of the serving stream measured inside the default run (0: skip)")
    ap.add_argument("--headline-fv", type=int, default=1,
                    help="add the Sod 2048 and Taylor-Green 256^3 measurements to the headline line (0: skip)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500,
                    help="timed steps (the default keeps the headline's timed region near one second, "
                         "so the clock samples fall inside it)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=200)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64-df", "fp64-exact", "fp32"])
    ap.add_argument("--no-df", action="store_true", help="skip the double-float measurement")
    ap.add_argument("--candidate", type=int, default=-1,
                    help="pin this stage kernel configuration instead of autotuning (profiler runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "uq":
        run_uq(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "uq-error":
        run_uq_error(args)
    elif args.workload == "tg":
        run_tg(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
