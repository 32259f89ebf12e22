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
    from alsvinn_gb300 import lib
    return lib.init_kelvin_helmholtz(n, sample=sample)


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
    precision = {"fp64": lib.FP64, "fp64-df": lib.FP64_DF, "fp64-exact": lib.FP64_EXACT}[args.precision]
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
    state_bytes = NVAR * s.total * 8
    e2e = {"value": world * cells * e2e_steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "steps": e2e_steps}

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
    alg_bytes_per_launch = cells * BYTES_PER_CELL_STEP / 3.0
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
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded KH interface perturbation, sample = rank)",
                "config": {"workload": WORKLOAD, "grid": [N, N], "equation": "euler2", "reconstruction": "weno2",
                           "flux": "hll3", "integrator": "rungekutta3", "precision": args.precision,
                           "l2": "flushed before every timed step (512 MiB memset, outside the events)",
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "stage_kernel": stage_kernel},
                "roofline": roofline, "cpu_baseline": base, "e2e": e2e, "clocks": clk,
                "gpu_launches": int(launches1 - launches0), "fp64_df": df,
                "sim": {"t": t_sim, "steps": steps_done}}
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_uq(args):
    """Batched UQ ensemble: `--uq-samples` Kelvin-Helmholtz samples, each with
    its own seeded perturbation (generator sample = member index), grid sizes
    drawn uniformly from {128^2, 256^2, 512^2} (log-uniform in size) with a
    fixed seed, FP32 state, FP64 Welford statistics per grid size at T = 2.
    The whole ensemble advances `--steps` time steps per timed region, each
    member with its own dt. samples/s is extrapolated to T = 2 from the
    measured ensemble cell-update rate and each size's initial dt; the plain
    FP64 one-solve-at-a-time path is timed per size the same way and
    extrapolated identically, so the ratio compares equal work."""
    import numpy as np
    import torch
    from alsvinn_gb300 import lib

    S = args.uq_samples
    sizes_choice = (128, 256, 512)
    rng = np.random.default_rng(20240611)
    sizes = rng.choice(sizes_choice, size=S)
    T = 2.0
    scheme = ("euler2", "hll3", "weno2", "rungekutta3", "periodic")
    b0 = lib.Batch(*scheme, 1 << 20, 1, gamma=1.4, cfl=0.4, precision=lib.FP32)
    pool = sum(b0.member_bytes((int(n), int(n), 1)) for n in sizes) + (64 << 20)
    b0.close()
    t0 = time.perf_counter()
    b = lib.Batch(*scheme, pool, S, gamma=1.4, cfl=0.4, precision=lib.FP32)
    if args.candidate >= 0:
        b.select_candidate(args.candidate)
    slots = []
    for s in range(S):
        n = int(sizes[s])
        slots.append(b.add((n, n, 1), (0, 0, 0), (1, 1, 0), lib.init_kelvin_helmholtz(n, sample=s),
                           group=sizes_choice.index(n)))
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(b.stream())
    b.advance(T, 1, args.warmup)
    torch.cuda.synchronize()
    # each size's dt after warm-up -> steps to T
    dts = {}
    for s in range(S):
        n = int(sizes[s])
        if n not in dts:
            t, st = b.member_time(slots[s])
            dts[n] = t / st
    launches0 = b.launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clocks:
        e0.record(stream)
        b.advance(T, 1, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = b.launches() - launches0
    cand, tma_members = b.current_candidate()
    tune_ms = b.autotune_result()
    cells = float(sum(int(n) ** 2 for n in sizes))
    rate = cells * args.steps / (ms * 1e-3)
    work_to_T = sum((int(n) ** 2) * (T / dts[int(n)]) for n in sizes)
    samples_per_s = S * rate / work_to_T
    b.close()
    probe = lib.Solver(*scheme, (128, 128, 1), (0, 0, 0), (1, 1, 0), precision=lib.FP32)
    cands = probe.candidates()
    probe.close()
    stage_kernel = {"candidate": cand, "tile": list(cands[cand][0]), "threads": cands[cand][1],
                    "tma": cands[cand][2], "members_staged_by_tma": tma_members,
                    "autotune_ms_per_launch": [{"tile": list(c[0]), "threads": c[1], "tma": c[2], "ms": m}
                                               for c, m in zip(cands, tune_ms)],
                    "autotune_score": "mean stage launch of one RK3 step over all members: (MODE_L + 2 x stage 1) / 3"}

    # plain FP64, one solve at a time, each size
    plain_step_ms = {}
    for n in sizes_choice:
        sv = lib.Solver(*scheme, (n, n, 1), (0, 0, 0), (1, 1, 0), gamma=1.4, cfl=0.4, precision=lib.FP64)
        sv.set_primitive(lib.init_kelvin_helmholtz(n, sample=0))
        sv.advance(T, 1, 3)
        st = torch.cuda.ExternalStream(sv.stream())
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        k = max(5, args.steps // 2)
        a0.record(st)
        sv.advance(T, 1, k)
        a1.record(st)
        torch.cuda.synchronize()
        plain_step_ms[n] = a0.elapsed_time(a1) / k
        sv.close()
    plain_time_to_T = sum(plain_step_ms[int(n)] * 1e-3 * (T / dts[int(n)]) for n in sizes)
    plain_samples_per_s = S / plain_time_to_T
    line = {"metric": "UQ samples/s", "value": samples_per_s, "unit": "samples/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 state, f64 statistics",
            "data": "synthetic (seeded KH perturbation per member, generator sample = member index)",
            "config": {"workload": "uq_kh_%d_samples_128_256_512_fp32" % S, "samples": S,
                       "size_counts": {str(n): int((sizes == n).sum()) for n in sizes_choice},
                       "end_time": T, "l2": "working set %.1f GB >> L2" % (pool / 1e9),
                       "stage_kernel": stage_kernel},
            "batched_cell_updates_per_s": rate,
            "plain_fp64_one_at_a_time_samples_per_s": plain_samples_per_s,
            "speedup_vs_plain_fp64": samples_per_s / plain_samples_per_s,
            "plain_fp64_step_ms": {str(k): v for k, v in plain_step_ms.items()},
            "initial_dt": {str(k): v for k, v in dts.items()},
            "extrapolation": "samples/s = samples * measured rate / sum_i n_i^2 * (T / dt_i(initial))",
            "setup_s": setup_s, "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving stream: `--serve-requests` solve requests with Poisson arrivals
    at `--serve-rate` per second (fixed seed), half 1D Burgers (1024-8192 cells,
    periodic, Godunov, WENO2, RK2, T=0.5, random phase U[-1,1]) and half 2D
    Kelvin-Helmholtz (128^2-1024^2, seeded perturbation, T=1.0), grid sizes
    log-uniform, FP32 state, FP64 statistics, 120 GB HBM budget. Latency is
    completion minus arrival. The plain FP64 one-at-a-time comparison uses
    measured FP64 step times per (kind, size) and each request's step count,
    served first-come first-served one after another on the same arrivals."""
    import numpy as np
    import torch
    from alsvinn_gb300 import lib

    rng = np.random.default_rng(20240612)
    R = args.serve_requests
    gaps = rng.exponential(1.0 / args.serve_rate, size=R)
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
    budget = 120 * (1 << 30)
    s = lib.Server(budget, precision=lib.FP32, max_slots=4096)
    ids = [s.submit(k, n, T, phase=ph, sample=sm, arrival=a) for (k, n, T, ph, sm, a) in reqs]
    t0 = time.perf_counter()
    with ClockSampler(0) as clocks:
        s.run(args.serve_chunk)
    wall = time.perf_counter() - t0
    res = [s.result(i) for i in ids]
    launches = s.launches()
    s.close()
    lat = np.array([r["finish"] - r["arrival"] for r in res])
    done = sum(1 for r in res if r["status"] == 2)
    steps = [r["steps"] for r in res]

    # plain FP64, one solve at a time: measured step time per (kind, n)
    step_ms = {}
    for (k, n) in sorted({(r[0], r[1]) for r in reqs}):
        if k == lib.REQUEST_BURGERS:
            sv = lib.Solver("burgers", "godunov", "weno2", "rungekutta2", "periodic", (n, 1, 1), (0, 0, 0),
                            (1, 1, 1), cfl=0.475, precision=lib.FP64)
            sv.set_primitive(lib.init_burgers_sine(n, 0.3))
            T = 0.5
        else:
            sv = lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", (n, n, 1), (0, 0, 0), (1, 1, 0),
                            cfl=0.4, precision=lib.FP64)
            sv.set_primitive(lib.init_kelvin_helmholtz(n, sample=0))
            T = 1.0
        sv.advance(T, 1, 5)
        st = torch.cuda.ExternalStream(sv.stream())
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        kk = 40 if k == lib.REQUEST_BURGERS else 10
        a0.record(st)
        sv.advance(T, 1, kk)
        a1.record(st)
        torch.cuda.synchronize()
        step_ms[(k, n)] = a0.elapsed_time(a1) / kk
        sv.close()
    clock = 0.0
    plain_lat = []
    for (k, n, T, ph, sm, a), nsteps in zip(reqs, steps):
        start = max(clock, a)
        clock = start + nsteps * step_ms[(k, n)] * 1e-3
        plain_lat.append(clock - a)
    plain_lat = np.array(plain_lat)
    plain_rate = R / (clock - arrivals[0])
    line = {"metric": "serving samples/s", "value": done / wall, "unit": "samples/s", "n_gpus": 1,
            "steps": int(sum(steps)), "warmup": 0, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 state, f64 statistics",
            "data": "synthetic (Poisson arrivals, seeded phases / perturbations)",
            "config": {"workload": "serve_burgers1d_kh2d_mix", "requests": R, "rate_per_s": args.serve_rate,
                       "budget_bytes": budget, "steps_per_chunk": args.serve_chunk},
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
            "completed": done, "wall_s": wall,
            "plain_fp64_one_at_a_time": {"samples_per_s": plain_rate,
                                         "latency_p50_s": float(np.percentile(plain_lat, 50)),
                                         "latency_p99_s": float(np.percentile(plain_lat, 99)),
                                         "method": "measured FP64 step time per (kind, n) x each request's "
                                                   "steps, served FIFO one at a time on the same arrivals"},
            "speedup_vs_plain_fp64": (done / wall) / plain_rate,
            "fp64_step_ms": {"%s_%d" % ("burgers" if k == 0 else "kh", n): v for (k, n), v in step_ms.items()},
            "gpu_launches": int(launches), "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="kh1024", choices=["kh1024", "uq", "serve"])
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=8.0)
    ap.add_argument("--serve-chunk", type=int, default=16)
    ap.add_argument("--uq-samples", type=int, default=4096)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=60)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64-df", "fp64-exact"])
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
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
