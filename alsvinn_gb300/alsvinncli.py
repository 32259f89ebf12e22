"""Command line front end for one deterministic run, the counterpart of
alsvinncli (alsvinncli/src/main.cpp:40-270):

    python -m alsvinn_gb300.alsvinncli input.xml [--precision fp64] [--output-dir DIR]

Reads the XML, evaluates the initial data program at the cell midpoints,
calls the writers once, steps to the end time on the GPU, and prints a one
line JSON report. Errors print the reference's message form on stderr and
exit with status 1 (EXIT_FAILURE).
"""
import argparse
import json
import os
import sys
import time

from . import config, initdata, lib
from .simulator import PRECISIONS, Simulator


def main(argv=None):
    ap = argparse.ArgumentParser(prog="alsvinncli", description=__doc__.split("\n\n")[0])
    ap.add_argument("input", help="alsvinn XML configuration")
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default="fp64",
                    help="state / arithmetic precision on the GPU (default fp64)")
    ap.add_argument("--output-dir", default=None, help="directory for the writer's files (default: the XML's)")
    args = ap.parse_args(argv)
    try:
        cfg = config.read_config(args.input)
        out_dir = args.output_dir or cfg.base_path
        os.makedirs(out_dir, exist_ok=True)
        t0 = time.perf_counter()
        prim = initdata.evaluate(cfg.fvm.python_program, cfg.fvm.equation, cfg.fvm.lower, cfg.fvm.upper,
                                 cfg.fvm.dimension, cfg.fvm.init_parameters)
        sim = Simulator(cfg.fvm, PRECISIONS[args.precision], num_samples=cfg.uq.samples if cfg.uq else 1,
                        output_dir=out_dir)
        try:
            sim.set_initial_value(prim)
            print("Running simulator... ", flush=True)
            t1 = time.perf_counter()
            sim.call_writers()
            sim.run()
            sim.finalize()
            t2 = time.perf_counter()
            report = {"program": "alsvinncli", "name": sim.get_name(), "platform": cfg.fvm.platform,
                      "precision": args.precision, "timesteps": sim.get_number_of_timesteps(),
                      "end_time": sim.get_current_time(), "setup_ms": (t1 - t0) * 1e3,
                      "run_ms": (t2 - t1) * 1e3}
        finally:
            sim.close()
        print(json.dumps(report), flush=True)
        return 0
    except (config.ConfigError, initdata.InitialDataError, lib.GbfvError, RuntimeError, ValueError) as e:
        print("An error occured.", file=sys.stderr)
        print("The error message was:", file=sys.stderr)
        print(e, file=sys.stderr)
        return 1


if __name__ == "__main__":
    sys.exit(main())
