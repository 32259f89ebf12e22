"""Command line front end for a UQ ensemble, the counterpart of alsuqcli
(alsuqcli/src/main.cpp:36-190):

    python -m alsvinn_gb300.alsuqcli input.xml [--precision fp64] [--engine auto|batch|serial]
    torchrun --nproc-per-node N -m alsvinn_gb300.alsuqcli input.xml     (N GPUs, samples sharded)

The samples split into contiguous blocks over the ranks (one GPU each, as
--multi-sample does over MPI ranks); each rank runs its block, the FP64
Welford statistics combine in one all-gather, rank 0 writes them. Errors
exit with status 1.
"""
import argparse
import json
import os
import sys

from . import config, initdata, lib
from .runner import Runner
from .simulator import PRECISIONS


def main(argv=None):
    ap = argparse.ArgumentParser(prog="alsuqcli", description=__doc__.split("\n\n")[0])
    ap.add_argument("input", help="alsvinn XML configuration with a <uq> section")
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default="fp64")
    ap.add_argument("--engine", choices=("auto", "batch", "serial"), default="auto",
                    help="batch: all samples of a wave in one ensemble launch per RK stage; serial: one after "
                         "another (default: batch when the schedule allows it)")
    ap.add_argument("--multi-sample", type=int, default=None,
                    help="number of sample-parallel ranks; must equal the launched world size")
    ap.add_argument("--output-dir", default=None)
    args = ap.parse_args(argv)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    try:
        if args.multi_sample is not None and args.multi_sample != world:
            raise config.ConfigError("--multi-sample %d but %d ranks were launched" % (args.multi_sample, world))
        if world > 1:
            import torch
            import torch.distributed as dist
            if torch.cuda.is_available():
                torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
                dist.init_process_group("nccl")
            else:
                dist.init_process_group("gloo")
        cfg = config.read_config(args.input)
        out_dir = args.output_dir or cfg.base_path
        os.makedirs(out_dir, exist_ok=True)
        runner = Runner(cfg, PRECISIONS[args.precision], rank=rank, world_size=world, output_dir=out_dir,
                        engine=args.engine)
        results = runner.run()
        if rank == 0:
            print(json.dumps({"program": "alsuqcli", "name": cfg.fvm.name, "engine": runner.engine,
                              "precision": args.precision, "ranks": world, "samples": cfg.uq.samples,
                              "timesteps_rank0": runner.timesteps, "statistics_saves": len(results),
                              "wall_ms": runner.wall_s * 1e3}), flush=True)
        return 0
    except (config.ConfigError, initdata.InitialDataError, lib.GbfvError, RuntimeError, ValueError) as e:
        print("An error occured.", file=sys.stderr)
        print("The error message was:", file=sys.stderr)
        print(e, file=sys.stderr)
        return 1
    finally:
        if dist is not None and dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
