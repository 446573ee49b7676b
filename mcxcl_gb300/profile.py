"""Run a few launches of the transport kernel on a named workload, for a
profiler to capture (e.g. ``ncu -k regex:mcx_transport -s 2 -c 1 python -m
mcxcl_gb300.profile --config 2 --photons 2e7``).

The problem is uploaded once (mcx_prepare_simulation); each launch runs all
photons on the resident data, as the benchmark's device-resident loop does.
"""
import argparse
import ctypes

from . import _lib, pmcxcl, workloads


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--config", type=int, default=2, help="workload: 1 cube, 2 cube+sphere+detectors, 3 head")
    ap.add_argument("--photons", type=float, default=2e7)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--block", type=int, default=256)
    ap.add_argument("--blocks-per-sm", type=int, default=3)
    ap.add_argument("--aggregate", action="store_true", help="warp-aggregate deposits")
    ap.add_argument("--exact", action="store_true", help="the IEEE-only kernel")
    args = ap.parse_args(argv)
    L = _lib.load()
    cfg = workloads.config(args.config)
    cfg["nphoton"] = int(args.photons)
    C = _lib.Config()
    pmcxcl.parse_config(cfg, C)
    L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    pmcxcl._check(C)
    s = L.mcx_prepare_simulation(ctypes.byref(C))
    pmcxcl._check(C)
    L.mcxg_set_launch(s, args.block, args.blocks_per_sm)
    flags = (1 if args.exact else 0) | (16 if args.aggregate else 2)
    ms = ctypes.c_float()
    for i in range(args.launches):
        rc = L.mcxg_simulate(s, flags, ctypes.byref(ms))
        if rc:
            raise RuntimeError(L.mcxg_error_string(rc).decode())
        print("launch %d: %.3f ms, %.1f photons/ms" % (i, ms.value, args.photons / ms.value), flush=True)
    L.mcx_clearcfg(ctypes.byref(C))


if __name__ == "__main__":
    main()
