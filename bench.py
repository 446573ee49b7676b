"""Benchmark: photons/ms of the GB300 transport kernel on the cube-with-sphere
workload (60^3 voxels, radius-15 sphere of a second medium, Fresnel on, 50
gates of 0.1 ns, four disk detectors saving detector id, per-medium scatter
counts and partial paths; 1e8 photons per step).

One step = one full simulation of the workload.  Prints one JSON line.

  value  : photons / ms of kernel time with every input resident in HBM
           (the problem is uploaded once; each step launches the transport
           kernel on it; CUDA events on the launching stream; L2 flushed
           between steps by a 256 MB write, since the working set -- volume,
           field, records -- fits in L2).
  e2e    : the same metric through the public API (mcxcl_gb300.run) with host
           buffers: dict -> Config, validation, detector masking, upload of
           the volume and seeds, the kernel, FP64 reductions, readback of the
           normalised field and the detected-photon records.
  roofline: FP32 issue -- the kernel's FP32 operations from a frozen operation
           model (48 per step + 65 per scattering + 20 per launch + 10 per
           Fresnel test) times event counts measured by the exact kernel on a
           sample of the same workload, over kernel time, against the FP32
           issue peak measured in the same run.
  cpu_baseline: the CPU oracle (a C restatement of the reference kernel) on
           all host cores, on a bounded sample of the workload.

Also reported: "batched" -- the batched workload's simulations/s in one
persistent launch against one launch per simulation; "gradient" -- forward
and replay-backward times of the differentiation workload and the backward
pass's agreement with central differences.

Also: "c1" and "c3" -- the homogeneous cube and the synthetic layered head
(181 x 217 x 181, five labels, 16 detectors, roulette), each with its own
photons/ms, end-to-end photons/ms through mcxcl_gb300.run, FP32-issue
roofline and DRAM traffic; "precision" (with
--precision P) -- the error of the compensated field, a plain float field and
the reference's spill field against an FP64 accumulation of the same P
photons on the cube and the cube + sphere workloads.

--launches N --config K: profiling mode, N launches of workload K on
resident data (one line per launch), for a profiler to capture.

--impl reference times the reference's CPU path (the oracle, since the
reference's OpenCL build does not run on this machine) on the host cores.
Multi-GPU: replicas only (photons do not exchange anything); each rank runs
the full workload with its own seed.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# frozen FP32 operation model (weights per event)
OPS_PER_STEP, OPS_PER_SCATTER, OPS_PER_LAUNCH, OPS_PER_REFLECT = 48, 65, 20, 10
MUFU_PER_STEP, MUFU_PER_SCATTER = 6, 11
MUFU_PER_SM_CLK = 16          # special-function results per SM per clock
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "traffic_mcx_transport_config%d.txt")
# one name for the headline workload, printed by both arms
WORKLOAD = ("60^3 cube + r15 sphere (label 2), Fresnel on, 50 gates x 0.1 ns, 4 r=1 detectors on z=0 saving "
            "detid/nscat/ppath + seeds, pencil (29,29,0) +z, 1e8 photons per step")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--photons", type=float, default=None, help="override photons per step")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-sims", type=int, default=512, help="simulations in the batched comparison (0: skip)")
    ap.add_argument("--no-gradient", action="store_true", help="skip the replay-gradient timing")
    ap.add_argument("--no-configs", action="store_true", help="skip the cube and head sub-measurements")
    ap.add_argument("--precision", type=float, default=0, help="photons of the FP64 precision check (0: skip)")
    # profiling mode
    ap.add_argument("--launches", type=int, default=0, help="profiling mode: launches of --config on resident data")
    ap.add_argument("--config", type=int, default=2, help="profiling mode: 1 cube, 2 cube + sphere, 3 head")
    ap.add_argument("--block", type=int, default=0, help="profiling mode: threads per block (0: automatic)")
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="profiling mode: resident blocks per SM")
    ap.add_argument("--flags", type=int, default=0, help="profiling mode: mcxg_simulate flags")
    ap.add_argument("--tile", type=int, default=-1,
                    help="profiling mode: hot-voxel tile elements (0: off; default: the library's choice)")
    return ap.parse_args()


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples (every 200 ms) while the timed region runs."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(photons=None):
    from mcxcl_gb300 import workloads
    cfg = workloads.config(2)
    if photons:
        cfg["nphoton"] = int(photons)
    return cfg


def cpu_baseline(cfg, target_s=15.0, kind="port"):
    """The oracle on every host core, on a sample sized to ~target_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    ncores = os.cpu_count() or 1
    nthread = 16384
    # grow a probe until it runs for a tenth of the target, then scale to the target
    n = 20000
    while True:
        t0 = time.perf_counter()
        oracle.run(dict(cfg, nphoton=n), nthread=nthread, core=nthread, mathmode=oracle.MATH_LIBM, nworkers=ncores)
        dt = max(time.perf_counter() - t0, 1e-3)
        if dt >= 0.1 * target_s or n >= cfg["nphoton"]:
            break
        n = int(min(cfg["nphoton"], n * max(2.0, 0.15 * target_s / dt)))
    n = int(min(cfg["nphoton"], max(20000, n * target_s / dt)))
    sample = dict(cfg, nphoton=n)
    t0 = time.perf_counter()
    r = oracle.run(sample, nthread=nthread, core=nthread, mathmode=oracle.MATH_LIBM, nworkers=ncores)
    dt = time.perf_counter() - t0
    return {"value": n / (dt * 1e3), "unit": "photons/ms", "cores": ncores, "kind": kind,
            "sample": "%d photons of the %d-photon workload, %d reference threads, OpenMP over %d cores, %.1f s"
                      % (n, int(cfg["nphoton"]), nthread, ncores, dt),
            "absorbed": (r["stat"]["energytot"] - r["stat"]["energyesc"]) / r["stat"]["energytot"]}


def batch_measure(nsim):
    """The batched workload (nsim cubes of edge 32-128, random media and
    inclusions, 1e5-1e7 photons each): all of them in one persistent launch
    against the same simulations run one launch each, both through the
    public API with host inputs and outputs.  Each simulation runs the same
    photon count in both arms, so the fluence error is equal by construction."""
    import mcxcl_gb300
    from mcxcl_gb300 import workloads
    sims = workloads.batch_configs(nsim=nsim, master_seed=7)
    photons = float(sum(c["nphoton"] for c in sims))
    mcxcl_gb300.run_batch(sims[:2])
    mcxcl_gb300.run(sims[0])
    t0 = time.perf_counter()
    res = mcxcl_gb300.run_batch(sims)
    tb = time.perf_counter() - t0
    kb = res[0]["stat"]["kernelms"]
    t0 = time.perf_counter()
    ks = 0.0
    for c in sims:
        ks += mcxcl_gb300.run(c)["stat"]["kernelms"]
    ts = time.perf_counter() - t0
    # precision: the batched launch with every deposit also accumulated in FP64
    sub = sims[:64]
    ver = mcxcl_gb300.run_batch(sub, verify=True)
    prec = {"simulations": len(sub),
            "relerr_max": max(r["stat"]["relerr_max"] for r in ver),
            "relerr_median_max": max(r["stat"]["relerr_median"] for r in ver),
            "relerr_total_max": max(r["stat"]["relerr_total"] for r in ver)}
    # error of each arm: two independent runs (seed, seed + 1) of 8 of the
    # simulations; per-voxel RSE = |a - b| / sqrt(2) / mean over voxels holding
    # at least 1% of the simulation's peak fluence
    rse = {"batched": [], "one_launch_per_sim": []}
    pick = [sims[i] for i in range(0, nsim, max(1, nsim // 8))][:8]
    alt = [dict(c, seed=int(c["seed"]) + 1) for c in pick]
    pairs = {"batched": zip(mcxcl_gb300.run_batch(pick), mcxcl_gb300.run_batch(alt)),
             "one_launch_per_sim": [(mcxcl_gb300.run(c), mcxcl_gb300.run(d)) for c, d in zip(pick, alt)]}
    for arm, pr in pairs.items():
        for ra, rb in pr:
            fa, fb = ra["flux"].astype(np.float64), rb["flux"].astype(np.float64)
            m = 0.5 * (fa + fb)
            sel = m > 0.01 * m.max()
            rse[arm].append(np.abs(fa - fb)[sel] / np.sqrt(2.0) / m[sel])
    err = {}
    for arm, lst in rse.items():
        v = np.concatenate(lst)
        # |a - b| / sqrt 2 is |N(0, sigma^2)|, whose median is 0.6745 sigma
        err[arm] = {"rse": float(np.median(v) / 0.6745), "voxels": int(v.size),
                    "estimator": "median over voxels >= 1% of peak of |a-b|/sqrt(2)/mean, / 0.6745"}
    return {"simulations": nsim, "photons": photons, "batched_sims_per_s": nsim / tb,
            "one_launch_per_sim_sims_per_s": nsim / ts, "ratio": ts / tb,
            "batched_wall_s": tb, "batched_kernel_ms": kb, "one_launch_per_sim_wall_s": ts,
            "one_launch_per_sim_kernel_ms": ks,
            "equal_error": "same photons per simulation in both arms; measured RSE below",
            "rse": err, "precision_vs_fp64": prec}


def gradient_measure():
    """The differentiation workload (100^3 float-mua field, 16 detectors, 1e7
    photons): forward readings, backward replay for d loss / d mua, and
    central differences (relative step 1e-3, common random numbers) on 8
    voxels drawn among those the detected photons visit."""
    from mcxcl_gb300 import diff, workloads
    cfg, mua, target = workloads.diff_config()
    sim = diff.ReplayGradient(cfg)
    Rt = sim.forward(target)

    def loss(R):
        return float(np.sum((np.log(R) - np.log(Rt)) ** 2))
    tf, tb = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        R = sim.forward(mua)
        tf.append(time.perf_counter() - t0)
        g = 2 * (np.log(R) - np.log(Rt)) / R
        t0 = time.perf_counter()
        gm = sim.backward(g)
        tb.append(time.perf_counter() - t0)
    rng = np.random.default_rng(64)
    support = np.flatnonzero(np.abs(gm).ravel() > 1e-3 * np.abs(gm).max())
    bw, fd = [], []
    for f in rng.choice(support, size=8, replace=False):
        v = np.unravel_index(f, mua.shape)
        h = np.float32(1e-3) * mua[v]
        mp, mm = mua.copy(), mua.copy()
        mp[v] += h
        mm[v] -= h
        fd.append((loss(sim.forward(mp)) - loss(sim.forward(mm))) / float(mp[v] - mm[v]))
        bw.append(gm[v])
    bw, fd = np.array(bw), np.array(fd)
    return {"forward_ms": 1e3 * min(tf), "backward_ms": 1e3 * min(tb), "backward_over_forward": min(tb) / min(tf),
            "detected_replayed": int(len(sim.last["w"])),
            "fd_rel_err_8_voxels": float(np.linalg.norm(bw - fd) / np.linalg.norm(fd))}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    cfg = workload(args.photons)
    res = None
    vals = []
    for i in range(args.warmup + args.steps):
        res = cpu_baseline(cfg, target_s=5.0, kind="port")
        if i >= args.warmup:
            vals.append(res["value"])
    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": "photons/ms", "value": v, "unit": "photons/ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(cfg["nphoton"]) / v,
        "ms_per_step_note": "a full step's photons at the sampled rate (each step times a bounded sample)",
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "photons_per_step": int(cfg["nphoton"])},
        "cpu_baseline": dict(res, value=v),
        "e2e": {"value": v, "unit": "photons/ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own CPU path is its OpenCL kernel, which needs an OpenCL CPU driver absent "
                "from this box; the C restatement of that kernel (oracle/) is timed instead, on a bounded "
                "sample of each step's photons (photons/ms is per-photon work, so the sample keeps the unit)",
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- helpers

def prepare(cfg):
    """Validated Config and a device-resident session of one workload."""
    import ctypes
    from mcxcl_gb300 import _lib, pmcxcl
    L = _lib.load()
    C = _lib.Config()
    pmcxcl.parse_config(cfg, C)
    L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    pmcxcl._check(C)
    sess = L.mcx_prepare_simulation(ctypes.byref(C))
    pmcxcl._check(C)
    return C, sess


def simulate(sess, flags=0):
    import ctypes
    from mcxcl_gb300 import _lib
    L = _lib.load()
    ms = ctypes.c_float()
    rc = L.mcxg_simulate(sess, flags, ctypes.byref(ms))
    if rc:
        raise RuntimeError(L.mcxg_error_string(rc).decode())
    return ms.value


def launch_shape(sess):
    import ctypes
    from mcxcl_gb300 import _lib
    g, b, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _lib.load().mcxg_get_launch(sess, ctypes.byref(g), ctypes.byref(b), ctypes.byref(r))
    return {"grid": g.value, "block": b.value, "regs": r.value}


def event_model(cfg, sample):
    """FP32 and MUFU operations per photon from the frozen model and the
    exact kernel's event counts on a sample of the workload."""
    import mcxcl_gb300
    rx = mcxcl_gb300.run(dict(cfg, nphoton=int(sample), exactmath=1))
    ev = rx["stat"]["eventcount"]
    per = {k: ev[k] / float(sample) for k in ("step", "scatter", "launch", "reflect")}
    ops = (OPS_PER_STEP * per["step"] + OPS_PER_SCATTER * per["scatter"] + OPS_PER_LAUNCH * per["launch"] +
           OPS_PER_REFLECT * per["reflect"])
    mufu = MUFU_PER_STEP * per["step"] + MUFU_PER_SCATTER * per["scatter"]
    return per, ops, mufu


def read_traffic(k):
    path = TRAFFIC_FILE % k
    if os.path.exists(path):
        for ln in open(path):
            if ln.startswith("dram_bytes_per_launch:"):
                return float(ln.split(":")[1])
    return None


def hbm_peak():
    """The measured copy bandwidth of the GB300s (GB/s) and its source."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback (6.8 TB/s, one earlier GB300 measurement)"


def roofline(per, ops, kms, nphoton, peak, k, sample):
    achieved = ops * nphoton / (kms * 1e-3) / 1e9
    traffic = read_traffic(k)
    hbm, hbm_src = hbm_peak()
    dram = traffic / (kms * 1e-3) / 1e9 if traffic else None
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "Gop/s",
            "frac": achieved / peak if peak else None, "traffic": traffic,
            "dram": {"achieved": dram, "peak": hbm, "unit": "GB/s", "frac": dram / hbm if dram else None,
                     "peak_source": hbm_src,
                     "note": "DRAM bytes of one full launch (traffic) over this run's kernel time: not the bound"},
            "traffic_from": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one full launch, "
                            "profiles/traffic_mcx_transport_config%d.txt" % k,
            "peak_source": "measured in this run: 8-chain FMA kernel, one FMA = one op",
            "ops_per_photon": ops, "events_per_photon": per,
            "model": "48*step + 65*scatter + 20*launch + 10*Fresnel FP32 ops",
            "events_from": "exact kernel (bit-identical to the oracle), %d-photon sample" % sample}


def timed_launches(sess, steps, warmup, flush, flags=0):
    """Kernel ms of `steps` launches after `warmup`, L2 flushed before each."""
    import torch
    for _ in range(max(3, warmup)):
        simulate(sess, flags)
    torch.cuda.synchronize()
    kms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        kms.append(simulate(sess, flags))
    torch.cuda.synchronize()
    return kms


def e2e_bytes(cfg, out):
    """Host-device bytes of one run() call: the packed labels, property rows,
    detector positions and the 31-word seed window in; the field, detected
    records, seeds, energy sums and counters out."""
    nvox = int(np.asarray(cfg["vol"]).size)
    nprop = len(cfg["prop"])
    ndetpos = len(cfg.get("detpos", []))
    gates = out["flux"].shape[3]
    ndet = out["detp"].shape[1] if "detp" in out else 0
    reclen = out["detp"].shape[0] if "detp" in out else 0
    nseed = out["seeds"].shape[1] if out.get("seeds") is not None else 0
    h2d = nvox * 1 + 16 * nprop + 16 * ndetpos + 4 * 31
    d2h = nvox * gates * 4 + ndet * reclen * 4 + nseed * 16 + 16 + 8 * 4 + 8 * 8
    return h2d, d2h


def config_measure(k, photons, steps, warmup, flush, peak):
    """photons/ms, roofline and traffic of workload k (1 cube, 3 head) on
    resident data, and end to end through mcxcl_gb300.run with host buffers."""
    import mcxcl_gb300
    from mcxcl_gb300 import _lib, workloads
    import ctypes
    cfg = workloads.config(k)
    cfg["nphoton"] = int(photons)
    C, sess = prepare(cfg)
    try:
        kms = timed_launches(sess, steps, warmup, flush)
        shape = launch_shape(sess)
    finally:
        _lib.load().mcx_clearcfg(ctypes.byref(C))
    ms = float(np.mean(kms))
    sample = 2000000 if k == 3 else 5000000
    per, ops, _ = event_model(cfg, sample)
    # warm the path: a loop that keeps each result while the next call runs
    # reaches its steady state (output buffers reused) on its third call
    for _ in range(2):
        last = mcxcl_gb300.run(dict(cfg))
    n_e2e = 2
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        last = mcxcl_gb300.run(dict(cfg))
    e2e_ms = (time.perf_counter() - t0) * 1e3 / n_e2e
    h2d, d2h = e2e_bytes(cfg, last)
    return {"workload": workloads.describe(k), "photons_per_step": int(photons), "steps": steps,
            "value": photons / ms, "unit": "photons/ms", "ms_per_step": ms, "launch": shape,
            "e2e": {"value": photons / e2e_ms, "unit": "photons/ms", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": n_e2e},
            "roofline": roofline(per, ops, ms, photons, peak, k, sample)}


def precision_measure(photons):
    """Error of the compensated field (the product: int64 fixed-point counts
    and a float remainder, merged in FP64), of a plain float field and of
    the reference's +-1000 spill field against an FP64 accumulation of the
    same deposits (one run, every deposit to all four), on the cube and the
    cube + sphere workloads; relative error over every non-zero element."""
    import ctypes
    from mcxcl_gb300 import _lib, workloads
    L = _lib.load()
    out = {}
    for k in (1, 2):
        cfg = workloads.config(k)
        cfg["nphoton"] = int(photons)
        C, sess = prepare(cfg)
        try:
            simulate(sess, 128)                                   # MCXG_VERIFY
            n = int(C.maxgate) * C.dim.x * C.dim.y * C.dim.z
            two = np.zeros(n, np.float64)
            f64 = np.zeros(n, np.float64)
            plain = np.zeros(n, np.float32)
            spill = np.zeros(n, np.float32)
            L.mcxg_get_field_f64(sess, two.ctypes.data)
            L.mcxg_get_verify(sess, f64.ctypes.data, plain.ctypes.data, spill.ctypes.data)
        finally:
            L.mcx_clearcfg(ctypes.byref(C))
        nz = f64 > 0
        res = {}
        for name, x in (("compensated", two), ("compensated_float_output", two.astype(np.float32).astype(np.float64)),
                        ("plain_float", plain.astype(np.float64)), ("reference_spill", spill.astype(np.float64))):
            r = np.abs(x[nz] - f64[nz]) / f64[nz]
            tot = abs(x.sum() - f64.sum()) / f64.sum()
            res[name] = {"max": float(r.max()), "median": float(np.median(r)), "p99": float(np.quantile(r, 0.99)),
                         "total": float(tot)}
        out["config%d" % k] = dict(res, photons=int(photons), elements=int(nz.sum()))
    return out


def profile_mode(args):
    """N launches of workload K on resident data, for a profiler to capture."""
    import ctypes
    from mcxcl_gb300 import _lib, workloads
    L = _lib.load()
    cfg = workloads.config(args.config)
    if args.photons:
        cfg["nphoton"] = int(args.photons)
    C, sess = prepare(cfg)
    if args.block or args.blocks_per_sm:
        L.mcxg_set_launch(sess, args.block, args.blocks_per_sm)
    if args.tile >= 0:
        L.mcxg_set_tile(sess, args.tile)
    box = np.zeros(8, np.uint32)
    for i in range(args.launches):
        ms = simulate(sess, args.flags)
        L.mcxg_get_tile(sess, box.ctypes.data)
        print("launch %d: %.3f ms, %.1f photons/ms, tile %s" % (i, ms, cfg["nphoton"] / ms, box.tolist()), flush=True)
    L.mcx_clearcfg(ctypes.byref(C))


def main():
    args = parse_args()
    rank, world, local = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return
    import ctypes
    import torch
    import mcxcl_gb300
    from mcxcl_gb300 import _lib

    torch.cuda.set_device(local)
    L = _lib.load()
    if args.launches:
        profile_mode(args)
        return
    cfg = workload(args.photons)
    cfg["gpuid"] = local + 1
    cfg["seed"] = int(cfg["seed"]) + rank
    nphoton = int(cfg["nphoton"])

    # ---- device-resident session
    C, sess = prepare(cfg)
    nthread = C.threadused

    # launch shape: the autotuner times the candidates on 2e6 photons of this workload
    tb, tp, tn = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = L.mcxg_autotune(sess, 2000000, ctypes.byref(tb), ctypes.byref(tp), ctypes.byref(tn))
    if rc:
        raise RuntimeError(L.mcxg_error_string(rc).decode())
    tuned = {"block": tb.value, "blocks_per_sm": tp.value, "warp_aggregation": not tn.value}

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    for _ in range(max(3, args.warmup)):
        simulate(sess)
    barrier(world)
    torch.cuda.synchronize()
    kms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            kms.append(simulate(sess))
        torch.cuda.synchronize()
    barrier(world)
    tot_ms = sum(kms)
    ms_per_step = allmax(tot_ms / args.steps, world)
    photons_all = allsum(nphoton * args.steps, world)
    value = photons_all / (ms_per_step * args.steps)
    shape = launch_shape(sess)

    # ---- event counts from the exact kernel on a sample, and the FP32 peak
    sample = min(nphoton, 5000000)
    per_photon, ops_per_photon, mufu_per_photon = event_model(cfg, sample)
    peak = ctypes.c_double()
    L.mcxg_fp32_peak(sess, ctypes.byref(peak))
    ms_avg = tot_ms / args.steps
    info = mcxcl_gb300.gpuinfo()[local]
    clock_summary = clk.summary()
    sm_mhz = clock_summary["sm_mhz"] or clock_summary["sm_max_mhz"] or 2070.0
    mufu_achieved = mufu_per_photon * nphoton / (ms_avg * 1e-3) / 1e9
    mufu_peak = info["sm"] * MUFU_PER_SM_CLK * sm_mhz * 1e6 / 1e9
    roof = roofline(per_photon, ops_per_photon, ms_avg, nphoton, peak.value, 2, sample)
    roof["fp32_nominal"] = info["sm"] * 128 * sm_mhz * 1e6 / 1e9
    roof["mufu"] = {"achieved": mufu_achieved, "peak": mufu_peak, "unit": "Gop/s", "frac": mufu_achieved / mufu_peak,
                    "model": "6*step + 11*scatter MUFU ops; peak 16/SM/clock at the sampled clock"}

    # ---- end to end through the public API, host buffers in and out
    e2e_steps = args.e2e_steps or max(2, min(args.steps, 3))
    # warm the path (session cache, page-ins): a loop that keeps each result
    # while the next call runs reaches its steady state (output buffers
    # reused) on its third call
    last = None
    for _ in range(2):
        last = mcxcl_gb300.run(dict(cfg))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        last = mcxcl_gb300.run(dict(cfg))
    torch.cuda.synchronize()
    e2e_wall = allmax(time.perf_counter() - t0, world)
    e2e_value = allsum(nphoton * e2e_steps, world) / (e2e_wall * 1e3)
    h2d, d2h = e2e_bytes(cfg, last)

    out = None
    if rank == 0:
        configs = None
        if not args.no_configs:
            configs = {"c1": config_measure(1, 1e8, 3, 2, flush, peak.value),
                       "c3": config_measure(3, 1e8, 3, 1, flush, peak.value)}
        precision = precision_measure(args.precision) if args.precision else None
        batched = batch_measure(args.batch_sims) if args.batch_sims > 0 else None
        gradient = None if args.no_gradient else gradient_measure()
        cpu = None if args.no_cpu_baseline else cpu_baseline(cfg)
        absorbed = last["stat"]["energyabs"] / last["stat"]["energytot"]
        out = {
            "metric": "photons/ms", "value": value, "unit": "photons/ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "photons_per_step": nphoton, "reference_threads": nthread,
                       "launch": dict(shape, autotuned=tuned),
                       "l2": "flushed between timed steps (256 MB write); working set < L2",
                       "parallelism": "replicas" if world > 1 else "1 GPU"},
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": "photons/ms", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "cpu_baseline": cpu,
            "clocks": clock_summary,
            "gpu_launches": args.steps,
            "absorbed": absorbed,
            "detected_per_step": int(last["stat"]["detected"]),
        }
        if configs:
            out.update(configs)
        if precision:
            out["precision"] = precision
        out["batched"] = batched
        out["gradient"] = gradient
        print(json.dumps(out))
    L.mcx_clearcfg(ctypes.byref(C))


if __name__ == "__main__":
    main()
