"""Build recipe for libmcxgb300.so (the CUDA kernels, the device layer and the C host driver).

Compiles in parallel, one -gencode (sm_103a), into mcxcl_gb300/_build/.  Run
``python -m mcxcl_gb300.build`` or call :func:`build`.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmcxgb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + INCLUDE] + ARCH
# per-unit floating-point flags: the production kernel uses the MUFU
# approximations; the verification kernel must evaluate IEEE basic operations
# exactly as written so it reproduces the CPU oracle bit for bit.  The
# production units also ask ptxas for register-frugal code (level 2 of 10):
# the transport kernel then fits 64 registers without spills, so 32 warps a
# SM are resident instead of 24 (cube 8 %, cube + sphere 7 %, head 8 %, the
# 512-simulation batch 8 % faster)
UNITS = {
    "mcx_kernel_fast.cu": ["--use_fast_math", "-Xptxas", "--register-usage-level=2"],
    "mcx_kernel_batch.cu": ["--use_fast_math", "-Xptxas", "--register-usage-level=2"],
    "mcx_kernel_exact.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
    "mcx_device.cu": [],
}
HEADERS = ["mcx_kernel.cuh", "mcx_pmath.cuh", "mcx_kparams.h", "mcx_launch.h"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; set NVCC or put the CUDA toolkit on PATH")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile every translation unit that changed and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdeps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mcx_gb300.h")]
    jobs = []
    objs = []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdeps):
            jobs.append([nvcc] + NVCC_COMMON + flags + ["-c", src, "-o", obj])
    for cunit in ("mcx_host.c", "mcx_mie.c", "mcx_json.c"):
        csrc = os.path.join(CSRC, cunit)
        cobj = os.path.join(BUILD, cunit.replace(".c", ".o"))
        objs.append(cobj)
        if force or _stale(cobj, [csrc, os.path.join(CSRC, "mcx_json.h")] + hdeps):
            jobs.append([os.environ.get("CC", "gcc"), "-std=gnu11", "-O2", "-fPIC", "-Wall", "-I" + CSRC,
                         "-I" + INCLUDE, "-c", csrc, "-o", cobj])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("build failed:\n" + msg)
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, "-shared"] + ARCH + ["-o", LIB] + objs + ["-lm"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
