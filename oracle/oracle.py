"""Python driver for the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` import this module.  It loads ``oracle/_build/libmcxoracle.so``
(the plain-C restatement, ``mcx_oracle.c``) and, when it was built here from
the reference sources, ``oracle/_ref/libmcxref.so`` (the reference kernel
itself compiled on the host).

``cfg`` dictionaries use the ``pmcxcl.run()`` keys of the reference Python
module (src/pmcxcl.cpp:428-1110); unspecified keys take the defaults of
``mcx_initcfg`` (src/mcx_utils.c:203-366).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmcxoracle.so")
REF_PATH = os.environ.get("MCXO_REF_PATH", os.path.join(HERE, "_ref", "libmcxref.so"))

MATH_LIBM, MATH_PMATH = 0, 1
VARIANT_OPENCL, VARIANT_NVCC = 0, 1
FIELD_FLOAT_SPILL, FIELD_DOUBLE = 0, 1

SRCTYPES = ["pencil", "isotropic", "cone", "gaussian", "planar", "pattern", "fourier", "arcsine", "disk",
            "fourierx", "fourierx2d", "zgaussian", "line", "slit", "pencilarray", "pattern3d", "hyperboloid",
            "ring"]
# pmcxcl's outputtype names (src/pmcxcl.cpp:854-872): from "wl" on the index drops by two
_OT_NAMES = ["flux", "fluence", "energy", "jacobian", "nscat", "wl", "wp", "wm", "rf", "length", "rfmus", "wltof",
             "wptof"]
OUTPUTTYPES = {n: (i - 2 if i >= 5 else i) for i, n in enumerate(_OT_NAMES)}
SEED_FROM_FILE = -999
SAVEFLAGS = "DSPMXVWI"


class MCXOInput(ctypes.Structure):
    _fields_ = [
        ("dimx", ctypes.c_uint), ("dimy", ctypes.c_uint), ("dimz", ctypes.c_uint),
        ("vol", ctypes.c_void_p), ("mediabyte", ctypes.c_int), ("prop", ctypes.c_void_p),
        ("medianum", ctypes.c_uint), ("unitinmm", ctypes.c_float),
        ("srctype", ctypes.c_int), ("srcpos", ctypes.c_float * 4), ("srcdir", ctypes.c_float * 4),
        ("srcparam1", ctypes.c_float * 4), ("srcparam2", ctypes.c_float * 4),
        ("srcpattern", ctypes.c_void_p), ("srcnum", ctypes.c_uint), ("extrasrclen", ctypes.c_uint),
        ("srcdata", ctypes.c_void_p), ("srcid", ctypes.c_int),
        ("detpos", ctypes.c_void_p), ("detnum", ctypes.c_uint), ("maxdetphoton", ctypes.c_uint),
        ("issavedet", ctypes.c_int), ("savedetflag", ctypes.c_uint), ("issaveseed", ctypes.c_int),
        ("issaveref", ctypes.c_int), ("issaveexit", ctypes.c_int), ("ismomentum", ctypes.c_int),
        ("tstart", ctypes.c_float), ("tstep", ctypes.c_float), ("tend", ctypes.c_float),
        ("isreflect", ctypes.c_int), ("bc", ctypes.c_char * 12), ("minenergy", ctypes.c_float),
        ("gscatter", ctypes.c_uint), ("voidtime", ctypes.c_int), ("isspecular", ctypes.c_int),
        ("maxvoidstep", ctypes.c_int), ("outputtype", ctypes.c_int), ("isnormalized", ctypes.c_int),
        ("issrcfrom0", ctypes.c_int), ("invcdf", ctypes.c_void_p), ("nphase", ctypes.c_uint),
        ("angleinvcdf", ctypes.c_void_p), ("nangle", ctypes.c_uint),
        ("nphoton", ctypes.c_double), ("nthread", ctypes.c_uint), ("core", ctypes.c_uint),
        ("seed", ctypes.c_int), ("debugrng", ctypes.c_int),
        ("mathmode", ctypes.c_int), ("variant", ctypes.c_int), ("fieldmode", ctypes.c_int),
        ("nworkers", ctypes.c_int),
        ("replayseed", ctypes.c_void_p), ("replayweight", ctypes.c_void_p), ("replaytof", ctypes.c_void_p),
        ("replaydetid", ctypes.c_void_p), ("nreplay", ctypes.c_uint), ("replaydet", ctypes.c_int),
        ("replaysiteown", ctypes.c_int), ("detweight_out", ctypes.c_void_p), ("omega", ctypes.c_float),
        ("smatrix", ctypes.c_void_p), ("polmedianum", ctypes.c_uint), ("s0", ctypes.c_float * 4),
        ("seedskip", ctypes.c_uint),
        ("debugmove", ctypes.c_int), ("maxtraj", ctypes.c_uint), ("traj_out", ctypes.c_void_p),
        ("ntraj_out", ctypes.c_void_p),
    ]


class MCXOStats(ctypes.Structure):
    _fields_ = [
        ("energytot", ctypes.c_double), ("energyesc", ctypes.c_double), ("energyabs", ctypes.c_double),
        ("normalizer", ctypes.c_double), ("detected", ctypes.c_uint), ("saved", ctypes.c_uint),
        ("threadphoton", ctypes.c_uint), ("oddphoton", ctypes.c_int), ("reclen", ctypes.c_uint),
        ("fieldlen", ctypes.c_uint), ("maxgate", ctypes.c_uint),
        ("nstep", ctypes.c_uint64), ("nscatter", ctypes.c_uint64), ("nlaunch", ctypes.c_uint64),
        ("nreflect", ctypes.c_uint64), ("nfailed", ctypes.c_uint64),
    ]


_lib = None
_ref = {}


def build(ref=None):
    """Compile the oracle (and, when the reference sources exist, the reference harness)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    refdir = ref or os.environ.get("MCX_REFERENCE", "")
    if refdir and os.path.isfile(os.path.join(refdir, "src", "mcx_core.cl")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + refdir], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.mcxo_run.restype = ctypes.c_int
        _lib.mcxo_reclen.restype = ctypes.c_uint
        _lib.mcxo_fieldlen.restype = ctypes.c_uint
        _lib.mcxo_fieldcomp.restype = ctypes.c_uint
        _lib.mcxo_pm_logf.restype = ctypes.c_float
        _lib.mcxo_pm_logf.argtypes = [ctypes.c_float]
        _lib.mcxo_pm_expf.restype = ctypes.c_float
        _lib.mcxo_pm_expf.argtypes = [ctypes.c_float]
        _lib.mcxo_pm_acosf.restype = ctypes.c_float
        _lib.mcxo_pm_acosf.argtypes = [ctypes.c_float]
        _lib.mcxo_replayinit.restype = ctypes.c_int
    return _lib


def ref_available():
    return os.path.exists(REF_PATH)


def reflib(pattern=False):
    """The reference harness; pattern=True: the build for pattern sources
    (photon-sharing deposits), as the reference compiles its kernel for them."""
    path = REF_PATH.replace("libmcxref.so", "libmcxref_pat.so") if pattern else REF_PATH
    if path not in _ref:
        _ref[path] = ctypes.CDLL(path)
        _ref[path].mcxref_run.restype = ctypes.c_int
    return _ref[path]


def ref_mie(x, m):
    """The reference's Mie routine (src/mcx_mie.cpp:91) from the harness:
    (181 x 4 Mueller rows, qsca, g)."""
    R = reflib()
    sm = np.zeros((181, 4), np.float32)
    q, g = ctypes.c_double(), ctypes.c_double()
    R.mcxref_mie(ctypes.c_double(x), ctypes.c_double(m), sm.ctypes.data_as(ctypes.c_void_p), ctypes.byref(q),
                 ctypes.byref(g))
    return sm, q.value, g.value


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _rows(v, ncol=4):
    a = np.asarray(v, dtype=np.float32)
    if a.ndim == 1:
        a = a.reshape(1, -1)
    out = np.zeros((a.shape[0], ncol), dtype=np.float32)
    out[:, :a.shape[1]] = a
    return out


def _flags(s, letters):
    if isinstance(s, (int, np.integer)):
        return int(s)
    v = 0
    for ch in str(s).upper():
        if ch in letters:
            v |= 1 << letters.index(ch)
    return v


def make_input(cfg, nthread=4096, core=None, mathmode=MATH_LIBM, variant=VARIANT_OPENCL,
               fieldmode=FIELD_DOUBLE, nworkers=0, seedskip=0):
    """Translate a pmcxcl-style dict into the oracle's input struct.

    Returns (struct, keepalive) -- keepalive holds the numpy buffers."""
    keep = {}
    inp = MCXOInput()
    # the pmcxcl volume encoding (src/pmcxcl.cpp:93-426): the oracle decodes the
    # same words the kernel gets, converted by numpy alone (no product code)
    import sys
    if os.path.dirname(HERE) not in sys.path:
        sys.path.insert(0, os.path.dirname(HERE))
    from mcxcl_gb300 import media
    words, inp.mediabyte, dims = media.encode(cfg["vol"], float(cfg.get("unitinmm", 1.0)), native=False)
    words = np.ascontiguousarray(words)
    keep["vol"] = words
    inp.dimx, inp.dimy, inp.dimz = [int(d) for d in dims]
    inp.vol = _ptr(words)
    prop = np.ascontiguousarray(_rows(cfg["prop"]))
    keep["prop"] = prop
    inp.prop = _ptr(prop)
    inp.medianum = prop.shape[0]
    inp.unitinmm = float(cfg.get("unitinmm", 1.0))

    st = cfg.get("srctype", "pencil")
    inp.srctype = SRCTYPES.index(st) if isinstance(st, str) else int(st)
    srcpos = _rows(cfg.get("srcpos", [0, 0, 0]))
    if srcpos.shape[0] == 1 and np.asarray(cfg.get("srcpos", [0, 0, 0])).size == 3:
        srcpos[0, 3] = 1.0
    srcdir = _rows(cfg.get("srcdir", [0, 0, 1]))
    p1 = _rows(cfg.get("srcparam1", [0, 0, 0, 0]))
    p2 = _rows(cfg.get("srcparam2", [0, 0, 0, 0]))
    n_src = max(srcpos.shape[0], srcdir.shape[0], p1.shape[0], p2.shape[0])

    def row(a, i):
        return a[i] if i < a.shape[0] else np.zeros(4, np.float32)
    for k, a in (("srcpos", srcpos), ("srcdir", srcdir), ("srcparam1", p1), ("srcparam2", p2)):
        getattr(inp, k)[:] = [float(x) for x in a[0]]
    inp.extrasrclen = n_src - 1
    if n_src > 1:
        sd = np.zeros((n_src - 1, 16), np.float32)
        for i in range(1, n_src):
            if srcpos.shape[0] > i and np.asarray(cfg["srcpos"]).shape[1] == 3:
                srcpos[i, 3] = 1.0
            sd[i - 1] = np.concatenate([row(srcpos, i), row(srcdir, i), row(p1, i), row(p2, i)])
        keep["srcdata"] = sd
        inp.srcdata = _ptr(sd)
    inp.srcid = int(cfg.get("srcid", 0))
    if "srcpattern" in cfg:
        pat = np.ascontiguousarray(np.asarray(cfg["srcpattern"], np.float32).reshape(-1, order="F"))
        keep["srcpattern"] = pat
        inp.srcpattern = _ptr(pat)
    inp.srcnum = int(cfg.get("srcnum", 1))
    inp.omega = float(cfg.get("omega", 0.0))
    if cfg.get("smatrix") is not None:
        # polarised transport: the Mueller rows of labels 1..N (N x 181 x 4) and the
        # Mie-derived properties already in cfg["prop"]
        sm = np.ascontiguousarray(np.asarray(cfg["smatrix"], np.float32).reshape(-1, 181, 4))
        keep["smatrix"] = sm
        inp.smatrix = _ptr(sm)
        inp.polmedianum = sm.shape[0]
    s0 = np.asarray(cfg.get("srciquv", [1, 0, 0, 0]), np.float32).ravel()
    for i in range(4):
        inp.s0[i] = float(s0[i])

    if "detpos" in cfg and np.asarray(cfg["detpos"]).size:
        det = np.ascontiguousarray(_rows(cfg["detpos"]))
        keep["det"] = det
        inp.detpos = _ptr(det)
        inp.detnum = det.shape[0]
    inp.maxdetphoton = int(cfg.get("maxdetphoton", 1000000))
    inp.issavedet = int(cfg.get("issavedet", 1))
    inp.savedetflag = _flags(cfg.get("savedetflag", 0x5), SAVEFLAGS)
    inp.issaveseed = int(bool(cfg.get("issaveseed", 0)))
    inp.issaveref = int(cfg.get("issaveref", 0))
    inp.issaveexit = int(bool(cfg.get("issaveexit", 0)))
    inp.ismomentum = int(bool(cfg.get("ismomentum", 0)))
    inp.tstart = float(cfg.get("tstart", 0.0))
    inp.tend = float(cfg.get("tend", 5e-9))
    inp.tstep = float(cfg.get("tstep", 5e-9))
    inp.isreflect = int(cfg.get("isreflect", 1))
    bc = str(cfg.get("bc", "")).encode()[:12]
    inp.bc = bc + b"\0" * (12 - len(bc))
    inp.minenergy = float(cfg.get("minenergy", 0.0))
    inp.gscatter = int(cfg.get("gscatter", 1000000000))
    inp.voidtime = int(cfg.get("voidtime", 1))
    inp.isspecular = int(bool(cfg.get("isspecular", 0)))
    inp.maxvoidstep = int(cfg.get("maxvoidstep", 1000))
    ot = cfg.get("outputtype", "flux")
    inp.outputtype = OUTPUTTYPES[ot] if isinstance(ot, str) else int(ot)
    inp.isnormalized = int(cfg.get("isnormalized", 1))
    inp.issrcfrom0 = int(cfg.get("issrcfrom0", 0))
    if "invcdf" in cfg:
        cdf = np.ascontiguousarray(np.asarray(cfg["invcdf"], np.float32).ravel())
        keep["invcdf"] = cdf
        inp.invcdf = _ptr(cdf)
        inp.nphase = cdf.size
    if "angleinvcdf" in cfg:
        acdf = np.ascontiguousarray(np.asarray(cfg["angleinvcdf"], np.float32).ravel())
        keep["angleinvcdf"] = acdf
        inp.angleinvcdf = _ptr(acdf)
        inp.nangle = acdf.size
    inp.nphoton = float(cfg.get("nphoton", 0))
    inp.nthread = int(nthread)
    inp.core = int(core if core is not None else nthread)
    inp.debugrng = int("R" in str(cfg.get("debuglevel", "")).upper())
    inp.debugmove = int(any(k in str(cfg.get("debuglevel", "")).upper() for k in "MT"))
    if inp.debugmove:
        inp.maxtraj = int(cfg.get("maxjumpdebug", 10000000))
        keep["traj"] = np.zeros(max(1, inp.maxtraj) * 6, np.float32)
        keep["ntraj"] = np.zeros(1, np.uint32)
        inp.traj_out = _ptr(keep["traj"])
        inp.ntraj_out = _ptr(keep["ntraj"])
    inp.mathmode = mathmode
    inp.variant = variant
    inp.fieldmode = fieldmode
    inp.nworkers = nworkers
    seed = cfg.get("seed", 0x623F9A9E)
    if isinstance(seed, np.ndarray) and seed.ndim == 2:
        _replay_input(inp, keep, cfg, seed)
    else:
        inp.seed = int(seed)
    inp.seedskip = int(seedskip)
    return inp, keep


def _replay_input(inp, keep, cfg, seed):
    """Replay: cfg['seed'] is the uint8 [16, N] seed array and
    cfg['detphotons'] the float32 [reclen, N] records of a previous run
    (src/pmcxcl.cpp:1006-1047); mcxo_replayinit picks and weights them."""
    s8 = np.asarray(seed, np.uint8)
    if s8.shape[0] != 16:
        raise ValueError("the row number of cfg.seed does not match RNG seed byte-length")
    n = s8.shape[1]
    seeds = np.ascontiguousarray(s8.T).view(np.uint64).reshape(n, 2).copy()
    inp.seed = SEED_FROM_FILE
    inp.replaydet = int(cfg.get("replaydet", 0))
    inp.replaysiteown = int(cfg.get("replaysiteown", 0))
    if "detphotons" not in cfg:
        # per-photon weight, time of flight and detector id given directly
        w = np.ascontiguousarray(np.asarray(cfg["replayweight"], np.float32).ravel())
        tof = np.ascontiguousarray(np.asarray(cfg["replaytof"], np.float32).ravel())
        did = np.ascontiguousarray(np.asarray(cfg["replaydetid"], np.int32).ravel())
        for name, a in (("rseed", seeds), ("rw", w), ("rtof", tof), ("rdid", did)):
            keep[name] = a
        inp.replayseed, inp.replayweight = _ptr(seeds), _ptr(w)
        inp.replaytof, inp.replaydetid = _ptr(tof), _ptr(did)
        inp.nreplay = n
        inp.nphoton = float(n)
        return
    detp = np.asarray(cfg["detphotons"], np.float32)
    if detp.ndim != 2 or detp.shape[1] != n:
        raise ValueError("the column numbers of detphotons and seed do not match")
    recs = np.ascontiguousarray(detp.T)
    out_seed = np.zeros((max(n, 1), 2), np.uint64)
    w = np.zeros(max(n, 1), np.float32)
    tof = np.zeros(max(n, 1), np.float32)
    did = np.zeros(max(n, 1), np.int32)
    k = lib().mcxo_replayinit(ctypes.byref(inp), _ptr(recs), ctypes.c_uint(recs.shape[1]), ctypes.c_uint(n),
                              _ptr(seeds), _ptr(out_seed), _ptr(w), _ptr(tof), _ptr(did))
    if k < 0:
        raise ValueError("replay initialisation failed with code %d" % k)
    for name, a in (("rseed", out_seed), ("rw", w), ("rtof", tof), ("rdid", did)):
        keep[name] = a
    inp.replayseed, inp.replayweight = _ptr(out_seed), _ptr(w)
    inp.replaytof, inp.replaydetid = _ptr(tof), _ptr(did)
    inp.nreplay = k
    inp.nphoton = float(k)


def run(cfg, nthread=4096, core=None, mathmode=MATH_LIBM, variant=VARIANT_OPENCL, fieldmode=FIELD_DOUBLE,
        nworkers=0, seedskip=0):
    """Run the oracle.  Returns a dict with the merged raw field (float64,
    Fortran-ordered [x, y, z, gate]), the normalised field, per-thread energies,
    detected-photon records, seeds, stats and event counters."""
    inp, keep = make_input(cfg, nthread, core, mathmode, variant, fieldmode, nworkers, seedskip)
    L = lib()
    fieldlen = L.mcxo_fieldlen(ctypes.byref(inp)) * L.mcxo_fieldcomp(ctypes.byref(inp))
    reclen = L.mcxo_reclen(ctypes.byref(inp))
    field = np.zeros(fieldlen, np.float64)
    fnorm = np.zeros(fieldlen, np.float32)
    energy = np.zeros(2 * inp.nthread, np.float32)
    maxdet = inp.maxdetphoton
    detp = np.zeros(max(1, maxdet * max(reclen, 1)), np.float32)
    seeds = np.zeros(max(2, maxdet * 2), np.uint64)
    masked = np.zeros(inp.dimx * inp.dimy * inp.dimz, np.uint32)
    detw = np.zeros(max(2, maxdet * 2), np.float32)
    inp.detweight_out = _ptr(detw)
    st = MCXOStats()
    rc = L.mcxo_run(ctypes.byref(inp), _ptr(field), _ptr(fnorm), _ptr(energy), _ptr(detp), _ptr(seeds),
                    _ptr(masked), ctypes.byref(st))
    if rc:
        raise RuntimeError("oracle failed with code %d" % rc)
    gates = st.maxgate
    shape = (inp.dimx, inp.dimy, inp.dimz, -1)
    nsaved = st.saved
    out = {
        "field_raw": field.reshape(shape, order="F"),
        "flux": fnorm.reshape(shape, order="F"),
        "energy": energy.reshape(-1, 2),
        "detp": detp[:nsaved * reclen].reshape(nsaved, reclen).T if reclen else np.zeros((0, 0), np.float32),
        "seeds": seeds[:2 * nsaved].reshape(nsaved, 2) if inp.issaveseed else None,
        "detweight": detw[:2 * nsaved].reshape(nsaved, 2).T.copy(),
        "masked": masked.reshape(inp.dimx, inp.dimy, inp.dimz, order="F"),
        "stat": {k: getattr(st, k) for k, _ in MCXOStats._fields_},
        "gates": gates,
    }
    if inp.debugmove:
        # trajectory records [6, n] as the reference module returns them (src/pmcxcl.cpp:1266-1282)
        n = min(int(keep["ntraj"][0]), inp.maxtraj)
        out["traj"] = keep["traj"][:6 * n].reshape(n, 6).T.copy()
        out["ntraj"] = int(keep["ntraj"][0])
    if inp.seed == SEED_FROM_FILE:
        n = inp.nreplay
        out["replay"] = {"weight": keep["rw"][:n].copy(), "tof": keep["rtof"][:n].copy(),
                         "detid": keep["rdid"][:n].copy(), "seed": keep["rseed"][:n].copy()}
    return out


def run_reference(cfg, nthread=4096, core=None, nblocksize=64, nworkers=1):
    """Run the reference kernel compiled on the host (serial when nworkers == 1).
    Returns the merged raw float field, per-thread energies, records, seeds."""
    inp, keep = make_input(cfg, nthread, core, MATH_LIBM, VARIANT_NVCC, FIELD_FLOAT_SPILL, 1)
    L = lib()
    R = reflib(pattern=inp.srctype in (5, 15))
    fieldlen = L.mcxo_fieldlen(ctypes.byref(inp)) * L.mcxo_fieldcomp(ctypes.byref(inp))
    reclen = L.mcxo_reclen(ctypes.byref(inp))
    field = np.zeros(fieldlen, np.float32)
    energy = np.zeros(2 * inp.nthread, np.float32)
    maxdet = inp.maxdetphoton
    detp = np.zeros(max(1, maxdet * max(reclen, 1)), np.float32)
    seeds = np.zeros(max(2, maxdet * 2), np.uint64)
    cnt = ctypes.c_uint(0)
    rc = R.mcxref_run(ctypes.byref(inp), ctypes.c_uint(nblocksize), ctypes.c_int(nworkers), _ptr(field),
                      _ptr(energy), _ptr(detp), _ptr(seeds), ctypes.byref(cnt))
    if rc:
        raise RuntimeError("reference harness failed with code %d" % rc)
    nsaved = min(cnt.value, maxdet)
    shape = (inp.dimx, inp.dimy, inp.dimz, -1)
    out = {
        "field_raw": field.reshape(shape, order="F"),
        "energy": energy.reshape(-1, 2),
        "detp": detp[:nsaved * reclen].reshape(nsaved, reclen).T if reclen else np.zeros((0, 0), np.float32),
        "seeds": seeds[:2 * nsaved].reshape(nsaved, 2) if inp.issaveseed else None,
        "detected": cnt.value,
    }
    if inp.debugmove:
        n = min(int(keep["ntraj"][0]), inp.maxtraj)
        out["traj"] = keep["traj"][:6 * n].reshape(n, 6).T.copy()
        out["ntraj"] = int(keep["ntraj"][0])
    return out


def cube60(**kw):
    """The reference's cube60 benchmark input (src/mcx_bench.h:33-85, pmcxcl/bench.py)."""
    cfg = {
        "nphoton": 1000000,
        "vol": np.ones((60, 60, 60), dtype=np.uint8),
        "tstart": 0, "tend": 5e-9, "tstep": 5e-9,
        "srcpos": [29, 29, 0], "srcdir": [0, 0, 1],
        "prop": [[0, 0, 1, 1], [0.005, 1, 0.01, 1.37], [0.002, 5, 0.9, 1]],
        "isreflect": 0, "seed": 1648335518,
        "detpos": [[29, 19, 0, 1], [29, 39, 0, 1], [19, 29, 0, 1], [39, 29, 0, 1]],
        "issrcfrom0": 1,
    }
    cfg.update(kw)
    return cfg


# ---------------------------------------------------------------- host layer

class RefCfgSummary(ctypes.Structure):
    """oracle/ref_utils.c refcfg_summary"""
    _fields_ = ([("dim", ctypes.c_uint * 3)] +
                [(n, ctypes.c_uint) for n in ("medianum", "detnum", "maxgate", "srcnum", "extrasrclen", "savedetflag",
                                               "debuglevel", "maxdetphoton")] +
                [(n, ctypes.c_int) for n in ("srctype", "seed", "isreflect", "issavedet", "issave2pt", "isnormalized",
                                              "outputtype", "mediabyte", "issrcfrom0", "issaveseed", "issaveexit",
                                              "issaveref", "ismomentum", "isspecular", "autopilot", "srcid")] +
                [("nphoton", ctypes.c_double)] +
                [(n, ctypes.c_float) for n in ("tstart", "tstep", "tend", "unitinmm", "minenergy")] +
                [("steps", ctypes.c_float * 3)] +
                [(n, ctypes.c_float * 4) for n in ("srcpos", "srcdir", "srcparam1", "srcparam2")] +
                [("bc", ctypes.c_char * 13), ("session", ctypes.c_char * 64)])


CONFIG_SCALARS = ["medianum", "detnum", "maxgate", "srcnum", "extrasrclen", "savedetflag", "debuglevel", "maxdetphoton",
                  "srctype", "seed", "isreflect", "issavedet", "issave2pt", "isnormalized", "outputtype", "mediabyte",
                  "issrcfrom0", "issaveseed", "issaveexit", "issaveref", "ismomentum", "isspecular", "autopilot",
                  "srcid", "nphoton", "tstart", "tstep", "tend", "unitinmm", "minenergy"]


def refutils():
    path = os.path.join(HERE, "_ref", "libmcxrefutils.so")
    if path not in _ref:
        _ref[path] = ctypes.CDLL(path)
    return _ref[path]


def refutils_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libmcxrefutils.so"))


def ref_readconfig(path):
    """The reference's mcx_readconfig on a JSON input (loading, shapes,
    preprocessing, detector mask): scalars, media, detectors and volume words
    of the loaded configuration."""
    R = refutils()
    s = RefCfgSummary()
    R.mcxref_readconfig(path.encode(), ctypes.byref(s))
    n = s.dim[0] * s.dim[1] * s.dim[2]
    vol = np.zeros(n, np.uint32)
    prop = np.zeros((s.medianum, 4), np.float32)
    det = np.zeros((max(s.detnum, 1), 4), np.float32)
    R.mcxref_copyconfig(_ptr(prop), _ptr(det), _ptr(vol))
    R.mcxref_release()
    out = {k: getattr(s, k) for k in CONFIG_SCALARS}
    out.update(dim=list(s.dim), steps=list(s.steps), bc=s.bc.decode(errors="replace"), session=s.session.decode(),
               prop=prop, detpos=det[:s.detnum], vol=vol,
               **{k: np.asarray(list(getattr(s, k)), np.float32) for k in ("srcpos", "srcdir", "srcparam1", "srcparam2")})
    return out


def ref_savedet(session, hist, histf, prop, detp, seeds, issaveseed, jdat):
    """The reference's detected-photon writer (mcx_savedetphoton / .jdat
    mcx_savejdet) into the current directory: hist = {version, maxmedia,
    detnum, colcount, totalphoton, detected, savedphoton, seedbyte, respin,
    srcnum, savedetflag, totalsource}, histf = {unitinmm, normalizer}, prop
    [maxmedia + 1, 4]; detp [count, colcount] float32, seeds [count, 16] uint8."""
    R = refutils()
    h = np.asarray(hist, np.uint32)
    hf = np.asarray(histf, np.float32)
    d = np.ascontiguousarray(detp, np.float32)
    sd = np.ascontiguousarray(seeds, np.uint8) if seeds is not None else None
    pr = np.ascontiguousarray(prop, np.float32)
    R.mcxref_savedet(session.encode(), _ptr(h), _ptr(hf), _ptr(pr), _ptr(d), _ptr(sd), ctypes.c_int(d.shape[0]),
                     ctypes.c_int(issaveseed), ctypes.c_int(jdat))


def ref_savejnii(vol, voxelsize, name, session="", maxgate=1, outputtype=0):
    """The reference's JNIfTI writer on a float32 volume (x fastest) into
    <name>.jnii, with the header's Name, LastSliceID and Description from
    session, maxgate and outputtype."""
    R = refutils()
    v = np.asfortranarray(np.asarray(vol, np.float32))
    flat = np.ascontiguousarray(v.ravel(order="F"))
    dims = np.asarray(v.shape, np.uint32)
    vs = np.asarray(list(voxelsize) + [1.0] * (v.ndim - len(voxelsize)), np.float32)
    R.mcxref_savejnii(_ptr(flat), ctypes.c_int(v.ndim), _ptr(dims), _ptr(vs), name.encode(), session.encode(),
                      ctypes.c_uint(maxgate), ctypes.c_int(outputtype))


def ref_adjoint(kind, field, ns, nd, nx, ny, nz, maxgate):
    """The reference's adjoint post-kernels (mcx_core.cl:3393-3512) on a float32
    field [nx ny nz maxgate (ns + nd)] (x fastest): [nx ny nz ns nd] floats."""
    R = reflib()
    f = np.ascontiguousarray(np.asarray(field, np.float32).ravel(order="F"))
    out = np.zeros(nx * ny * nz * ns * nd, np.float32)
    R.mcxref_adjoint(ctypes.c_int(kind), _ptr(f), _ptr(out), ctypes.c_uint(nx * ny * nz), ctypes.c_uint(maxgate),
                     ctypes.c_uint(ns), ctypes.c_uint(nd), ctypes.c_uint(nx), ctypes.c_uint(ny))
    return out
