"""The ``pmcxcl`` Python interface, backed by the GB300 transport path.

``run(**cfg)`` takes the reference module's keys and returns the same output
dictionary (src/pmcxcl.cpp:428-1553): the dict is turned into a `Config`
(parse_config, 428-1110), validated, simulated through the C ABI
(mcx_run_simulation) and unpacked (1263-1521).  ``gpuinfo()`` and
``version()`` mirror the reference's module functions (1600-1664).

Arrays follow the reference's conventions: volumes and outputs are
Fortran-ordered (x fastest), ``flux`` is ``[Nx, Ny, Nz, gates]``, ``detp`` is
``[reclen, ndetected]`` and ``seeds`` is ``uint8 [16, ndetected]``.
"""
import ctypes
import weakref

import numpy as np

from . import _lib, media
from ._lib import Config, ExtraSrc, Float4, GPUInfo, Medium

SEED_FROM_FILE = -999

SRCTYPES = ["pencil", "isotropic", "cone", "gaussian", "planar", "pattern", "fourier", "arcsine", "disk",
            "fourierx", "fourierx2d", "zgaussian", "line", "slit", "pencilarray", "pattern3d", "hyperboloid",
            "ring"]
OUTPUTTYPES = ["flux", "fluence", "energy", "jacobian", "nscat", "wl", "wp", "wm", "rf", "length", "rfmus",
               "wltof", "wptof", "adjoint", "adjoint_dcoeff", "adjoint_mus", "adjoint_musp", "adjoint_mua_d",
               "adjoint_mua_musp"]
SAVEFLAGS = "DSPMXVWI"
DEBUGFLAGS = "RMPT"        # R: RNG stream, M: trajectories, P: progress, T: trajectories only (mcx_utils.c:117)

_SCALARS_INT = ["nphoton", "nblocksize", "nthread", "maxdetphoton", "maxgate", "maxjumpdebug", "respin", "isreflect", "isrefint",
                "isnormalized", "isgpuinfo", "issrcfrom0", "autopilot", "voidtime", "issaveref", "maxvoidstep",
                "gscatter", "srcnum", "srcid", "isatomic", "internalsrc", "issavedet", "exactmath",
                "savethreadenergy", "autotune"]
_SCALARS_BOOL = ["issaveexit", "ismomentum", "isspecular", "issave2pt", "issaveseed"]
_SCALARS_FLOAT = ["tstart", "tstep", "tend", "minenergy", "unitinmm", "omega"]


class MCXError(RuntimeError):
    """Raised when the simulation reports an error (the reference raises RuntimeError)."""


def _cbuf(arr, ctype):
    """Copy a numpy array into malloc'd memory owned by the Config (freed by mcx_clearcfg)."""
    arr = np.ascontiguousarray(arr)
    libc = _lib.libc()
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    p = libc.malloc(max(arr.nbytes, 1))
    if not p:
        raise MemoryError("malloc failed")
    ctypes.memmove(p, arr.ctypes.data, arr.nbytes)
    return ctypes.cast(p, ctypes.POINTER(ctype))


def _cempty(n, ctype, dtype):
    """malloc'd memory owned by the Config (freed by mcx_clearcfg), as a
    pointer and a numpy view of n elements."""
    libc = _lib.libc()
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    p = libc.malloc(max(n * np.dtype(dtype).itemsize, 1))
    if not p:
        raise MemoryError("malloc failed")
    ptr = ctypes.cast(p, ctypes.POINTER(ctype))
    return ptr, np.ctypeslib.as_array(ptr, shape=(n,)).view(dtype)


def _rows(v, ncol):
    a = np.asarray(v, dtype=np.float32)
    if a.ndim == 1:
        a = a.reshape(1, -1)
    if a.shape[1] > ncol:
        raise ValueError("too many columns")
    return a


def _flags(s, letters):
    if isinstance(s, (int, np.integer)):
        return int(s)
    v = 0
    for ch in str(s).upper():
        if ch in letters:
            v |= 1 << letters.index(ch)
    return v


def _set_volume(C, vol, unitinmm=1.0):
    """parseVolume (src/pmcxcl.cpp:93-426): dtype and leading dimension decide
    the media format (mcxcl_gb300.media)."""
    held = []

    def alloc(n):
        ptr, view = _cempty(n, ctypes.c_uint, np.uint32)
        held.append((ptr, view))
        return view

    words, C.mediabyte, dims = media.encode(vol, unitinmm, alloc)
    C.dim.x, C.dim.y, C.dim.z = [int(d) for d in dims]
    if held and words is held[0][1]:
        C.vol = held[0][0]
    else:
        for ptr, _ in held:
            _lib.libc().free(ptr)
        C.vol = _cbuf(words, ctypes.c_uint)


def _set_sources(C, cfg):
    keys = ("srcpos", "srcdir", "srcparam1", "srcparam2")
    rows = {k: _rows(cfg[k], 4) for k in keys if k in cfg}
    n = max([r.shape[0] for r in rows.values()] + [1])
    for k, r in rows.items():
        f = getattr(C, k)
        vals = list(r[0]) + [None] * (4 - r.shape[1])
        for comp, v in zip("xyzw", vals):
            if v is not None:
                setattr(f, comp, float(v))
    if n > 1:
        extra = (ExtraSrc * (n - 1))()
        for i in range(1, n):
            e = extra[i - 1]
            e.srcpos.w = 1.0
            for k, r in rows.items():
                if i < r.shape[0]:
                    f = getattr(e, k)
                    for comp, v in zip("xyzw", r[i]):
                        setattr(f, comp, float(v))
        C.extrasrclen = n - 1
        arr = np.frombuffer(extra, dtype=np.float32).copy()
        C.srcdata = _cbuf(arr, ExtraSrc)


def parse_config(cfg, C):
    """Fill a Config from a pmcxcl-style dict (src/pmcxcl.cpp:428-1110)."""
    L = _lib.load()
    L.mcx_initcfg(ctypes.byref(C))
    C.parentid = _lib.mpPython
    C.flog = None
    for k in _SCALARS_INT:
        if k in cfg:
            v = int(cfg[k])
            setattr(C, k, bytes([v & 0xFF]) if isinstance(getattr(C, k), bytes) else v)
    for k in _SCALARS_BOOL:
        if k in cfg:
            setattr(C, k, bytes([1 if cfg[k] else 0]))
    for k in _SCALARS_FLOAT:
        if k in cfg:
            setattr(C, k, float(cfg[k]))
    if "steps" in cfg:
        s = np.asarray(cfg["steps"], np.float32).ravel()
        C.steps.x, C.steps.y, C.steps.z = [float(x) for x in s[:3]]
    if "vol" not in cfg:
        raise ValueError("Configuration must specify a 2/3/4D volume.")
    _set_volume(C, cfg["vol"], float(cfg.get("unitinmm", 1.0)))
    _set_sources(C, cfg)
    if "detpos" in cfg and np.asarray(cfg["detpos"]).size:
        d = _rows(cfg["detpos"], 4)
        if d.shape[1] != 4:
            raise ValueError("the 'detpos' field must have 4 columns (x,y,z,radius)")
        C.detnum = d.shape[0]
        C.detpos = _cbuf(d, Float4)
    if "detdir" in cfg:
        # per detector {vx, vy, vz, focal length}: detectors run as sources for the adjoint outputs
        # (src/pmcxcl.cpp:693-724)
        dd = np.asarray(cfg["detdir"], np.float32)
        dd = dd.reshape(1, -1) if dd.ndim == 1 else dd
        if dd.shape[1] != 4:
            raise ValueError("the 'detdir' field must have 4 columns (vx,vy,vz,focallength)")
        if dd.shape[0] != C.detnum:
            raise ValueError("the number of rows in 'detdir' must match 'detpos'")
        C.detdir = _cbuf(dd, Float4)
    if "prop" not in cfg:
        raise ValueError("You must define 'vol' and 'prop' field.")
    p = _rows(cfg["prop"], 4)
    if p.shape[1] != 4:
        raise ValueError("the 'prop' field must have 4 columns (mua,mus,g,n)")
    C.medianum = p.shape[0]
    C.prop = _cbuf(p, Medium)
    if "polprop" in cfg:
        # scatterers of labels 1..N for the polarised transport: rows {mua, radius (um), number
        # density (1/um^3), n_sphere, n_background} (src/pmcxcl.cpp:754-784)
        pp = np.asarray(cfg["polprop"], np.float32)
        if pp.ndim == 1:
            pp = pp.reshape(1, -1)
        if pp.ndim != 2 or pp.shape[1] != 5:
            raise ValueError("the 'polprop' field must have 5 columns (mua, radius, rho, n_sph,n_bkg)")
        C.polmedianum = pp.shape[0]
        C.polprop = _cbuf(pp, ctypes.c_float)
    if "lambda" in cfg:
        C.lambda_ = float(cfg["lambda"])
    if "srciquv" in cfg:
        q = np.asarray(cfg["srciquv"], np.float32).ravel()
        if q.size != 4:
            raise ValueError("the 'srciquv' field must have 4 elements (I, Q, U, V)")
        C.srciquv = Float4(*[float(v) for v in q])
    if "session" in cfg:
        C.session = str(cfg["session"]).encode()[:63]
    if "srctype" in cfg:
        st = str(cfg["srctype"]).lower()
        if st not in SRCTYPES:
            raise ValueError("the specified source type is not supported")
        C.srctype = bytes([SRCTYPES.index(st)])
    if "outputtype" in cfg:
        ot = str(cfg["outputtype"]).lower()
        if ot not in OUTPUTTYPES:
            raise ValueError("the specified output type is not supported")
        idx = OUTPUTTYPES.index(ot)
        if idx >= 5:                 # the reference maps wl to jacobian, wp to nscat
            idx -= 2
        C.outputtype = bytes([idx])
    if "debuglevel" in cfg:
        C.debuglevel = _flags(cfg["debuglevel"], DEBUGFLAGS)
    if "savedetflag" in cfg:
        C.savedetflag = _flags(cfg["savedetflag"], SAVEFLAGS)
    if "srcpattern" in cfg:
        pat = np.asarray(cfg["srcpattern"], np.float32).reshape(-1, order="F")
        C.srcpattern = _cbuf(pat, ctypes.c_float)
    if "invcdf" in cfg:
        t = np.asarray(cfg["invcdf"], np.float32).ravel()
        C.nphase = t.size
        C.invcdf = _cbuf(t, ctypes.c_float)
    if "angleinvcdf" in cfg:
        t = np.asarray(cfg["angleinvcdf"], np.float32).ravel()
        C.nangle = t.size
        C.angleinvcdf = _cbuf(t, ctypes.c_float)
    if "bc" in cfg:
        b = str(cfg["bc"]).encode()
        if not b or len(b) > 12:
            raise ValueError("the 'bc' field must be a non-empty string of at most 12 characters")
        C.bc = b + b"\0" * (13 - len(b))
    if "seed" in cfg:
        sv = cfg["seed"]
        if isinstance(sv, (int, float, np.integer, np.floating)):
            C.seed = int(sv)
        else:
            # replay: the uint8 [16, N] seeds of a previous run's detected photons (src/pmcxcl.cpp:1021-1047)
            s8 = np.asfortranarray(np.asarray(sv), dtype=np.uint8)
            if s8.ndim != 2 or s8.shape[0] != 16:
                raise ValueError("the row number of cfg.seed does not match RNG seed byte-length")
            raw = np.ascontiguousarray(s8.T).tobytes()
            buf = _libc_malloc(max(len(raw), 1))
            ctypes.memmove(buf, raw, len(raw))
            C.replay.seed = buf
            C.seed = SEED_FROM_FILE
            C.nphoton = s8.shape[1]
    if "replaydet" in cfg:
        C.replaydet = int(cfg["replaydet"])
    if C.seed == SEED_FROM_FILE and "detphotons" not in cfg and "replayweight" in cfg:
        # GB300 addition: each replayed photon's weight, time of flight and detector id given directly
        n = int(C.nphoton)
        for key, field, dt, ct in (("replayweight", "weight", np.float32, ctypes.c_float),
                                   ("replaytof", "tof", np.float32, ctypes.c_float),
                                   ("replaydetid", "detid", np.int32, ctypes.c_int)):
            a = np.ascontiguousarray(np.asarray(cfg[key], dt).ravel())
            if a.size != n:
                raise ValueError("'%s' must have one entry per replayed photon" % key)
            buf = _libc_malloc(max(a.nbytes, 4))
            ctypes.memmove(buf, a.ctypes.data, a.nbytes)
            setattr(C.replay, field, ctypes.cast(buf, ctypes.POINTER(ct)))
    for key in ("savedetweight", "replaysiteown"):
        if key in cfg:
            setattr(C, key, int(cfg[key]))
    if "gpuid" in cfg:
        g = cfg["gpuid"]
        C.deviceid = b"\0" * 256
        if isinstance(g, (int, np.integer)):
            if not 0 < g < 256:
                raise ValueError("GPU id must be positive and can not be more than 256")
            C.deviceid = b"0" * (g - 1) + b"1"
        else:
            C.deviceid = str(g).encode()[:256]
    if "workload" in cfg:
        w = np.asarray(cfg["workload"], np.float32).ravel()
        for i, v in enumerate(w[:256]):
            C.workload[i] = float(v)
    return C


_libc = None


def _libc_malloc(n):
    """Host buffers the Config owns are freed by mcx_clearcfg, so they come from malloc."""
    global _libc
    if _libc is None:
        _libc = ctypes.CDLL(None)
        _libc.malloc.restype = ctypes.c_void_p
        _libc.malloc.argtypes = [ctypes.c_size_t]
    p = _libc.malloc(n)
    if not p:
        raise MemoryError("malloc failed")
    return p


def _detphotons(cfg):
    """cfg['detphotons']: the float32 [reclen, N] records of the baseline run
    (src/pmcxcl.cpp:1006-1018); a dict with a 'data' entry is accepted too."""
    d = cfg.get("detphotons")
    if d is None:
        return None
    if isinstance(d, dict):
        d = d.get("data", d.get("detp"))
    d = np.asarray(d, np.float32)
    if d.ndim != 2:
        raise ValueError("Invalid detphotons field value")
    return np.ascontiguousarray(d.T)


def _check(C):
    if C.errorcode:
        raise MCXError("MCX ERROR(%d): %s" % (C.errorcode, C.errormsg.decode(errors="replace")))


def run(cfg=None, **kwargs):
    """Run one simulation; returns the reference's output dictionary.

    Extra (GB300) keys accepted: ``exactmath`` -- run the IEEE-only kernel
    that reproduces the CPU oracle bit for bit (slower, for verification);
    ``autotune`` -- time the launch shapes on a photon sample (once per
    problem shape and GPU) and run with the fastest; ``savethreadenergy`` --
    return each reference thread's escaped and launched weight;
    ``savedetweight`` -- return ``detweight`` [2, N], each detected photon's
    weight and time of flight when detected; a replay may give
    ``replayweight``/``replaytof``/``replaydetid`` (one entry per seed column)
    instead of ``detphotons``, and ``replaysiteown`` = 1 makes the
    scattering-site outputs use each photon's own entries.

    Random numbers: with the default ``autopilot`` the fast kernel runs
    nphoton/2 threads (at least 64 x 64 x SM count, at most 32 times that),
    where the reference runs 64 x 64 x SM count,
    so the same ``seed`` gives the same statistics but not the same photons
    as the reference.  Give ``autopilot=0`` with the reference's ``nthread``
    and ``nblocksize`` (and ``exactmath=1``) to follow its photons one for
    one.

    Device memory: one session per GPU stays cached between calls (see
    ``keep_sessions``).  Output arrays: ``flux`` (a real field without saved
    reflectance), ``detp``, ``seeds`` and ``detweight`` are views of the library's own output buffers, handed over
    without a copy (writable, ``base`` not None); a buffer goes back to the
    library when its last view is collected, and while sessions are kept the
    next call reads its outputs into it."""
    cfg = dict(cfg or {}, **kwargs)
    L = _lib.load()
    C = Config()
    try:
        parse_config(cfg, C)
        recs = _detphotons(cfg)
        if recs is not None:
            dims = (ctypes.c_int * 2)(recs.shape[1], recs.shape[0])
            seedbyte = 16 if C.seed == SEED_FROM_FILE else 0
            L.mcx_validatecfg(ctypes.byref(C), recs.ctypes.data_as(ctypes.c_void_p), dims, seedbyte)
        else:
            L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
        _check(C)
        L.mcx_run_simulation(ctypes.byref(C), None, None)
        _check(C)
        return _outputs(cfg, C)
    finally:
        L.mcx_clearcfg(ctypes.byref(C))


def keep_sessions(keep=True):
    """keep=True (the default): one device session per GPU stays cached
    between ``run`` calls, reusing its buffers, uploaded volume and tuned
    launch shape.  keep=False releases the cached sessions now and after
    every later call, so no device memory outlives a call, as with the
    reference's module."""
    _lib.load().mcx_keep_sessions(1 if keep else 0)


def run_batch(cfgs, photons_per_thread=0, graph=False, aggregate=False, verify=False):
    """Run many simulations in one persistent launch (a GB300 addition).

    cfgs: a list of run() dictionaries (label volumes, no detectors).  Returns
    the list of their output dictionaries, as run() would give one by one.
    photons_per_thread sets how many photons each reference thread (RNG
    stream) runs (0: 1 up to 2**18 photons, 2 above); graph=True
    captures the launch as a CUDA graph.  verify=True also accumulates every
    deposit in FP64 and adds to each output's 'stat' the compensated field's
    max and median relative error over its non-zero elements and the error
    of its total against it ('relerr_max', 'relerr_median', 'relerr_total')."""
    L = _lib.load()
    Cs = [Config() for _ in cfgs]
    try:
        for cfg, C in zip(cfgs, Cs):
            parse_config(dict(cfg), C)
            L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
            _check(C)
        arr = (ctypes.POINTER(Config) * len(Cs))(*[ctypes.pointer(C) for C in Cs])
        rel = None
        if verify:
            rel = np.zeros(3 * len(Cs), np.float64)
            L.mcx_run_batch_verify(arr, len(Cs), ctypes.c_uint(int(photons_per_thread)),
                                   rel.ctypes.data_as(ctypes.c_void_p))
        else:
            flags = (32 if graph else 0) | (16 if aggregate else 0)
            L.mcx_run_batch(arr, len(Cs), ctypes.c_uint(int(photons_per_thread)), ctypes.c_uint(flags))
        _check(Cs[0])
        outs = [_outputs(cfg, C) for cfg, C in zip(cfgs, Cs)]
        if rel is not None:
            for k, o in enumerate(outs):
                o["stat"].update(relerr_max=float(rel[3 * k]), relerr_median=float(rel[3 * k + 1]),
                                 relerr_total=float(rel[3 * k + 2]))
        return outs
    finally:
        for C in Cs:
            L.mcx_clearcfg(ctypes.byref(C))


def _take(C, name, ctype, n):
    """A 1-D array of n ctype items over the library's output buffer C.<name>,
    without a copy: the Config lets go of the buffer (mcx_clearcfg skips a
    NULL pointer) and the array frees it with mcx_free_buffer when the last
    view of it is collected."""
    addr = ctypes.cast(getattr(C, name), ctypes.c_void_p).value
    arr = np.ctypeslib.as_array(ctypes.cast(addr, ctypes.POINTER(ctype)), shape=(n,))
    setattr(C, name, None)
    weakref.finalize(arr, _lib.load().mcx_free_buffer, addr)
    return arr


def _outputs(cfg, C):
    """Assemble the output dictionary (src/pmcxcl.cpp:1263-1521).  The field
    and the detected-photon records are the library's buffers, taken over
    without a copy."""
    L = _lib.load()
    out = {}
    reclen = L.mcx_detreclen(ctypes.byref(C))
    ndet = C.detectedcount
    if C.issaveseed != b"\0" and ndet:
        out["seeds"] = _take(C, "seeddata", ctypes.c_uint8, ndet * 16).reshape(ndet, 16).T
    if C.issavedet != b"\0" and ndet:
        out["detp"] = _take(C, "exportdetected", ctypes.c_float, ndet * reclen).reshape(ndet, reclen).T
        if C.savedetweight and C.exportdetweight:
            out["detweight"] = _take(C, "exportdetweight", ctypes.c_float, ndet * 2).reshape(ndet, 2).T
    if C.issave2pt != b"\0":
        gates = int((C.tend - C.tstart) / C.tstep + 0.5)
        nsrc = C.extrasrclen + 1 if (C.extrasrclen and C.srcid < 0) else 1
        ndetblk = C.detnum if (C.seed == SEED_FROM_FILE and C.replaydet == -1) else 1
        # photon sharing: one field per pattern, patterns innermost (src/pmcxcl.cpp:1330)
        nshare = C.srcnum if (C.srcnum > 1 and ord(C.srctype) in (5, 15)) else 1
        # complex fields (src/pmcxcl.cpp:1339-1341, 1388-1409): the RF transport
        # returns complex64, the rf / rfmus replay outputs a trailing axis of 2
        replay = C.seed == SEED_FROM_FILE
        rffwd = C.omega > 0 and not replay
        rfrep = replay and ord(C.outputtype) in (OUTPUTTYPES.index("rf") - 2, OUTPUTTYPES.index("rfmus") - 2)
        comps = 2 if (rffwd or rfrep) else 1
        n = C.dim.x * C.dim.y * C.dim.z * gates * nsrc * ndetblk * nshare
        f = _take(C, "exportfield", ctypes.c_float, n * comps)
        if rffwd:
            f = f[:n] + 1j * f[n:]
            f = f.astype(np.complex64)
        if rfrep:
            dims = (C.dim.x, C.dim.y, C.dim.z, gates) + ((ndetblk,) if ndetblk > 1 else (1,)) + (2,)
        elif nshare > 1:
            dims = (nshare * C.dim.x, C.dim.y, C.dim.z, gates)
        elif nsrc > 1:
            dims = (C.dim.x, C.dim.y, C.dim.z, gates, ndetblk, nsrc)
        elif ndetblk > 1:
            dims = (C.dim.x, C.dim.y, C.dim.z, gates, ndetblk)
        else:
            dims = (C.dim.x, C.dim.y, C.dim.z, gates)
        flux = f.reshape(dims, order="F")
        if C.issaveref != b"\0":
            vol = np.ctypeslib.as_array(C.vol, shape=(C.dim.x * C.dim.y * C.dim.z,))
            mask = (vol & 0x7FFFFFFF).reshape((1, C.dim.x, C.dim.y, C.dim.z), order="F") != 0
            fl = flux.reshape((nshare, C.dim.x, C.dim.y, C.dim.z, -1), order="F")
            dt = np.complex64 if np.iscomplexobj(fl) else np.float32
            dref = np.where(mask[..., None], 0.0, -fl).astype(dt).reshape(dims, order="F")
            flux = np.where(mask[..., None], fl, 0.0).astype(dt).reshape(dims, order="F")
            out["dref"] = dref
        out["flux"] = flux
        out["stat"] = {
            "runtime": C.runtime,
            "nphoton": C.nphoton * (C.respin if C.respin > 1 else 1),
            "energytot": C.energytot,
            "energyabs": C.energyabs,
            "normalizer": C.normalizer,
            "unitinmm": C.unitinmm,
            "workload": [C.workload[0]],
            # GB300 additions
            "kernelms": C.kernelms,
            "detected": C.his.detected,
            "energyesc": C.energyesc,
            "failedlaunch": C.failedlaunch,
        }
        if C.exactmath:
            out["stat"]["eventcount"] = dict(zip(("step", "scatter", "launch", "reflect", "failed"),
                                                 [int(x) for x in C.eventcount]))
    if C.polprop and C.polmedianum:
        # the labels' properties after Mie theory set their mus and g, per mm (src/pmcxcl.cpp:1510-1521)
        pr = np.ctypeslib.as_array(ctypes.cast(C.prop, ctypes.POINTER(ctypes.c_float)), shape=(C.medianum * 4,))
        pr = pr.reshape(C.medianum, 4).copy()
        pr[1:C.polmedianum + 1, :2] /= C.unitinmm
        out["prop"] = pr.T
        if C.smatrix:
            # GB300 addition: the Mueller rows the run used, [polmedianum, 181, {S11, S12, S33, S34}]
            sm = np.ctypeslib.as_array(ctypes.cast(C.smatrix, ctypes.POINTER(ctypes.c_float)),
                                       shape=(C.polmedianum * 181 * 4,))
            out["smatrix"] = sm.reshape(C.polmedianum, 181, 4).copy()
    if C.outputtype[0] >= 11 and C.exportjacob:
        # adjoint Jacobians by name, [Nx, Ny, Nz, sources x detectors] (src/pmcxcl.cpp:1413-1480)
        ot = C.outputtype[0]
        ns = C.extrasrclen + 1 - C.detnum
        npair = ns * C.detnum
        n = C.dim.x * C.dim.y * C.dim.z * npair
        names = {11: ("jmua",), 12: ("jd",), 13: ("jmus",), 14: ("jmusp",), 15: ("jmua", "jd"), 16: ("jmua", "jmusp")}[ot]
        j = np.ctypeslib.as_array(C.exportjacob, shape=(n * len(names),)).copy()
        for k, name in enumerate(names):
            out[name] = j[k * n:(k + 1) * n].reshape((C.dim.x, C.dim.y, C.dim.z, npair), order="F")
    if (C.debuglevel & 10) and C.exportdebugdata:
        # trajectory records [6, n] (src/pmcxcl.cpp:1266-1282): photon id as uint bits, x, y, z, w, source id
        n = C.debugdatalen
        tr = np.ctypeslib.as_array(C.exportdebugdata, shape=(max(n, 1) * 6,))[:n * 6].copy()
        out["traj"] = tr.reshape(n, 6).T
    if C.savethreadenergy and C.exportenergy:
        e = np.ctypeslib.as_array(C.exportenergy, shape=(2 * C.threadused,)).copy()
        out["threadenergy"] = e.reshape(C.threadused, 2)
    if cfg.get("dumpmask"):
        vol = np.ctypeslib.as_array(C.vol, shape=(C.dim.x * C.dim.y * C.dim.z,)).copy()
        out["vol"] = vol.reshape((C.dim.x, C.dim.y, C.dim.z), order="F")
    return out


def gpuinfo():
    """List CUDA devices as the reference's pmcxcl.gpuinfo() lists OpenCL ones."""
    L = _lib.load()
    C = Config()
    L.mcx_initcfg(ctypes.byref(C))
    C.flog = None
    info = ctypes.POINTER(GPUInfo)()
    n = L.mcx_list_gpu(ctypes.byref(C), None, ctypes.byref(info))
    out = []
    for i in range(n):
        g = info[i]
        out.append({k: (getattr(g, k).decode() if k == "name" else getattr(g, k))
                    for k in ("name", "id", "devcount", "major", "minor", "globalmem", "constmem", "sharedmem",
                              "regcount", "clock", "sm", "core", "autoblock", "autothread", "maxgate")})
    if n:
        L.mcx_cleargpuinfo(ctypes.byref(info))
    return out


def version():
    return _lib.load().mcx_version().decode()
