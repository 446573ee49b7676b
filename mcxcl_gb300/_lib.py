"""ctypes binding of libmcxgb300.so (include/mcx_gb300.h).

Loading fails loudly: there is no CPU fallback for the transport path.  Build
the library first with ``python -m mcxcl_gb300.build`` (or
``__graft_entry__.build()``).
"""
import ctypes
import os

from . import build as _build

MAX_SESSION_LENGTH = 64
MAX_DEVICE = 256
mpStandalone, mpMATLAB, mpPython = 0, 1, 2


class Float4(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float), ("w", ctypes.c_float)]


class UInt4(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint), ("w", ctypes.c_uint)]


class Medium(ctypes.Structure):
    _fields_ = [("mua", ctypes.c_float), ("mus", ctypes.c_float), ("g", ctypes.c_float), ("n", ctypes.c_float)]


class ExtraSrc(ctypes.Structure):
    _fields_ = [("srcpos", Float4), ("srcdir", Float4), ("srcparam1", Float4), ("srcparam2", Float4)]


class History(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_char * 4), ("version", ctypes.c_uint), ("maxmedia", ctypes.c_uint),
                ("detnum", ctypes.c_uint), ("colcount", ctypes.c_uint), ("totalphoton", ctypes.c_uint),
                ("detected", ctypes.c_uint), ("savedphoton", ctypes.c_uint), ("unitinmm", ctypes.c_float),
                ("seedbyte", ctypes.c_uint), ("normalizer", ctypes.c_float), ("respin", ctypes.c_int),
                ("srcnum", ctypes.c_uint), ("savedetflag", ctypes.c_uint), ("totalsource", ctypes.c_uint),
                ("reserved", ctypes.c_int * 1)]


class GPUInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * MAX_SESSION_LENGTH), ("id", ctypes.c_int), ("devcount", ctypes.c_int),
                ("platformid", ctypes.c_int), ("major", ctypes.c_int), ("minor", ctypes.c_int),
                ("globalmem", ctypes.c_size_t), ("constmem", ctypes.c_size_t), ("sharedmem", ctypes.c_size_t),
                ("regcount", ctypes.c_int), ("clock", ctypes.c_int), ("sm", ctypes.c_int), ("core", ctypes.c_int),
                ("autoblock", ctypes.c_size_t), ("autothread", ctypes.c_size_t), ("maxgate", ctypes.c_uint),
                ("maxmpthread", ctypes.c_int), ("iscpu", ctypes.c_int), ("vendor", ctypes.c_int)]


class Replay(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_void_p), ("weight", ctypes.POINTER(ctypes.c_float)),
                ("tof", ctypes.POINTER(ctypes.c_float)), ("detid", ctypes.POINTER(ctypes.c_int))]


class Config(ctypes.Structure):
    """Mirror of `Config` in include/mcx_gb300.h (checked field by field
    against mcx_config_offsetof by the test suite)."""
    _fields_ = [
        ("nphoton", ctypes.c_size_t), ("nblocksize", ctypes.c_uint), ("nthread", ctypes.c_uint),
        ("seed", ctypes.c_int), ("srcpos", Float4), ("srcdir", Float4), ("tstart", ctypes.c_float),
        ("tstep", ctypes.c_float), ("tend", ctypes.c_float), ("steps", Float4), ("dim", UInt4),
        ("medianum", ctypes.c_uint), ("detnum", ctypes.c_uint), ("maxdetphoton", ctypes.c_uint),
        ("prop", ctypes.POINTER(Medium)), ("detpos", ctypes.POINTER(Float4)), ("maxgate", ctypes.c_uint),
        ("respin", ctypes.c_int), ("gpuid", ctypes.c_int), ("vol", ctypes.POINTER(ctypes.c_uint)),
        ("session", ctypes.c_char * MAX_SESSION_LENGTH),
        ("isrowmajor", ctypes.c_char), ("isreflect", ctypes.c_char), ("isrefint", ctypes.c_char),
        ("isnormalized", ctypes.c_char), ("issavedet", ctypes.c_char), ("issave2pt", ctypes.c_char),
        ("isgpuinfo", ctypes.c_char), ("isspecular", ctypes.c_char), ("issrcfrom0", ctypes.c_char),
        ("ismomentum", ctypes.c_char), ("internalsrc", ctypes.c_char), ("issaveseed", ctypes.c_char),
        ("issaveexit", ctypes.c_char), ("isatomic", ctypes.c_char), ("issaveref", ctypes.c_char),
        ("srctype", ctypes.c_char), ("autopilot", ctypes.c_char), ("outputtype", ctypes.c_char),
        ("minenergy", ctypes.c_float), ("unitinmm", ctypes.c_float), ("flog", ctypes.c_void_p),
        ("his", History), ("energytot", ctypes.c_double), ("energyabs", ctypes.c_double),
        ("energyesc", ctypes.c_double), ("maxvoidstep", ctypes.c_int), ("voidtime", ctypes.c_int),
        ("srcparam1", Float4), ("srcparam2", Float4), ("srcnum", ctypes.c_uint),
        ("srcpattern", ctypes.POINTER(ctypes.c_float)), ("deviceid", ctypes.c_char * MAX_DEVICE),
        ("workload", ctypes.c_float * MAX_DEVICE), ("exportfield", ctypes.POINTER(ctypes.c_float)),
        ("exportdetected", ctypes.POINTER(ctypes.c_float)), ("debuglevel", ctypes.c_uint),
        ("normalizer", ctypes.c_float), ("seeddata", ctypes.c_void_p), ("gscatter", ctypes.c_uint),
        ("savedetflag", ctypes.c_uint), ("detectedcount", ctypes.c_uint), ("runtime", ctypes.c_uint),
        ("parentid", ctypes.c_int), ("mediabyte", ctypes.c_uint), ("bc", ctypes.c_char * 13),
        ("nphase", ctypes.c_uint), ("invcdf", ctypes.POINTER(ctypes.c_float)), ("nangle", ctypes.c_uint),
        ("angleinvcdf", ctypes.POINTER(ctypes.c_float)), ("srcid", ctypes.c_int), ("extrasrclen", ctypes.c_uint),
        ("srcdata", ctypes.POINTER(ExtraSrc)), ("replay", Replay), ("replaydet", ctypes.c_int),
        ("detdir", ctypes.POINTER(Float4)), ("exportjacob", ctypes.POINTER(ctypes.c_float)),
        ("exactmath", ctypes.c_int), ("kernelms", ctypes.c_float),
        ("eventcount", ctypes.c_uint64 * 5), ("failedlaunch", ctypes.c_uint), ("threadused", ctypes.c_uint),
        ("exportenergy", ctypes.POINTER(ctypes.c_float)), ("savethreadenergy", ctypes.c_int),
        ("autotune", ctypes.c_int), ("savedetweight", ctypes.c_int),
        ("exportdetweight", ctypes.POINTER(ctypes.c_float)), ("replaysiteown", ctypes.c_int),
        ("omega", ctypes.c_float),
        ("polprop", ctypes.POINTER(ctypes.c_float)), ("polmedianum", ctypes.c_uint), ("lambda_", ctypes.c_float),
        ("srciquv", Float4), ("smatrix", ctypes.POINTER(Float4)),
        ("maxjumpdebug", ctypes.c_uint), ("debugdatalen", ctypes.c_uint),
        ("exportdebugdata", ctypes.POINTER(ctypes.c_float)),
        ("errorcode", ctypes.c_int),
        ("errormsg", ctypes.c_char * 256),
    ]


class DevInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 64), ("major", ctypes.c_int), ("minor", ctypes.c_int),
                ("sm", ctypes.c_int), ("clock_khz", ctypes.c_int), ("globalmem", ctypes.c_size_t),
                ("sharedmem_per_block", ctypes.c_size_t), ("constmem", ctypes.c_size_t),
                ("regs_per_block", ctypes.c_int), ("max_threads_per_sm", ctypes.c_int)]


# every symbol include/mcx_gb300.h declares
EXPORTS = [
    "mcx_initcfg", "mcx_clearcfg", "mcx_validatecfg", "mcx_list_gpu", "mcx_cleargpuinfo", "mcx_run_simulation",
    "mcx_normalize", "mcx_error", "mcx_last_error", "mcx_detreclen", "mcx_version", "mcx_rand_words", "mcx_rand_blocks", "mcx_config_sizeof",
    "mcx_config_offsetof", "mcx_release_sessions", "mcx_prepare_simulation",
    "mcxg_device_count", "mcxg_device_info", "mcxg_error_string", "mcxg_create", "mcxg_destroy",
    "mcxg_set_problem", "mcxg_set_params", "mcxg_set_seeds", "mcxg_set_seeds_lfib", "mcxg_set_trajectory", "mcxg_get_trajectory", "mcxg_set_launch", "mcxg_simulate",
    "mcxg_get_energy", "mcxg_get_thread_energy", "mcxg_get_field", "mcxg_get_field_f64", "mcxg_get_detected",
    "mcxg_get_counters", "mcxg_get_launch", "mcxg_fp32_peak", "mcxg_energy_sum_noalloc", "mcxg_autotune",
    "mcxg_set_replay", "mcxg_get_field_blocks", "mcxg_get_field_interleaved", "mcxg_set_polarization", "mcx_mie", "mcxg_get_detweight", "mcx_run_batch", "mcxg_batch_set",
    "mcxg_batch_simulate", "mcxg_batch_get_energy", "mcxg_batch_get_field", "mcx_savedetphoton",
    "mcxg_adjoint", "mcxg_get_verify", "mcx_readconfig", "mcx_parsejson", "mcxg_adjoint_field",
    "mcxg_get_field_planes", "mcxg_set_adjoint", "mcxg_get_adjoint_grad", "mcxg_batch_get_verify",
    "mcx_run_batch_verify", "mcx_keep_sessions", "mcxg_set_tile", "mcxg_get_tile", "mcx_free_buffer",
    "mcxg_set_seeds_window", "mcxg_get_seeds", "mcx_labels_u8",
    "mcxg_batch_set_words",
]

_lib = None


def load():
    """Load the shared library (raises ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("MCXGB300_LIB", _build.LIB)
    if not os.path.exists(path):
        raise ImportError("libmcxgb300.so is not built (%s); run `python -m mcxcl_gb300.build` -- "
                          "the GB300 transport path has no CPU fallback" % path)
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    L.mcx_initcfg.argtypes = [P(Config)]
    L.mcx_clearcfg.argtypes = [P(Config)]
    L.mcx_validatecfg.argtypes = [P(Config), vp, vp, ctypes.c_int]
    L.mcx_run_simulation.argtypes = [P(Config), vp, vp]
    L.mcx_readconfig.argtypes = [ctypes.c_char_p, P(Config)]
    L.mcx_parsejson.argtypes = [ctypes.c_char_p, P(Config)]
    L.mcx_list_gpu.argtypes = [P(Config), P(ctypes.c_uint), P(P(GPUInfo))]
    L.mcx_list_gpu.restype = ctypes.c_int
    L.mcx_cleargpuinfo.argtypes = [P(P(GPUInfo))]
    L.mcx_free_buffer.argtypes = [ctypes.c_void_p]
    L.mcx_free_buffer.restype = None
    L.mcx_detreclen.argtypes = [P(Config)]
    L.mcx_detreclen.restype = ctypes.c_uint
    L.mcx_version.restype = ctypes.c_char_p
    L.mcx_rand_words.argtypes = [ctypes.c_uint, vp, ctypes.c_size_t]
    L.mcx_rand_blocks.argtypes = [ctypes.c_uint, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, vp]
    L.mcx_labels_u8.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, vp]
    L.mcx_labels_u8.restype = None
    L.mcx_prepare_simulation.argtypes = [P(Config)]
    L.mcx_keep_sessions.argtypes = [ctypes.c_int]
    L.mcx_keep_sessions.restype = None
    L.mcx_prepare_simulation.restype = vp
    L.mcx_config_sizeof.restype = ctypes.c_size_t
    L.mcx_config_offsetof.argtypes = [ctypes.c_char_p]
    L.mcx_config_offsetof.restype = ctypes.c_size_t
    L.mcxg_error_string.argtypes = [ctypes.c_int]
    L.mcxg_error_string.restype = ctypes.c_char_p
    L.mcxg_device_count.argtypes = [P(ctypes.c_int)]
    L.mcxg_device_info.argtypes = [ctypes.c_int, P(DevInfo)]
    L.mcxg_create.argtypes = [ctypes.c_int, P(vp)]
    L.mcxg_destroy.argtypes = [vp]
    L.mcxg_set_problem.argtypes = [vp, vp, ctypes.c_size_t, vp, ctypes.c_uint32, vp, vp, vp, vp, vp, vp,
                                   ctypes.c_size_t]
    L.mcxg_set_params.argtypes = [vp, vp, ctypes.c_size_t]
    L.mcxg_set_seeds.argtypes = [vp, vp, ctypes.c_uint32]
    L.mcxg_set_seeds_window.argtypes = [vp, vp, ctypes.c_uint32]
    L.mcxg_get_seeds.argtypes = [vp, vp, ctypes.c_uint32]
    L.mcxg_set_launch.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.mcxg_set_tile.argtypes = [vp, ctypes.c_uint32]
    L.mcxg_get_tile.argtypes = [vp, vp]
    L.mcxg_simulate.argtypes = [vp, ctypes.c_uint, P(ctypes.c_float)]
    L.mcxg_get_energy.argtypes = [vp, P(ctypes.c_double), P(ctypes.c_double)]
    L.mcxg_get_thread_energy.argtypes = [vp, vp]
    L.mcxg_get_field.argtypes = [vp, vp, ctypes.c_double]
    L.mcxg_get_field_f64.argtypes = [vp, vp]
    L.mcxg_get_verify.argtypes = [vp, vp, vp, vp]
    L.mcxg_get_field_planes.argtypes = [vp, vp, vp]
    L.mcxg_set_adjoint.argtypes = [vp, vp, ctypes.c_uint32]
    L.mcxg_get_adjoint_grad.argtypes = [vp, vp, vp]
    u32 = ctypes.c_uint32
    L.mcxg_adjoint_field.argtypes = [vp, ctypes.c_int, vp, u32, u32, u32, u32, u32, u32, vp]
    L.mcxg_get_detected.argtypes = [vp, vp, vp, P(ctypes.c_uint32)]
    L.mcxg_get_counters.argtypes = [vp, vp, vp]
    L.mcxg_get_launch.argtypes = [vp, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int)]
    L.mcxg_fp32_peak.argtypes = [vp, P(ctypes.c_double)]
    L.mcxg_energy_sum_noalloc.argtypes = [ctypes.c_int, vp, ctypes.c_uint32, vp]
    L.mcxg_autotune.argtypes = [vp, ctypes.c_uint32, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int)]
    _lib = L
    return L


def libc():
    return ctypes.CDLL(None)
