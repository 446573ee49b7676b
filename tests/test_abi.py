"""The C ABI without a GPU: the library loads, exports every symbol the public
header declares, the Python mirror of Config matches the C layout, and
errors come back as exceptions (library mode) instead of exiting."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mcx_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from mcxcl_gb300 import build
    build.build()
    from mcxcl_gb300 import _lib
    return _lib.load()


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(mcxg?_[a-z0-9_]+)\s*\(", text))
    return sorted(n for n in names if not n.isupper())


def test_header_declarations_are_exported(lib):
    from mcxcl_gb300 import _lib
    declared = _declared_functions()
    assert declared, "no declarations parsed"
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == declared


def test_config_layout_matches(lib):
    from mcxcl_gb300 import _lib
    assert lib.mcx_config_sizeof() == ctypes.sizeof(_lib.Config)
    for name, _ in _lib.Config._fields_:
        assert lib.mcx_config_offsetof(name.encode()) == getattr(_lib.Config, name).offset, name
    assert lib.mcx_config_offsetof(b"no_such_field") == ctypes.c_size_t(-1).value


def test_initcfg_defaults(lib):
    """mcx_initcfg defaults, src/mcx_utils.c:203-366."""
    from mcxcl_gb300 import _lib
    C = _lib.Config()
    lib.mcx_initcfg(ctypes.byref(C))
    assert C.tend == pytest.approx(5e-9) and C.tstep == pytest.approx(5e-9)
    assert C.nthread == 16384 and C.nblocksize == 64 and C.seed == 0x623F9A9E
    assert C.isreflect == b"\x01" and C.isnormalized == b"\x01" and C.issavedet == b"\x01"
    assert C.savedetflag == 5 and C.maxdetphoton == 1000000 and C.gscatter == 1000000000
    assert C.maxvoidstep == 1000 and C.autopilot == b"\x01" and C.srcpos.w == 1.0
    assert C.deviceid[0:1] == b"1"


def test_device_layer_reports_no_device_cleanly(lib):
    n = ctypes.c_int(-1)
    rc = lib.mcxg_device_count(ctypes.byref(n))
    if rc != 0:
        assert n.value == 0
    assert lib.mcxg_error_string(6) == b"no CUDA device"


def test_validate_errors_raise(lib):
    import mcxcl_gb300
    vol = np.ones((4, 4, 4), np.uint8) * 3
    with pytest.raises(mcxcl_gb300.MCXError, match="less than the labels"):
        mcxcl_gb300.run(nphoton=10, vol=vol, prop=[[0, 0, 1, 1], [0.1, 1, 0, 1]], srcpos=[1, 1, 0],
                        srcdir=[0, 0, 1])
    with pytest.raises(mcxcl_gb300.MCXError, match="time gate"):
        mcxcl_gb300.run(nphoton=10, vol=np.ones((4, 4, 4), np.uint8), prop=[[0, 0, 1, 1], [0.1, 1, 0, 1]],
                        srcpos=[1, 1, 0], srcdir=[0, 0, 1], tstart=1e-9, tend=0.5e-9)
    with pytest.raises(mcxcl_gb300.MCXError, match="unitary"):
        mcxcl_gb300.run(nphoton=10, vol=np.ones((4, 4, 4), np.uint8), prop=[[0, 0, 1, 1], [0.1, 1, 0, 1]],
                        srcpos=[1, 1, 0], srcdir=[0, 0, 2])
    with pytest.raises(mcxcl_gb300.MCXError, match="Jacobian output"):
        mcxcl_gb300.run(nphoton=10, vol=np.ones((4, 4, 4), np.uint8), prop=[[0, 0, 1, 1], [0.1, 1, 0, 1]],
                        srcpos=[1, 1, 0], srcdir=[0, 0, 1], outputtype="jacobian")
    with pytest.raises(ValueError):
        mcxcl_gb300.run(nphoton=10, vol=np.ones((4, 4, 4), np.uint8), prop=[[0, 0, 1]], srcpos=[1, 1, 0])


def test_pmath_bits_match_oracle_copy():
    """The kernel's exact-math header and the oracle's copy produce the same bits."""
    import subprocess
    import tempfile
    src = r'''
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include "mcx_pmath.cuh"
#include "oracle_pmath.h"
int main(void) {
    uint32_t bad = 0, n = 0;
    for (uint32_t k = 0; k < 2000000; k++) {
        float u = (float)k / 2000000.f;
        float xs[5] = {u + 1.19209290e-07f, -u * 40.f, u * 6.28318530717959f, 2.f * u - 1.f, u * 1e3f};
        float a = pm_logf(xs[0]), b = opm_logf(xs[0]);
        float c = pm_expf(xs[1]), d = opm_expf(xs[1]);
        float s1, c1, s2, c2;
        pm_sincosf(xs[2], &s1, &c1);
        opm_sincosf(xs[2], &s2, &c2);
        float e = pm_acosf(xs[3]), f = opm_acosf(xs[3]);
        float g1, h1, g2, h2;
        pm_sincosf(xs[4], &g1, &h1);
        opm_sincosf(xs[4], &g2, &h2);
        bad += memcmp(&a, &b, 4) != 0;
        bad += memcmp(&c, &d, 4) != 0;
        bad += memcmp(&s1, &s2, 4) != 0;
        bad += memcmp(&c1, &c2, 4) != 0;
        bad += memcmp(&e, &f, 4) != 0;
        bad += memcmp(&g1, &g2, 4) != 0;
        bad += memcmp(&h1, &h2, 4) != 0;
        n += 7;
    }
    printf("%u %u\n", bad, n);
    return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "mcxcl_gb300", "csrc"),
                        "-I", os.path.join(ROOT, "oracle"), c, "-o", exe, "-lm"], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    assert out[0] == "0", out


def test_pmath_accuracy():
    """The oracle's deterministic math stays within a few ulp of double precision."""
    import oracle
    L = oracle.lib()
    rs = np.random.RandomState(0)
    for fn, ref, xs in (
            (L.mcxo_pm_logf, np.log, rs.uniform(1.2e-7, 1.0, 20000)),
            (L.mcxo_pm_expf, np.exp, rs.uniform(-80, 5, 20000)),
            (L.mcxo_pm_acosf, np.arccos, rs.uniform(-1, 1, 20000))):
        xs = xs.astype(np.float32)
        got = np.array([fn(float(x)) for x in xs], np.float64)
        want = ref(xs.astype(np.float64))
        ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
        err = np.abs(got - want) / np.maximum(ulp, 1e-45)
        assert err.max() < 4.0, (fn.__name__, err.max())
    s = ctypes.c_float()
    c = ctypes.c_float()
    for x in rs.uniform(0, 2 * np.pi, 20000).astype(np.float32):
        L.mcxo_pm_sincosf(ctypes.c_float(x), ctypes.byref(s), ctypes.byref(c))
        assert abs(s.value - np.sin(np.float64(x))) < 3e-7
        assert abs(c.value - np.cos(np.float64(x))) < 3e-7


def test_volume_encodings():
    """pmcxcl's volume encodings (src/pmcxcl.cpp:93-426): float mua scaled by
    unitinmm with 0 -> EPS and NaN -> 0; the reference's truncating
    float -> half conversion; label + half property; byte and short words."""
    from mcxcl_gb300 import media
    v = np.zeros((1, 2, 1, 1), np.float32)
    v[0, 0], v[0, 1] = 0.0, np.nan
    w, mb, dims = media.encode(v, 0.5)
    assert mb == 101 and dims == (2, 1, 1)
    assert w[0] == np.float32(1e-10).view(np.uint32) and w[1] == 0
    w, _, _ = media.encode(np.full((1, 1, 1, 1), 0.02, np.float32), 0.5)
    assert w[0] == np.float32(np.float32(0.02) * np.float32(0.5)).view(np.uint32)
    # normal numbers: sign | (exponent - 112) << 10 | top ten mantissa bits (truncation, not rounding)
    x = np.array([1.0, 0.5, 0.01, 1.37, 3.0, 0.333333], np.float32)
    b = x.view(np.uint32).astype(np.int64)
    want = ((((b >> 31) << 5) | (((b >> 23) & 0xFF) - 112)) << 10) | ((b >> 13) & 0x3FF)
    assert np.array_equal(media.float_to_half_bits(x).astype(np.int64), want)
    v2 = np.zeros((2, 1, 1, 1), np.float32)
    v2[:, 0, 0, 0] = [0.01, 1.0]
    w, mb, _ = media.encode(v2)
    assert mb == 100 and w[0] == (0x211E | (0x3C00 << 16))
    w, mb, _ = media.encode(np.zeros((2, 1, 1, 1), np.float32))
    assert w[0] == 0x00010000                       # an all-zero voxel is not void
    v3 = np.zeros((3, 1, 1, 1), np.float32)
    v3[:, 0, 0, 0] = [0.7, 2, 5]                    # g of label 5 -> 0.7
    w, mb, _ = media.encode(v3)
    assert mb == 99 and (w[0] & 0x3FFF) == 5 and ((w[0] >> 14) & 3) == 2
    assert (w[0] >> 16) == media.float_to_half_bits(np.array([0.7], np.float32))[0]
    v4 = np.zeros((4, 2, 1, 1), np.uint8)
    v4[:, 1, 0, 0] = [1, 2, 3, 4]
    w, mb, _ = media.encode(v4)
    assert mb == 103 and w[1] == 0x04030201
    v5 = np.zeros((2, 1, 1, 1), np.int16)
    v5[:, 0, 0, 0] = [7, 9]
    w, mb, _ = media.encode(v5)
    assert mb == 104 and w[0] == (9 << 16 | 7)
    v8 = np.zeros((8, 2, 1, 1), np.uint8)
    v8[:, 1, 0, 0] = [2, 1, 10, 20, 30, 40, 50, 60]     # lower, upper, point x y z, normal x y z
    w, mb, dims = media.encode(v8)
    assert mb == 97 and dims == (2, 1, 1) and w.size == 4
    assert w[1] == (20 | 10 << 8 | 1 << 16 | 2 << 24) and w[3] == (60 | 50 << 8 | 40 << 16 | 30 << 24)
    with pytest.raises(ValueError):
        media.encode(np.zeros((3, 2, 2, 2), np.int16))


def test_seed_words_match_the_c_library(lib):
    """The per-thread seed words (mcx_host.cpp:696-700, 759-768: srand(seed)
    then rand() four times per reference thread) come from the library's own
    copy of glibc's generator: the same words as the C library's rand() for
    ordinary, zero and above-2^31 seeds."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    libc.rand.restype = ctypes.c_int
    n = 5000
    for seed in (1648335518, 0, 1, 29012392, 2**31, 2**32 - 1, 12345):
        libc.srand(seed)
        want = np.array([libc.rand() for _ in range(n)], np.uint32)
        got = np.zeros(n, np.uint32)
        lib.mcx_rand_words(seed, got.ctypes.data, n)
        assert np.array_equal(got, want), seed


def _expand_window(w, n):
    """n words of the additive generator from a 31-word window of its
    unshifted outputs: o[k] = o[k-3] + o[k-31] (mod 2^32), word = o >> 1."""
    o = [int(v) for v in w]
    for _ in range(n):
        o.append((o[-3] + o[-31]) & 0xFFFFFFFF)
    return np.array(o[31:], np.uint64).astype(np.uint32) >> 1


def test_seed_jump_ahead_matches_the_stream(lib):
    """The device seed path: 31-word windows from the host's jump-ahead
    (matrix powers mod 2^32) expand to the same words as the serial
    generator, at block starts and after long skips (a repetition's skip is
    the previous repetitions' 4 x threads words)."""
    for seed, skip, nblock, blocklen in ((1648335518, 0, 5, 300), (12345, 7, 3, 1024),
                                         (29012392, 19922944, 2, 64), (1, 2**20 + 3, 4, 97)):
        starts = np.zeros(31 * nblock, np.uint32)
        assert lib.mcx_rand_blocks(seed, skip, nblock, blocklen, starts.ctypes.data) == 0
        total = skip + nblock * blocklen
        want = np.zeros(total, np.uint32)
        lib.mcx_rand_words(seed, want.ctypes.data, total)
        for j in range(nblock):
            got = _expand_window(starts[31 * j:31 * j + 31], blocklen)
            assert np.array_equal(got, want[skip + j * blocklen:skip + (j + 1) * blocklen]), (seed, skip, j)


def _mie(lib, x, m):
    sm = np.zeros((181, 4), np.float32)
    q, g = ctypes.c_double(), ctypes.c_double()
    lib.mcx_mie.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert lib.mcx_mie(x, m, sm.ctypes.data, ctypes.byref(q), ctypes.byref(g)) == 0
    return sm, q.value, g.value


def test_mie_series_limits(lib):
    """The library's Mie series (Bohren & Huffman) in its limits: Rayleigh
    scattering for a small sphere (S11(90 deg) = S11(0)/2, -S12/S11 = 1 at 90
    deg, g ~ 0, Q_sca = 8/3 x^4 |(m^2-1)/(m^2+2)|^2) and the extinction
    paradox for a large one (Q_sca -> 2 for a weakly refracting sphere is
    approached from above, g -> 1)."""
    x, m = 0.01, 1.2
    sm, q, g = _mie(lib, x, m)
    assert abs(sm[90, 0] / sm[0, 0] - 0.5) < 1e-4
    assert abs(-sm[90, 1] / sm[90, 0] - 1) < 1e-4
    assert abs(g) < 1e-4
    ray = 8.0 / 3.0 * x ** 4 * ((m * m - 1) / (m * m + 2)) ** 2
    assert abs(q / ray - 1) < 1e-3
    sm, q, g = _mie(lib, 200.0, 1.33)
    assert 1.9 < q < 2.3 and g > 0.8


def test_mie_matches_the_reference_routine(lib, oracle_mod):
    """Against the reference's own Mie routine (src/mcx_mie.cpp, compiled into
    the oracle's reference harness when the reference sources are present):
    the same Mueller rows to float rounding for size parameters from 0.5 up
    (below 0.1 the reference switches to a small-sphere expansion whose S2
    groups the quadrupole term with the wrong angular factor)."""
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference harness not built (reference sources absent)")
    for x, m in ((0.5, 1.2), (2.0, 1.05), (6.96, 1.59 / 1.33), (30.0, 1.05), (80.0, 1.2)):
        a, qa, ga = O.ref_mie(x, m)
        b, qb, gb = _mie(lib, x, m)
        assert abs(qa / qb - 1) < 1e-6 and abs(ga - gb) < 1e-6
        assert np.all(np.abs(a - b) <= 5e-6 * np.abs(a[:, :1]) + 1e-30), (x, m)


@pytest.mark.timeout(120)
def test_run_lock_released_on_error_paths(lib):
    """Without a usable device, run() fails in library mode; the lock that
    serialises runs across host threads is released on that path (a second
    call, and one from another thread, fail the same way instead of
    waiting)."""
    import threading

    import mcxcl_gb300
    if mcxcl_gb300.gpuinfo():
        pytest.skip("a device is visible: the error path is not taken")
    cfg = dict(nphoton=1000, vol=np.ones((4, 4, 4), np.uint8), prop=[[0, 0, 1, 1], [0.01, 1, 0.5, 1.37]],
               srcpos=[2, 2, 0], srcdir=[0, 0, 1], tstart=0, tend=5e-9, tstep=5e-9)
    errors = []

    def call():
        try:
            mcxcl_gb300.run(cfg)
        except mcxcl_gb300.MCXError as e:
            errors.append(str(e))
    call()
    t = threading.Thread(target=call)
    t.start()
    t.join(60)
    assert not t.is_alive() and len(errors) == 2


def test_label_bytes_to_words_x_fastest(lib):
    """mcx_labels_u8 (the Python module's uint8 volume conversion) gives the
    Config's x-fastest uint32 words from a C- or Fortran-ordered byte volume,
    for shapes that are not multiples of its 32 x 32 tiles, and media.encode
    agrees with numpy's own transpose-and-widen."""
    from mcxcl_gb300 import media
    rng = np.random.default_rng(11)
    for shape in [(1, 1, 1), (33, 1, 65), (7, 40, 3), (64, 31, 33), (60, 60, 60)]:
        vol = (rng.random(shape) * 255).astype(np.uint8)
        want = np.empty(vol.size, np.uint32)
        want.reshape(vol.shape[::-1])[...] = vol.T
        for order, c in (("C", 1), ("F", 0)):
            v = np.asarray(vol, order=order)
            got = np.zeros(vol.size, np.uint32)
            lib.mcx_labels_u8(v.ctypes.data, shape[0], shape[1], shape[2], c, got.ctypes.data)
            assert np.array_equal(got, want), (shape, order)
            w, mb, dims = media.encode(v)
            assert np.array_equal(w, want) and mb == 1 and tuple(dims) == shape


def test_label_scan_finds_an_out_of_range_label_anywhere(lib):
    """The label check scans eight voxels at a time plus a remainder: a label
    past the property table is found in the first voxel, inside a group of
    eight and in the remainder, and a volume of valid labels passes."""
    from mcxcl_gb300 import _lib, pmcxcl
    prop = [[0, 0, 1, 1], [0.1, 1, 0, 1], [0.2, 1, 0, 1]]
    for n, bad in ((13, 0), (13, 5), (13, 12), (16, 15), (3, 2)):
        vol = np.ones((n, 1, 1), np.uint8)
        vol[bad, 0, 0] = 3
        C = _lib.Config()
        pmcxcl.parse_config({"nphoton": 10, "vol": vol, "prop": prop, "srcpos": [0, 0, 0], "srcdir": [1, 0, 0],
                             "issrcfrom0": 1}, C)
        lib.mcx_validatecfg(ctypes.byref(C), None, None, 0)
        assert C.errorcode != 0 and b"less than the labels" in C.errormsg, (n, bad)
        lib.mcx_clearcfg(ctypes.byref(C))
    C = _lib.Config()
    pmcxcl.parse_config({"nphoton": 10, "vol": np.full((13, 1, 1), 2, np.uint8), "prop": prop, "srcpos": [0, 0, 0],
                         "srcdir": [1, 0, 0], "issrcfrom0": 1}, C)
    lib.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    assert C.errorcode == 0, C.errormsg
    lib.mcx_clearcfg(ctypes.byref(C))
