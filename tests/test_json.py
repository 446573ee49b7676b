"""JSON input (mcx_readconfig / mcx_parsejson) against the dict interface and
the reference's shape semantics.

The inputs are the reference's own built-in benchmark files
(tests/golden/bench_*.json, extracted from src/mcx_bench.h by
tests/golden/make_json_fixtures.py).  A JSON input and the equivalent
pmcxcl dictionary must give the same validated Config; the shape tags must
label the voxels the reference's rasterisers label (src/mcx_shapes.c, restated
below in numpy); a malformed input is an error, not a crash.  The GPU test
runs cube60 from its JSON file through mcx_run_simulation and lands in the
reference's own known-answer band (test/testmcx.sh:61, 65).
"""
import ctypes
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _lib():
    from mcxcl_gb300 import _lib
    return _lib, _lib.load()


def _from_json(src, standalone=False):
    """A validated Config from a JSON file name or text; (Config, error)."""
    _l, L = _lib()
    C = _l.Config()
    L.mcx_initcfg(ctypes.byref(C))
    C.parentid = _l.mpPython
    C.flog = None
    if src.lstrip()[:1] in ("{", "["):
        L.mcx_parsejson(src.encode(), ctypes.byref(C))       # JSON text
    else:
        L.mcx_readconfig(src.encode(), ctypes.byref(C))      # a .json file
    return C, (C.errorcode, C.errormsg.decode())


def _from_dict(cfg):
    from mcxcl_gb300 import pmcxcl
    _l, L = _lib()
    C = _l.Config()
    pmcxcl.parse_config(cfg, C)
    L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    pmcxcl._check(C)
    return C


def _vol(C):
    n = C.dim.x * C.dim.y * C.dim.z
    v = np.ctypeslib.as_array(C.vol, shape=(n,)).copy()
    return v.reshape((C.dim.x, C.dim.y, C.dim.z), order="F")


def _f4(p, n):
    """n records of four floats (float4 or Medium) as an array."""
    return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)), shape=(4 * n,)).reshape(n, 4).copy()


def _clear(*cs):
    _l, L = _lib()
    for C in cs:
        L.mcx_clearcfg(ctypes.byref(C))


def _golden(name):
    return os.path.join(GOLDEN, "bench_%s.json" % name)


@pytest.mark.parametrize("name", ["cube60", "cube60b", "cube60planar", "cubesph60b"])
def test_json_matches_dict_interface(name):
    """The reference's benchmark file and the same benchmark as a pmcxcl
    dictionary give the same validated Config."""
    from mcxcl_gb300 import workloads
    J, (rc, msg) = _from_json(_golden(name))
    assert rc == 0, msg
    D = _from_dict(workloads.builtin(name))
    try:
        for f in ("nphoton", "seed", "medianum", "detnum", "issrcfrom0", "isreflect", "srctype",
                  "issavedet", "issave2pt", "isnormalized", "outputtype", "mediabyte", "extrasrclen"):
            assert getattr(J, f) == getattr(D, f), f
        for f in ("tstart", "tend", "tstep", "unitinmm", "minenergy"):
            assert getattr(J, f) == pytest.approx(getattr(D, f), rel=1e-7), f
        assert (J.dim.x, J.dim.y, J.dim.z) == (D.dim.x, D.dim.y, D.dim.z)
        for f in ("srcpos", "srcdir", "srcparam1", "srcparam2"):
            a, b = getattr(J, f), getattr(D, f)
            assert (a.x, a.y, a.z, a.w) == (b.x, b.y, b.z, b.w), f
        np.testing.assert_array_equal(_f4(J.prop, J.medianum), _f4(D.prop, D.medianum))
        np.testing.assert_array_equal(_f4(J.detpos, J.detnum), _f4(D.detpos, D.detnum))
        # label words after validation, detector-mask bits included
        np.testing.assert_array_equal(_vol(J), _vol(D))
        assert J.session.decode() == name
    finally:
        _clear(J, D)


def _raster_reference(shapes, dim, orig):
    """numpy restatement of the reference's shape rasterisers
    (src/mcx_shapes.c:234-838), for the test only."""
    vol = np.ones(dim, np.uint32)
    c = [np.arange(n, dtype=np.float32) + np.float32(0.5) for n in dim]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    I, J, K = np.meshgrid(*[np.arange(n) for n in dim], indexing="ij")
    orig = np.asarray(orig, np.float32)
    for item in shapes:
        (tag, obj), = item.items()
        if tag == "Grid":
            dim = tuple(int(v) for v in obj["Size"])
            vol = np.full(dim, obj.get("Tag", 0), np.uint32)
        elif tag == "Sphere":
            o = np.asarray(obj["O"], np.float32)
            r = np.float32(obj["R"])
            vol[(X - o[0]) ** 2 + (Y - o[1]) ** 2 + (Z - o[2]) ** 2 <= r * r] = obj.get("Tag", 0)
        elif tag == "Box":
            o = np.asarray(obj["O"], np.float32) - orig
            s = np.asarray(obj["Size"], np.float32)
            m = np.ones(dim, bool)
            for ax, A in enumerate((X, Y, Z)):
                m &= (A >= o[ax]) & (A <= o[ax] + s[ax])
            vol[m] = obj.get("Tag", 0)
        elif tag == "Subgrid":
            o = (np.asarray(obj["O"]) - 1 - orig).astype(int)
            s = np.asarray(obj["Size"], int)
            m = np.ones(dim, bool)
            for ax, A in enumerate((I, J, K)):
                m &= (A >= o[ax]) & (A <= o[ax] + s[ax])
            vol[m] = obj.get("Tag", 0)
        elif tag == "Cylinder":
            c0 = np.asarray(obj["C0"], np.float32) - orig
            c1 = np.asarray(obj["C1"], np.float32) - orig
            ax = c1 - c0
            d0 = np.float32(np.sqrt(np.sum(ax * ax)))
            ax = ax / d0
            dx, dy, dz = X - c0[0], Y - c0[1], Z - c0[2]
            along = ax[0] * dx + ax[1] * dy + ax[2] * dz
            m = (along <= d0) & (along >= 0) & (dx * dx + dy * dy + dz * dz - along * along <= np.float32(obj["R"]) ** 2)
            vol[m] = obj.get("Tag", 0)
        elif tag in ("XLayers", "YLayers", "ZLayers"):
            ax = "XYZ".index(tag[0])
            rows = [obj] if not isinstance(obj[0], list) else obj
            A = (I, J, K)[ax]
            for lo, hi, t in rows:
                lo, hi = max(lo, 1) - 1, min(hi, dim[ax])
                vol[(A >= lo) & (A < hi)] = t
        elif tag in ("XSlabs", "YSlabs", "ZSlabs"):
            ax = "XYZ".index(tag[0])
            b = obj["Bound"]
            rows = [b] if not isinstance(b[0], list) else b
            A = (I, J, K)[ax]
            for lo, hi in rows:
                lo, hi = int(max(lo - 0.5, 0)), int(min(hi, dim[ax]))
                vol[(A >= lo) & (A < hi)] = obj.get("Tag", 0)
        elif tag == "UpperSpace":
            cf = np.asarray(obj["Coef"], np.float32)
            vol[cf[0] * X + cf[1] * Y + cf[2] * Z > cf[3]] = obj.get("Tag", 0)
    return vol


@pytest.mark.parametrize("name", ["onecube", "twocube"])
def test_json_inline_jdata_volume(name):
    """A volume given inline as a JData array (the onecube / twocube
    benchmarks) in place of the Shapes list."""
    import json
    spec = json.load(open(_golden(name)))
    J, (rc, msg) = _from_json(_golden(name))
    try:
        assert rc == 0, msg
        shape = tuple(spec["Shapes"]["_ArraySize_"])
        want = np.asarray(spec["Shapes"]["_ArrayData_"], np.uint32).reshape(shape)   # row-major
        np.testing.assert_array_equal(_vol(J) & 0x7FFFFFFF, want)
    finally:
        _clear(J)


@pytest.mark.parametrize("name", ["cubesph60b", "skinvessel", "sphshells", "spherebox"])
def test_json_shapes_match_reference_rasterisers(name):
    import json
    spec = json.load(open(_golden(name)))
    J, (rc, msg) = _from_json(_golden(name))
    assert rc == 0, msg
    try:
        dom = spec["Domain"]
        origin = [0, 0, 0] if dom.get("OriginType", 0) else [1, 1, 1]
        for item in spec["Shapes"]:
            if "Origin" in item:
                origin = item["Origin"]
        dim = tuple(dom.get("Dim", (0, 0, 0)))
        want = _raster_reference(spec["Shapes"], dim, origin)
        got = _vol(J) & 0x7FFFFFFF
        assert got.shape == want.shape
        np.testing.assert_array_equal(got, want)
        assert len(np.unique(got)) >= 2
    finally:
        _clear(J)


def test_json_inline_text_and_flat_keys():
    """JSON text (mcx_parsejson, and mcx_readconfig given text that starts
    with '{'), keys as dotted full names at the root, the flag strings and
    the output type letter."""
    text = ('{"Session.Photons": 1000, "Session": {"RNGSeed": 7, "DoMismatch": true, "SaveDataMask": "dspx",'
            ' "OutputType": "f", "DebugFlag": "M"}, "Forward": {"T0": 0, "T1": 2e-9, "Dt": 1e-9},'
            ' "Domain": {"Dim": [10, 12, 14], "OriginType": 1, "Media": [[0,0,1,1],[0.01,1,0.9,1.37],[0.02,2,0.9,1.37]]},'
            ' "Optode": {"Source": {"Type": "Cone", "Pos": [5,6,0], "Dir": [0,0,1,"_NaN_"], "Param1": [0.3]},'
            ' "Detector": [{"Pos": [5, 2, 0], "R": 1.5}, [5, 9, 0, 2]]},'
            ' "Shapes": [{"Grid": {"Tag": 1, "Size": [10, 12, 14]}}, {"ZLayers": [8, 14, 2]}]}')
    J, (rc, msg) = _from_json(text)
    try:
        assert rc == 0, msg
        assert J.nphoton == 1000 and J.seed == 7 and J.isreflect == b"\x01"
        assert J.savedetflag == 0b10111          # D S P X
        assert ord(J.outputtype) == 1 and J.debuglevel == 2
        assert ord(J.srctype) == 2 and np.isnan(J.srcdir.w) and J.srcparam1.x == pytest.approx(0.3)
        assert J.maxgate == 2 and J.detnum == 2
        np.testing.assert_array_equal(_f4(J.detpos, 2), np.float32([[5, 2, 0, 1.5], [5, 9, 0, 2]]))
        v = _vol(J) & 0x7FFFFFFF
        assert v.shape == (10, 12, 14) and np.all(v[:, :, 7:] == 2) and np.all(v[:, :, :7] == 1)
        _l, L = _lib()
        R = _l.Config()
        L.mcx_initcfg(ctypes.byref(R))
        R.parentid = _l.mpPython
        R.flog = None
        L.mcx_readconfig(text.encode(), ctypes.byref(R))
        assert R.errorcode == 0 and R.nphoton == 1000
        np.testing.assert_array_equal(_vol(R), _vol(J))
        _clear(R)
    finally:
        _clear(J)


def test_json_volume_file(tmp_path):
    """Domain.VolumeFile: a binary label volume, x fastest."""
    vol = np.ones((8, 9, 10), np.uint8)
    vol[2:5, 3:7, 4:9] = 2
    f = tmp_path / "vol.bin"
    vol.ravel(order="F").tofile(f)
    text = ('{"Session": {"Photons": 10}, "Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9},'
            ' "Domain": {"Dim": [8, 9, 10], "OriginType": 1, "MediaFormat": "byte", "VolumeFile": "%s",'
            ' "Media": [[0,0,1,1],[0.01,1,0.9,1.37],[0.02,2,0.9,1.37]]},'
            ' "Optode": {"Source": {"Pos": [4, 4, 0], "Dir": [0, 0, 1]}}}' % f)
    J, (rc, msg) = _from_json(text)
    try:
        assert rc == 0, msg
        np.testing.assert_array_equal(_vol(J) & 0x7FFFFFFF, vol)
    finally:
        _clear(J)


@pytest.mark.parametrize("text,needle", [
    ('{"Session": {"Photons": 10', "invalid JSON input"),
    ('{"Session": {"Photons": 10}} trailing', "invalid JSON input"),
    ('[1, 2]', "must be an object"),
    ('{"Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9}, "Domain": {"Dim": [4,4,4], "Media": [[0,0,1,1]]},'
     ' "Shapes": [{"Torus": {"Tag": 1}}]}', "undefined tag"),
    ('{"Forward": {"T0": 0, "T1": 1e-9, "Dt": 0}, "Domain": {"Dim": [4,4,4]}, "Shapes": []}', "time gate"),
    ('{"Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9}, "Domain": {"Dim": [4,4,4], "VolumeFile": "x.bin"},'
     ' "Shapes": [{"Grid": {"Tag": 1, "Size": [4,4,4]}}]}', "both Domain.VolumeFile and Shapes"),
    ('{"Forward": {"T0": 0, "T1": 1e-9, "Dt": 1e-9}, "Domain": {"Dim": [4,4,4], "Media": [{"mua": 0}]},'
     ' "Shapes": []}', "scattering coeff"),
])
def test_json_errors_are_reported(text, needle):
    J, (rc, msg) = _from_json(text)
    try:
        assert rc != 0 and needle in msg, (rc, msg)
    finally:
        _clear(J)


def test_json_missing_file_is_an_error(tmp_path):
    J, (rc, msg) = _from_json(str(tmp_path / "none.json"))
    _clear(J)
    assert rc != 0 and "can not load" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("name,lo,hi", [("cube60", 0.17, 0.18), ("cube60b", 0.27, 0.28)])
def test_json_benchmark_runs_in_reference_band(name, lo, hi):
    """The reference's cube60 / cube60b input files through mcx_readconfig and
    mcx_run_simulation: absorbed 17.x % / 27.x % (test/testmcx.sh:61, 65)."""
    _l, L = _lib()
    J, (rc, msg) = _from_json(_golden(name))
    try:
        assert rc == 0, msg
        L.mcx_run_simulation(ctypes.byref(J), None, None)
        assert J.errorcode == 0, J.errormsg
        absorbed = (J.energytot - J.energyesc) / J.energytot
        assert lo <= absorbed < hi, absorbed
        assert abs(J.energytot - 1e6) <= 10
        assert J.detectedcount > 0
    finally:
        _clear(J)
