"""The host-side formats pinned to the reference's own code.

tests/golden/ref_host_pins.json holds what the reference's configuration
layer and writers produce, run from the reference sources by
tests/golden/make_host_pins.py:

* the configuration its mcx_readconfig loads from each built-in benchmark
  input (src/mcx_utils.c:2011-2071, 2401-3287, shapes src/mcx_shapes.c,
  preprocessing and detector mask 1521-1809, 4085-4198): this library's
  mcx_readconfig must load the same scalars, volume words (labels and
  detector-mask bits), media, detectors and sources;
* the .mch file of mcx_savedetphoton (src/mcx_utils.c:963-998): the same
  bytes from the C writer and from mcxcl_gb300.io;
* the .jdat (mcx_savejdet, 1010-1190) and .jnii (mcx_savejnii, 761-884)
  documents: the same header values and the same decoded arrays (the JSON
  text itself is formatted differently);
* the adjoint post-kernels (mcx_adjoint_kernel, mcx_adjoint_dcoeff_kernel,
  src/mcx_core.cl:3393-3512) on seeded fields: the float32 restatement the
  GPU kernels follow reproduces their bits here, and the GPU kernels
  themselves reproduce them on the GPU (test marked gpu).
"""
import base64
import ctypes
import hashlib
import json
import os
import zlib

import numpy as np
import pytest

from mcxcl_gb300 import io

HERE = os.path.dirname(os.path.abspath(__file__))
PINS = json.load(open(os.path.join(HERE, "golden", "ref_host_pins.json")))
SCALARS = ["medianum", "detnum", "maxgate", "srcnum", "extrasrclen", "savedetflag", "debuglevel", "maxdetphoton",
           "srctype", "seed", "isreflect", "issavedet", "issave2pt", "isnormalized", "outputtype", "mediabyte",
           "issrcfrom0", "issaveseed", "issaveexit", "issaveref", "ismomentum", "isspecular", "autopilot",
           "srcid", "nphoton", "tstart", "tstep", "tend", "unitinmm", "minenergy"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _arr(ptr, n, dtype=ctypes.c_float):
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(dtype)), shape=(n,)).copy()


@pytest.mark.parametrize("name", sorted(PINS["json"]))
def test_json_reader_loads_what_the_reference_loads(name):
    from mcxcl_gb300 import _lib
    L = _lib.load()
    want = PINS["json"][name]
    C = _lib.Config()
    L.mcx_initcfg(ctypes.byref(C))
    C.parentid = _lib.mpPython
    C.flog = None
    try:
        L.mcx_readconfig(os.path.join(HERE, "golden", "bench_%s.json" % name).encode(), ctypes.byref(C))
        assert C.errorcode == 0, C.errormsg
        for k in SCALARS:
            v = getattr(C, k)
            v = ord(v) if isinstance(v, bytes) else v
            w = want["scalars"][k]
            if isinstance(w, float):
                assert np.float32(v) == np.float32(w), k
            else:
                assert int(v) == w, k
        assert [C.dim.x, C.dim.y, C.dim.z] == want["dim"]
        n = C.dim.x * C.dim.y * C.dim.z
        vol = _arr(C.vol, n, ctypes.c_uint32)
        assert _sha(vol) == want["vol_sha"], (np.unique(vol), want["labels"], int((vol >> 31).sum()), want["masked"])
        assert _sha(_arr(C.prop, 4 * C.medianum).reshape(-1, 4)) == want["prop_sha"]
        det = _arr(C.detpos, 4 * C.detnum).reshape(-1, 4) if C.detnum else np.zeros((0, 4), np.float32)
        assert _sha(det) == want["detpos_sha"]
        for k in ("srcpos", "srcparam1", "srcparam2"):
            v = getattr(C, k)
            assert np.array_equal(np.float32([v.x, v.y, v.z, v.w]), np.float32(want[k])), k
        d = C.srcdir
        assert np.array_equal(np.float32([d.x, d.y, d.z, d.w]), np.float32(want["srcdir"]), equal_nan=True)
    finally:
        L.mcx_clearcfg(ctypes.byref(C))


def _writer_inputs():
    w = PINS["writers"]
    detp = np.asarray(w["detp"], np.float32)            # [n, colcount]
    seeds = np.asarray(w["seeds"], np.uint8)            # [n, 16]
    h = w["hist"]
    hdr = io.header(maxmedia=h[1], detnum=h[2], colcount=h[3], totalphoton=h[4], detected=h[5], savedphoton=h[6],
                    unitinmm=w["histf"][0], seedbyte=h[7], normalizer=w["histf"][1], respin=h[8], srcnum=h[9],
                    savedetflag=h[10], totalsource=h[11])
    return w, detp, seeds, hdr


def test_mch_bytes_match_the_reference_writer(tmp_path):
    """The C writer (mcx_savedetphoton) and mcxcl_gb300.io.save_mch give the
    reference writer's exact bytes for the same header, records and seeds."""
    from mcxcl_gb300 import _lib
    L = _lib.load()
    w, detp, seeds, hdr = _writer_inputs()
    p = tmp_path / "py.mch"
    io.save_mch(p, detp.T, hdr, seeds.T)
    raw = p.read_bytes()
    assert len(raw) == w["mch_size"] and hashlib.sha256(raw).hexdigest() == w["mch_sha"]
    C = _lib.Config()
    L.mcx_initcfg(ctypes.byref(C))
    C.parentid = _lib.mpPython
    C.flog = None
    try:
        C.session = b"cw"
        C.issaveseed = b"\x01"
        h = w["hist"]
        for k, v in zip(("version", "maxmedia", "detnum", "colcount", "totalphoton", "detected", "savedphoton",
                         "seedbyte", "respin", "srcnum", "savedetflag", "totalsource"), h):
            setattr(C.his, k, v)
        C.his.unitinmm, C.his.normalizer = w["histf"]
        cwd = os.getcwd()
        os.chdir(tmp_path)
        try:
            L.mcx_savedetphoton(detp.ctypes.data_as(ctypes.c_void_p), seeds.ctypes.data_as(ctypes.c_void_p),
                                ctypes.c_int(detp.shape[0]), ctypes.c_int(0), ctypes.byref(C))
        finally:
            os.chdir(cwd)
        assert C.errorcode == 0
        assert hashlib.sha256((tmp_path / "cw.mch").read_bytes()).hexdigest() == w["mch_sha"]
    finally:
        L.mcx_clearcfg(ctypes.byref(C))


def _same_json_values(a, b, path=""):
    """Equal structure; numbers equal (floats as the float32 they hold)."""
    if isinstance(b, dict):
        assert isinstance(a, dict) and sorted(a) == sorted(b), (path, sorted(a), sorted(b))
        for k in b:
            _same_json_values(a[k], b[k], path + "." + k)
    elif isinstance(b, list):
        assert isinstance(a, list) and len(a) == len(b), path
        for i, (x, y) in enumerate(zip(a, b)):
            _same_json_values(x, y, "%s[%d]" % (path, i))
    elif isinstance(b, (int, float)) and not isinstance(b, bool):
        assert np.float32(a) == np.float32(b), (path, a, b)
    else:
        assert a == b, (path, a, b)


def test_jdat_matches_the_reference_writer(tmp_path):
    """Info values and every PhotonData column group decode to the same
    arrays (types, shapes, bits) as the reference's .jdat."""
    w, detp, seeds, hdr = _writer_inputs()
    p = tmp_path / "py_detp.jdat"
    io.save_jdet(p, detp.T, hdr, w["prop"], seeds.T)
    ours = json.load(open(p))["MCXData"]
    ref = w["jdat"]["MCXData"]
    _same_json_values(ours["Info"], ref["Info"], "Info")
    assert sorted(ours["PhotonData"]) == sorted(ref["PhotonData"])
    for k, obj in ref["PhotonData"].items():
        a, b = io.jdata_decode(ours["PhotonData"][k]), io.jdata_decode(obj)
        assert a.dtype == b.dtype and a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), k
        for key in ("_ArrayType_", "_ArraySize_", "_ArrayZipType_", "_ArrayZipSize_"):
            assert ours["PhotonData"][k][key] == obj[key], (k, key)


def test_jnii_matches_the_reference_writer(tmp_path):
    """NIFTIHeader values and the decoded NIFTIData of a 4-D volume are the
    reference's (session name, gate count and output type in the header)."""
    w = PINS["writers"]
    vol = np.asarray(w["vol"], np.float32).reshape(w["vol_shape"], order="F")
    p = tmp_path / "py.jnii"
    io.save_jnii(p, vol, voxelsize=(0.5, 0.5, 0.5), name="pins", outputtype=1, maxgate=3)
    ours = json.load(open(p))
    ref = w["jnii"]
    _same_json_values(ours["NIFTIHeader"], ref["NIFTIHeader"], "NIFTIHeader")
    a, b = io.jdata_decode(ours["NIFTIData"]), io.jdata_decode(ref["NIFTIData"])
    assert a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(a, vol)
    for key in ("_ArrayType_", "_ArraySize_", "_ArrayOrder_", "_ArrayZipType_", "_ArrayZipSize_"):
        assert ours["NIFTIData"][key] == ref["NIFTIData"][key], key


def _adjoint_cases():
    for c in PINS["adjoint"]:
        nx, ny, nz = c["shape"]
        raw = zlib.decompress(base64.b64decode(c["field_zlib_b64"]))
        field = np.frombuffer(raw, np.float32).reshape((nx, ny, nz, c["maxgate"], c["ns"] + c["nd"]), order="F")
        yield c, field


def test_adjoint_restatement_matches_reference_bits():
    from test_adjoint import _adjoint_ref
    for c, field in _adjoint_cases():
        for kind in (0, 1):
            out = _adjoint_ref(field, c["ns"], c["nd"], kind).astype(np.float32)
            assert _sha(out.ravel(order="F")) == c["sha%d" % kind], (c["shape"], kind)


@pytest.mark.gpu
def test_adjoint_gpu_kernels_match_reference_bits():
    """mcxg_adjoint_field (the GPU post-kernels) on the pinned fields: the
    reference's bits, for both kinds and both shapes."""
    from mcxcl_gb300 import _lib
    L = _lib.load()
    s = ctypes.c_void_p()
    assert L.mcxg_create(0, ctypes.byref(s)) == 0
    try:
        for c, field in _adjoint_cases():
            nx, ny, nz = c["shape"]
            f = np.ascontiguousarray(field.ravel(order="F"))
            for kind in (0, 1):
                out = np.zeros(nx * ny * nz * c["ns"] * c["nd"], np.float32)
                rc = L.mcxg_adjoint_field(s, kind, f.ctypes.data, c["ns"], c["nd"], nx, ny, nz, c["maxgate"],
                                          out.ctypes.data)
                assert rc == 0, L.mcxg_error_string(rc)
                assert _sha(out) == c["sha%d" % kind], (c["shape"], kind)
    finally:
        L.mcxg_destroy(s)
