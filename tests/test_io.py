"""Output files: .mch (binary detected photons), _detp.jdat (JData JSON) and
.jnii (JNIfTI JSON) in the reference's layouts, written and read back."""
import ctypes
import json
import os
import struct

import numpy as np

import cases
from mcxcl_gb300 import io


def _records(O):
    cfg = cases.small_two_media(nphoton=3000)
    r = O.run(cfg, nthread=128, core=128)
    seeds8 = np.ascontiguousarray(r["seeds"]).view(np.uint8).reshape(-1, 16).T
    return cfg, r["detp"], seeds8, r


def test_mch_round_trip_and_layout(tmp_path, oracle_mod):
    cfg, detp, seeds, r = _records(oracle_mod)
    hdr = io.header(maxmedia=2, detnum=2, colcount=detp.shape[0], totalphoton=3000, detected=detp.shape[1],
                    savedphoton=detp.shape[1], seedbyte=16, normalizer=1.5, savedetflag=0x7F)
    p = tmp_path / "a.mch"
    io.save_mch(p, detp, hdr, seeds)
    raw = p.read_bytes()
    assert raw[:4] == b"MCXH" and len(raw) == 64 + detp.size * 4 + seeds.size
    assert struct.unpack_from("<I", raw, 16)[0] == detp.shape[0]          # colcount
    d2, s2, h2 = io.load_mch(p)
    assert np.array_equal(d2.view(np.uint32), detp.view(np.uint32))
    assert np.array_equal(s2, seeds)
    assert h2["normalizer"] == 1.5 and h2["savedetflag"] == 0x7F
    io.save_mch(p, detp, hdr, seeds, append=True)
    d3, _, h3 = io.load_mch(p)
    assert d3.shape[1] == 2 * detp.shape[1] and h3["savedphoton"] == 2 * detp.shape[1]


def test_c_savedetphoton_writes_the_same_layout(tmp_path, oracle_mod):
    from mcxcl_gb300 import _lib, pmcxcl
    cfg, detp, seeds, r = _records(oracle_mod)
    L = _lib.load()
    C = _lib.Config()
    try:
        pmcxcl.parse_config(dict(cfg, session="cwrite"), C)
        L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
        assert not C.errorcode
        C.his.totalphoton = 3000
        C.his.detected = detp.shape[1]
        C.his.savedphoton = detp.shape[1]
        C.his.seedbyte = 16
        recs = np.ascontiguousarray(detp.T)
        sd = np.ascontiguousarray(seeds.T)
        cwd = os.getcwd()
        os.chdir(tmp_path)
        try:
            L.mcx_savedetphoton(recs.ctypes.data_as(ctypes.c_void_p), sd.ctypes.data_as(ctypes.c_void_p),
                                ctypes.c_int(detp.shape[1]), ctypes.c_int(0), ctypes.byref(C))
        finally:
            os.chdir(cwd)
        assert not C.errorcode
        d2, s2, h2 = io.load_mch(tmp_path / "cwrite.mch")
        assert np.array_equal(d2.view(np.uint32), detp.view(np.uint32))
        assert np.array_equal(s2, seeds)
        assert h2["colcount"] == detp.shape[0] and h2["maxmedia"] == 2 and h2["detnum"] == 2
        assert h2["savedetflag"] == C.savedetflag
    finally:
        L.mcx_clearcfg(ctypes.byref(C))


def test_jdet_column_groups(tmp_path, oracle_mod):
    cfg, detp, seeds, r = _records(oracle_mod)
    flag = 0x7F                                      # dspmxvw
    hdr = io.header(maxmedia=2, detnum=2, colcount=detp.shape[0], totalphoton=3000, detected=detp.shape[1],
                    savedphoton=detp.shape[1], seedbyte=16, savedetflag=flag)
    p = tmp_path / "a_detp.jdat"
    io.save_jdet(p, detp, hdr, cfg["prop"], seeds)
    cols, info = io.load_jdet(p)
    n = detp.shape[1]
    assert info["DetectedPhoton"] == n and info["Media"][1]["mus"] == 1.0
    assert cols["detid"].shape == (n, 1) and cols["detid"].dtype == np.uint32
    assert np.array_equal(cols["detid"][:, 0], detp[0].astype(np.uint32))
    assert np.array_equal(cols["nscat"], detp[1:3].T.astype(np.uint32))
    assert np.array_equal(cols["ppath"], detp[3:5].T)
    assert np.array_equal(cols["p"], detp[7:10].T)
    assert np.array_equal(cols["w0"][:, 0], detp[13])
    assert np.array_equal(cols["seed"], seeds.T)
    doc = json.load(open(p))
    assert doc["MCXData"]["PhotonData"]["ppath"]["_ArrayZipType_"] == "zlib"


def test_jnii_round_trip(tmp_path):
    v = np.random.default_rng(1).random((7, 5, 3, 4)).astype(np.float32)
    p = tmp_path / "f.jnii"
    io.save_jnii(p, v, voxelsize=(0.5, 0.5, 0.5), name="f")
    w, hdr = io.load_jnii(p)
    assert np.array_equal(w, v)
    assert hdr["Dim"] == [7, 5, 3, 4] and hdr["VoxelSize"][:3] == [0.5, 0.5, 0.5]
    doc = json.load(open(p))
    assert doc["NIFTIData"]["_ArrayOrder_"] == "c"
