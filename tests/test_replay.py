"""Photon replay (the reference's cfg.seed = seed array + cfg.detphotons):
re-launching detected photons from their saved RNG states and depositing
the replay outputs -- Jacobian (wl), scattering counts (nscat / wp),
momentum transfer (wm), and their time-of-flight weighted forms.

* The oracle's replay reproduces the reference kernel's replay bit for bit
  (digests in golden/ref_pins.json, made by replaying the reference's own
  baseline records).
* The C host's replay initialisation (mcx_replayinit, src/mcx_utils.c:
  1355-1421) gives the oracle's weights, times of flight and detector ids.
* On the GPU, the exact kernel replays to the oracle's bits; the fast kernel
  re-detects every replayed photon and lands in the reference's absorbed
  band (test/testmcx.sh:120-128).
"""
import ctypes
import hashlib
import json
import os
import platform

import numpy as np
import pytest

import cases

HERE = os.path.dirname(os.path.abspath(__file__))
PINS = json.load(open(os.path.join(HERE, "golden", "ref_pins.json")))


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _baseline(O, nthread=128, **kw):
    base = cases.small_two_media(**kw)
    b = O.run(base, nthread=nthread, core=nthread, mathmode=O.MATH_LIBM, variant=O.VARIANT_NVCC,
              fieldmode=O.FIELD_FLOAT_SPILL)
    return base, b


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"),
                    reason="libm-mode digests were recorded with x86-64 glibc")
@pytest.mark.parametrize("name,bkw,rkw,nthread", cases.REPLAY_PINS, ids=[c[0] for c in cases.REPLAY_PINS])
def test_oracle_replay_matches_reference_bits(oracle_mod, name, bkw, rkw, nthread):
    O = oracle_mod
    pin = PINS[name]
    base, b = _baseline(O, **bkw)
    cfg = cases.replay_cfg(base, b["detp"], b["seeds"], **rkw)
    r = O.run(cfg, nthread=nthread, core=nthread, mathmode=O.MATH_LIBM, variant=O.VARIANT_NVCC,
              fieldmode=O.FIELD_FLOAT_SPILL)
    assert _sha(np.asarray(r["energy"], np.float32).view(np.uint32)) == pin["energy_sha"]
    field = np.asarray(r["field_raw"], np.float32)
    assert _sha(np.asfortranarray(field).ravel(order="F").view(np.uint32)) == pin["field_sha"]
    assert r["detp"].shape[1] == pin["ndet"]
    assert _sha(np.asarray(r["detp"], np.float32).view(np.uint32)) == pin["detp_sha"]


def test_replay_redetects_every_photon_in_the_oracle(oracle_mod):
    """A replayed photon follows its baseline path to the same detector."""
    O = oracle_mod
    base, b = _baseline(O, nphoton=3000)
    cfg = cases.replay_cfg(base, b["detp"], b["seeds"], outputtype="jacobian")
    r = O.run(cfg, nthread=128, core=128, mathmode=O.MATH_LIBM, variant=O.VARIANT_NVCC)
    assert r["stat"]["detected"] == b["detp"].shape[1]
    np.testing.assert_array_equal(np.sort(r["detp"][0]), np.sort(b["detp"][0]))


def _host_replay(cfg):
    """Run the product's parse + mcx_validatecfg (no GPU needed) and read the
    replay arrays it prepared."""
    from mcxcl_gb300 import _lib, pmcxcl
    L = _lib.load()
    C = _lib.Config()
    try:
        pmcxcl.parse_config(cfg, C)
        recs = pmcxcl._detphotons(cfg)
        dims = (ctypes.c_int * 2)(recs.shape[1], recs.shape[0])
        L.mcx_validatecfg(ctypes.byref(C), recs.ctypes.data_as(ctypes.c_void_p), dims, 16)
        if C.errorcode:
            raise pmcxcl.MCXError(C.errormsg.decode())
        n = int(C.nphoton)
        w = np.ctypeslib.as_array(C.replay.weight, shape=(max(n, 1),))[:n].copy()
        t = np.ctypeslib.as_array(C.replay.tof, shape=(max(n, 1),))[:n].copy()
        d = np.ctypeslib.as_array(C.replay.detid, shape=(max(n, 1),))[:n].copy()
        s = np.ctypeslib.as_array(ctypes.cast(C.replay.seed, ctypes.POINTER(ctypes.c_uint64)),
                                  shape=(max(2 * n, 2),))[:2 * n].copy().reshape(n, 2)
        return n, w, t, d, s, C.replaydet
    finally:
        L.mcx_clearcfg(ctypes.byref(C))


@pytest.mark.parametrize("rkw", [dict(), dict(replaydet=-1), dict(replaydet=2), dict(unitinmm=0.5),
                                 dict(tend=2e-9)], ids=["all", "perdet", "det2", "unitinmm", "window"])
def test_host_replayinit_matches_oracle(oracle_mod, rkw):
    O = oracle_mod
    base, b = _baseline(O, nphoton=3000)
    cfg = cases.replay_cfg(base, b["detp"], b["seeds"], outputtype="jacobian", **rkw)
    n, w, t, d, s, _ = _host_replay(cfg)
    inp, keep = O.make_input(cfg, nthread=128)
    assert n == inp.nreplay
    assert np.array_equal(w.view(np.uint32), keep["rw"][:n].view(np.uint32))
    assert np.array_equal(t.view(np.uint32), keep["rtof"][:n].view(np.uint32))
    assert np.array_equal(d, keep["rdid"][:n])
    assert np.array_equal(s, keep["rseed"][:n])
    if rkw.get("replaydet", 0) > 0:
        assert np.all((d & 0xFFFF) == rkw["replaydet"])


def test_host_replay_errors(oracle_mod):
    from mcxcl_gb300 import pmcxcl
    O = oracle_mod
    base, b = _baseline(O, nphoton=3000)
    # partial paths are needed to weight the replayed photons
    with pytest.raises(pmcxcl.MCXError, match="partial-path"):
        _host_replay(cases.replay_cfg(base, b["detp"], b["seeds"], outputtype="jacobian", savedetflag="dx"))
    # a replay output without a replay
    with pytest.raises(pmcxcl.MCXError, match="reply mode"):
        from mcxcl_gb300 import _lib
        L = _lib.load()
        C = _lib.Config()
        pmcxcl.parse_config(dict(base, outputtype="jacobian"), C)
        L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
        msg = C.errormsg.decode()
        L.mcx_clearcfg(ctypes.byref(C))
        if msg:
            raise pmcxcl.MCXError(msg)
    # detector ids outside 1..detnum cannot index a per-detector output
    bad = np.array(b["detp"], copy=True)
    bad[0, 0] = 7
    with pytest.raises(pmcxcl.MCXError, match="detector id"):
        _host_replay(cases.replay_cfg(base, bad, b["seeds"], outputtype="jacobian", replaydet=-1))


# ---------------------------------------------------------------- GPU

REPLAY_GPU = [("jacobian", 0), ("jacobian", -1), ("jacobian", 1), ("nscat", 0), ("wm", -1), ("wltof", 0),
              ("wptof", 0), ("flux", 0), ("rf", 0), ("rf", -1), ("rfmus", 0)]


@pytest.fixture(scope="module")
def gpu():
    import mcxcl_gb300
    info = mcxcl_gb300.gpuinfo()
    if not info:
        pytest.fail("no CUDA device visible to the transport library")
    return info[0]


@pytest.mark.gpu
@pytest.mark.parametrize("ot,rd", REPLAY_GPU, ids=["%s_%d" % x for x in REPLAY_GPU])
@pytest.mark.parametrize("nthread", [256, 16])
def test_exact_replay_matches_oracle(gpu, oracle_mod, ot, rd, nthread):
    import mcxcl_gb300
    O = oracle_mod
    base = cases.small_two_media(nphoton=6000)
    b = O.run(base, nthread=256, core=256, mathmode=O.MATH_PMATH)
    # the rf outputs are phased at 100 MHz; the oracle's FP64 mode keeps their
    # launch phase where the deposits read it (the reference's float path, pinned
    # above, stores it elsewhere and comes out zero)
    cfg = cases.replay_cfg(base, b["detp"], b["seeds"], outputtype=ot, replaydet=rd,
                           omega=2 * np.pi * 1e8 if ot.startswith("rf") else 0.0)
    g = mcxcl_gb300.run(dict(cfg, autopilot=0, nthread=nthread, nblocksize=16, exactmath=1, savethreadenergy=1))
    r = O.run(cfg, nthread=nthread, core=gpu["core"], mathmode=O.MATH_PMATH, fieldmode=O.FIELD_DOUBLE)
    assert np.array_equal(g["threadenergy"].view(np.uint32), np.asarray(r["energy"], np.float32).view(np.uint32))
    assert g["stat"]["detected"] == r["stat"]["detected"]
    gd = np.ascontiguousarray(g["detp"].T).view(np.uint32)
    rdp = np.ascontiguousarray(r["detp"].T).view(np.uint32)
    assert np.array_equal(gd[np.lexsort(gd.T[::-1])], rdp[np.lexsort(rdp.T[::-1])])
    # the field agrees to the rounding of the accumulation order; the oracle
    # normalises as the reference host does (per detector block for replaydet -1)
    ref = np.asarray(r["flux"], np.float64).reshape(g["flux"].shape, order="F")
    scale = max(np.abs(ref).max(), 1e-30)
    np.testing.assert_allclose(g["flux"], ref, rtol=1e-4, atol=1e-6 * scale)
    assert g["stat"]["normalizer"] == pytest.approx(r["stat"]["normalizer"], rel=1e-6)


@pytest.mark.gpu
def test_fast_replay_reference_known_answer(gpu):
    """test/testmcx.sh:120-128: cube60 saved with seeds, then replayed: every
    replayed photon is detected again, and 30-38% of the replayed weight is
    absorbed."""
    import mcxcl_gb300
    base = cases.cube60(nphoton=1000000, issaveseed=1, savedetflag="dp")
    b = mcxcl_gb300.run(base)
    nd = b["detp"].shape[1]
    assert nd > 1000
    r = mcxcl_gb300.run(cases.replay_cfg(base, b["detp"], b["seeds"], outputtype="jacobian"))
    assert r["stat"]["detected"] == nd
    a = r["stat"]["energyabs"] / r["stat"]["energytot"]
    assert 0.30 <= a < 0.39, a
    assert np.all(np.isfinite(r["flux"])) and r["flux"].sum() > 0
