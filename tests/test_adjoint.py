"""Adjoint Jacobians (outputtype 'adjoint', 'adjoint_dcoeff', 'adjoint_mus',
'adjoint_musp', 'adjoint_mua_d', 'adjoint_mua_musp'): detectors run as
sources (mcx_utils.c:1902-1926), then per voxel phi_src x phi_det or
grad phi_src . grad phi_det of the time-integrated fluences
(mcx_core.cl:3320-3512), scaled as mcx_host.cpp:1466-1642 does.

The post-kernels are checked bit for bit against a float32 restatement of
the reference kernels on the GPU's own fluence; the forward run with the
detectors as sources against the oracle."""
import ctypes

import numpy as np
import pytest

import cases

DETDIR = [[0, 0, 1, 0], [0, 0, 1, 0]]


def _cfg(**kw):
    cfg = cases.small_two_media(nphoton=20000, issavedet=0, detdir=DETDIR, **kw)
    cfg.pop("savedetflag", None)
    cfg.pop("issaveseed", None)
    return cfg


def test_detectors_become_sources(tmp_path):
    from mcxcl_gb300 import _lib, pmcxcl
    L = _lib.load()
    for from0 in (1, 0):
        C = _lib.Config()
        try:
            pmcxcl.parse_config(_cfg(outputtype="adjoint", issrcfrom0=from0), C)
            L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
            assert not C.errorcode, C.errormsg
            assert C.extrasrclen == 2 and C.srcid == -1
            for i, d in enumerate(cases.small_two_media()["detpos"]):
                e = C.srcdata[i]
                # taken before the detectors' own shift to 0-based positions, as the reference does
                assert (e.srcpos.x, e.srcpos.y, e.srcpos.z, e.srcpos.w) == (d[0], d[1], d[2], 1.0)
                assert (e.srcdir.z, e.srcparam1.x) == (1.0, d[3])
        finally:
            L.mcx_clearcfg(ctypes.byref(C))


def test_adjoint_needs_detector_directions():
    from mcxcl_gb300 import pmcxcl
    cfg = _cfg(outputtype="adjoint")
    cfg.pop("detdir")
    with pytest.raises(pmcxcl.MCXError, match="detdir"):
        pmcxcl.run(cfg)


# ---- float32 restatement of the post-kernels --------------------------------

def _cw(phi, slot):
    s = np.zeros(phi.shape[:3], np.float32)
    for t in range(phi.shape[3]):
        s = s + phi[:, :, :, t, slot]
    return s


def _grad(c, axis):
    n = c.shape[axis]
    g = np.zeros_like(c)
    if n <= 1:
        return g
    c = np.moveaxis(c, axis, 0)
    g = np.moveaxis(g, axis, 0)
    f32 = np.float32
    if n == 2:
        g[0] = c[1] - c[0]
        g[1] = c[1] - c[0]
    else:
        g[0] = ((f32(-3) * c[0] + f32(4) * c[1]) - c[2]) * f32(0.5)
        g[-1] = ((c[-3] - f32(4) * c[-2]) + f32(3) * c[-1]) * f32(0.5)
        g[1:-1] = (c[2:] - c[:-2]) * f32(0.5)
    return np.moveaxis(g, 0, axis)


def _adjoint_ref(phi, ns, nd, kind):
    out = []
    for s in range(ns):
        cs = _cw(phi, s)
        gs = [_grad(cs, a) for a in range(3)]
        for d in range(nd):
            cd = _cw(phi, ns + d)
            if kind == 0:
                out.append(cs * cd - np.float32(0))
            else:
                gd = [_grad(cd, a) for a in range(3)]
                out.append((gs[0] * gd[0] + gs[1] * gd[1]) + gs[2] * gd[2])
    return np.stack(out, axis=3)


@pytest.mark.gpu
@pytest.mark.parametrize("ot", ["adjoint", "adjoint_dcoeff", "adjoint_mus", "adjoint_musp", "adjoint_mua_d",
                                "adjoint_mua_musp"])
def test_adjoint_post_kernels_match_restatement(ot):
    import mcxcl_gb300
    cfg = _cfg(outputtype=ot, isreflect=0)
    r = mcxcl_gb300.run(cfg)
    phi = r["flux"].reshape(40, 40, 40, -1, 3, order="F")
    ns, nd = 1, 2
    f32 = np.float32
    vox = f32(1.0)
    vol = cfg["vol"]
    prop = np.asarray(cfg["prop"], np.float32)

    def opscale(form):
        mus, onemg = prop[vol, 1], f32(1) - prop[vol, 2]
        if form == 1:
            return f32(1) / (f32(3) * onemg * mus * mus)
        return f32(1) / (f32(3) * onemg * onemg * mus * mus)
    mua = _adjoint_ref(phi, ns, nd, 0) * -vox
    dco = _adjoint_ref(phi, ns, nd, 1) * -f32(1.0)
    want = {"adjoint": {"jmua": mua}, "adjoint_dcoeff": {"jd": dco},
            "adjoint_mus": {"jmus": dco * opscale(1)[..., None]},
            "adjoint_musp": {"jmusp": dco * opscale(2)[..., None]},
            "adjoint_mua_d": {"jmua": mua, "jd": dco},
            "adjoint_mua_musp": {"jmua": mua, "jmusp": dco * opscale(2)[..., None]}}[ot]
    for k, v in want.items():
        assert r[k].shape == (40, 40, 40, ns * nd)
        assert np.array_equal(r[k].view(np.uint32), v.astype(np.float32).view(np.uint32)), k


@pytest.mark.gpu
def test_adjoint_forward_matches_oracle(oracle_mod):
    """The forward part: the source and both detectors sharing photons (srcid -1)."""
    import mcxcl_gb300
    O = oracle_mod
    cfg = _cfg(outputtype="adjoint")
    g = mcxcl_gb300.run(dict(cfg, autopilot=0, nthread=256, nblocksize=64, exactmath=1, savethreadenergy=1))
    dets = cases.small_two_media()["detpos"]
    explicit = dict(cfg, srcpos=[[20, 20, 0, 1]] + [[d[0], d[1], d[2], 1] for d in dets],
                    srcdir=[[0, 0, 1, 0]] * 3, srcparam1=[[0, 0, 0, 0]] + [[d[3], 0, 0, 0] for d in dets],
                    srcid=-1, outputtype="fluence")
    explicit.pop("detdir")
    info = mcxcl_gb300.gpuinfo()[0]
    r = O.run(explicit, nthread=256, core=info["core"], mathmode=O.MATH_PMATH, fieldmode=O.FIELD_DOUBLE)
    assert np.array_equal(g["threadenergy"].view(np.uint32), np.asarray(r["energy"], np.float32).view(np.uint32))
    ref = np.asarray(r["flux"], np.float64).reshape(g["flux"].shape, order="F")
    np.testing.assert_allclose(g["flux"], ref, rtol=1e-4, atol=1e-6 * np.abs(ref).max())
