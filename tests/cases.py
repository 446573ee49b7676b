"""Named simulation inputs shared by the tests and the golden-fixture script.

Every case is a ``pmcxcl.run()``-style dict (the reference Python module's
keys, src/pmcxcl.cpp:428-1110).  Volumes are built procedurally so fixtures
only need to store results, not inputs.
"""
import numpy as np


def cube60(**kw):
    """The reference's built-in cube60 benchmark (src/mcx_bench.h:33-85)."""
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


def sphere_volume(n=60, center=(30, 30, 30), radius=15, inner=2, outer=1):
    """A cube of label `outer` with a sphere of label `inner`; a voxel is inside
    when its centre is (the rule of mcx_raster_sphere, src/mcx_shapes.c:234-293)."""
    idx = np.arange(n, dtype=np.float64) + 0.5
    x, y, z = np.meshgrid(idx, idx, idx, indexing="ij")
    d2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
    vol = np.full((n, n, n), outer, dtype=np.uint8)
    vol[d2 < radius * radius] = inner
    return vol


def cubesph60(**kw):
    """60^3 cube with a radius-15 sphere of label 2, Fresnel on, 50 gates of
    0.1 ns and four disk detectors on the z=0 face: the two-medium benchmark
    (the benchmark workload; src/mcx_bench.h:200-252 is the 1-gate original)."""
    cfg = cube60(
        vol=sphere_volume(),
        prop=[[0, 0, 1, 1], [0.005, 1.0, 0.01, 1.37], [0.002, 5.0, 0.9, 1.0]],
        isreflect=1, tstep=1e-10, nphoton=100000000,
        detpos=[[30, 20, 0, 1], [30, 40, 0, 1], [20, 30, 0, 1], [40, 30, 0, 1]],
        savedetflag="dsp", issaveseed=1,
    )
    cfg.update(kw)
    return cfg


def small_two_media(**kw):
    """40^3 cube with a 20^3 inner block of a second medium; the workhorse of
    the bit-exact pins."""
    vol = np.ones((40, 40, 40), np.uint8)
    vol[10:30, 10:30, 10:30] = 2
    cfg = dict(nphoton=2000, vol=vol, prop=[[0, 0, 1, 1], [0.01, 1, 0.5, 1.37], [0.02, 5, 0.9, 1.45]],
               srcpos=[20, 20, 0], srcdir=[0, 0, 1], issrcfrom0=1, seed=12345, tstart=0, tend=5e-9,
               tstep=2.5e-10, isreflect=1, detpos=[[20, 10, 0, 2], [10, 20, 0, 2]], savedetflag="dspmxvw",
               issaveseed=1)
    cfg.update(kw)
    return cfg


def _voidtop():
    vol = np.ones((40, 40, 40), np.uint8)
    vol[10:30, 10:30, 10:30] = 2
    vol[:, :, 39] = 0
    return vol


def _svmc_vol():
    """Split voxels (MEDIA_2LABEL_SPLIT): a radius-10 sphere of label 2 in
    label 1 whose surface voxels carry the tangent plane (normal outward, so
    the upper side is label 1), and a top layer split at z = 39.5 with
    background above (normal down: the lower side is background)."""
    n = 40
    v = np.zeros((8, n, n, n), np.uint8)
    x, y, z = np.meshgrid(np.arange(n) + 0.5, np.arange(n) + 0.5, np.arange(n) + 0.5, indexing="ij")
    c = np.array([20.0, 20.0, 20.0])
    r = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
    v[0] = np.where(r < 10, 2, 1)
    split = np.abs(r - 10) < 0.8
    nx, ny, nz = (x - c[0]) / r, (y - c[1]) / r, (z - c[2]) / r
    px, py, pz = [np.clip(q + (10 - r) * d - np.floor(q), 0, 1) for q, d in ((x, nx), (y, ny), (z, nz))]
    for k, a in enumerate((px, py, pz)):
        v[2 + k] = np.where(split, np.round(a * 255), 0).astype(np.uint8)
    for k, a in enumerate((nx, ny, nz)):
        v[5 + k] = np.where(split, np.round((a + 1) * 127.5), 0).astype(np.uint8)
    v[0] = np.where(split, 2, v[0])
    v[1] = np.where(split, 1, 0)
    top = (slice(None), slice(None), n - 1)
    v[0][top], v[1][top] = 0, 1
    v[2][top], v[3][top], v[4][top] = 128, 128, 128
    v[5][top], v[6][top], v[7][top] = 128, 128, 0
    return v


def _pattern(n, seed):
    return np.random.RandomState(seed).rand(*n).astype(np.float32)


# Variants of small_two_media covering each source type and boundary feature.
VARIANTS = {
    "pencil_gates": {},
    "isotropic": dict(srctype="isotropic", srcpos=[20, 20, 20]),
    "cone": dict(srctype="cone", srcparam1=[0.5, 0, 0, 0]),
    "gaussian": dict(srctype="gaussian", srcparam1=[3, 0, 0, 0]),
    "planar": dict(srctype="planar", srcpos=[5, 5, -5], srcparam1=[30, 0, 0, 0], srcparam2=[0, 30, 0, 0]),
    "fourier": dict(srctype="fourier", srcpos=[5, 5, 0], srcparam1=[30, 0, 0, 2], srcparam2=[0, 30, 0, 1]),
    "arcsine": dict(srctype="arcsine", srcpos=[20, 20, 20]),
    "disk": dict(srctype="disk", srcparam1=[5, 0, 0, 0]),
    "fourierx": dict(srctype="fourierx", srcpos=[5, 5, 0], srcparam1=[30, 0, 0, 30], srcparam2=[1, 2, 0.5, 0.5]),
    "fourierx2d": dict(srctype="fourierx2d", srcpos=[5, 5, 0], srcparam1=[30, 0, 0, 30],
                       srcparam2=[1, 2, 0.5, 0.5]),
    "zgaussian": dict(srctype="zgaussian", srcparam1=[0.3, 0, 0, 0]),
    "line": dict(srctype="line", srcpos=[10, 20, 20], srcparam1=[20, 0, 0, 0]),
    "slit": dict(srctype="slit", srcpos=[10, 20, 0], srcparam1=[20, 0, 0, 0]),
    "pencilarray": dict(srctype="pencilarray", srcpos=[5, 5, 0], srcparam1=[30, 0, 0, 4],
                        srcparam2=[0, 30, 0, 3]),
    "hyperboloid": dict(srctype="hyperboloid", srcparam1=[2, 10, 5, 0]),
    "ring": dict(srctype="ring", srcparam1=[5, 2, 0, 0]),
    "pattern": dict(srctype="pattern", srcpos=[5, 5, 0], srcparam1=[30, 0, 0, 4], srcparam2=[0, 30, 0, 4],
                    srcpattern=_pattern((4, 4), 1)),
    "pattern3d": dict(srctype="pattern3d", srcpos=[5, 5, 5], srcparam1=[4, 4, 4, 0],
                      srcpattern=_pattern((4, 4, 4), 2)),
    # photon sharing: one photon, srcnum patterns (srcpattern [srcnum, ...], patterns innermost);
    # a void top layer gives the escaping photons' saved-reflectance deposits
    "pattern_share": dict(srctype="pattern", srcpos=[5, 5, 0], srcparam1=[30, 0, 0, 4], srcparam2=[0, 30, 0, 4],
                          srcnum=3, srcpattern=_pattern((3, 4, 4), 4), issaveref=1, vol=_voidtop()),
    "pattern3d_share": dict(srctype="pattern3d", srcpos=[5, 5, 5], srcparam1=[4, 4, 4, 0], srcnum=2,
                            srcpattern=_pattern((2, 4, 4, 4), 5)),
    # RF forward: complex photon weights at 100 MHz (omega in rad/s), and with roulette
    "rf_forward": dict(omega=2 * np.pi * 1e8),
    "rf_roulette": dict(omega=2 * np.pi * 3e8, minenergy=0.01, outputtype="fluence"),
    # split voxels: without Fresnel, and with Fresnel at the planes (indices 1.37 / 1.45) and
    # at the voxel faces
    "svmc": dict(vol=_svmc_vol(), isreflect=0),
    "svmc_refl": dict(vol=_svmc_vol(), isreflect=1),
    # ... with a detector over the split top layer: detection in a background half follows the
    # reference's OpenCL kernel (its host-compiled kernel detects only in fully void voxels)
    "svmc_topdet": dict(vol=_svmc_vol(), isreflect=0, detpos=[[20, 20, 39, 6]], nphoton=20000),
    "focus": dict(srcdir=[0, 0, 1, 10]),
    "lambert": dict(srcdir=[0, 0, 1, -np.inf]),
    "noreflect": dict(isreflect=0),
    "cyclic": dict(bc="ccrrcc", isreflect=0),
    "facedet": dict(bc="aaaaaa001000", isreflect=0),
    "roulette": dict(minenergy=0.01),
    # edge cases: fewer photons than reference threads (every thread but the
    # first `oddphoton` runs none), and a one-voxel domain with a detector over
    # its face (the detector mask's single-voxel radius rule, mcx_utils.c:4141)
    "fewphotons": dict(nphoton=100),
    "onevoxel": dict(vol=np.ones((1, 1, 1), np.uint8), srcpos=[0.5, 0.5, 0], detpos=[[0.5, 0.5, 0, 1]],
                     nphoton=500),
    "unitinmm": dict(unitinmm=0.5),
    "gscatter": dict(gscatter=3),
    "outside_src_specular": dict(srcpos=[20, 20, -5], isspecular=1),
    "multisrc": dict(srcpos=[[20, 20, 0, 1], [10, 10, 0, 1]], srcdir=[[0, 0, 1, 0], [0, 0, 1, 0]]),
    "multisrc_id": dict(srcpos=[[20, 20, 0, 1], [10, 10, 0, 1]], srcdir=[[0, 0, 1, 0], [0, 0, 1, 0]], srcid=-1),
    "energy_out": dict(outputtype="energy"),
    "fluence_out": dict(outputtype="fluence"),
    "invcdf": dict(invcdf=(np.sign(np.linspace(-1, 1, 101)) *
                           np.abs(np.linspace(-1, 1, 101)) ** 0.7).astype(np.float32)),
    "angleinvcdf": dict(angleinvcdf=np.linspace(0, 0.3, 21).astype(np.float32)),
    # per-voxel float mua (MEDIA_MUA_FLOAT); the reference's __NVCC__ branch cannot run it
    "muafloat": dict(vol=(0.005 + 0.02 * np.random.RandomState(3).rand(1, 40, 40, 40)).astype(np.float32),
                     prop=[[0, 0, 1, 1], [0.01, 1, 0.5, 1.37]], savedetflag="dxvw"),
}
def _f2h_vol():
    r = np.random.RandomState(4)
    v = np.zeros((2, 40, 40, 40), np.float32)
    v[0] = 0.005 + 0.02 * r.rand(40, 40, 40)
    v[1] = 0.5 + 1.5 * r.rand(40, 40, 40)
    return v


def _labelhalf_vol():
    v = np.zeros((3, 40, 40, 40), np.float32)
    v[2] = 1
    v[2, 10:30, 10:30, 10:30] = 2
    v[1, 10:30, 10:30, 10:30] = 2               # replace g of label 2 ...
    v[0, 10:30, 10:30, 10:30] = 0.7             # ... by 0.7
    return v


VARIANTS.update({
    # half-precision mua/mus per voxel (MEDIA_AS_F2H)
    "asf2h": dict(vol=_f2h_vol(), prop=[[0, 0, 1, 1], [0.01, 1, 0.5, 1.37]], savedetflag="dxvw"),
    # labels with one property overridden in half precision (MEDIA_LABEL_HALF)
    "labelhalf": dict(vol=_labelhalf_vol(), savedetflag="dxvw"),
    # byte and short mixtures of property rows 1 and 2 (MEDIA_ASGN_BYTE, MEDIA_AS_SHORT)
    # (the top bit of each word is the detector flag, so the last byte/short stays below 2^7 / 2^15)
    "asgnbyte": dict(vol=(np.random.RandomState(5).randint(0, 256, (4, 40, 40, 40)) |
                          np.array([1, 0, 0, 0])[:, None, None, None]).astype(np.uint8) &
                         np.array([255, 255, 255, 127], np.uint8)[:, None, None, None],
                     savedetflag="dxvw"),
    "asshort": dict(vol=np.random.RandomState(6).randint(1, 32767, (2, 40, 40, 40)).astype(np.int16),
                    savedetflag="dxvw"),
})
NOT_PINNED = {"muafloat", "asf2h", "labelhalf", "asgnbyte", "asshort", "svmc_topdet"}
# Cases where a photon can leave the domain on the step right after a Fresnel
# reflection at the domain boundary: the reference then has lost the voxel's
# detector bit (its isdet still holds the face's boundary code, mcx_core.cl:2796,
# 3212) and does not record the photon; the oracle and the product do.  The
# pins hold the reference's records there, which must be a subset of the
# oracle's; energies and field are bit-identical.
DETECT_AFTER_REFLECT = {"onevoxel"}


def variant(name, **kw):
    cfg = small_two_media(**VARIANTS[name])
    cfg.update(kw)
    return cfg


def twod(**kw):
    cfg = small_two_media(vol=np.ones((1, 40, 40), np.uint8), srcpos=[0, 20, 0], detpos=[[0, 20, 0, 3]])
    cfg.update(kw)
    return cfg


# trajectory capture (-D M): records at photon closes, launches and scattering sites
TRAJ_PINS = [("traj", dict(nphoton=300, debuglevel="M", maxjumpdebug=100000)),
             ("traj_multisrc", dict(VARIANTS["multisrc"], nphoton=300, debuglevel="M", maxjumpdebug=100000))]


def traj_digest(traj):
    """SHA-256 of trajectory records [6, n] in a canonical order (the record
    slots come from an atomic counter)."""
    import hashlib
    t = np.ascontiguousarray(np.asarray(traj, np.float32).T).view(np.uint32)
    t = t[np.lexsort(t.T[::-1])] if t.size else t
    return hashlib.sha256(np.ascontiguousarray(t).tobytes()).hexdigest()


def pin_cases():
    """(name, cfg, nthread) triples pinned against the reference kernel."""
    out = [("cube60", cube60(nphoton=3000), 256),
           ("cube60b", cube60(nphoton=3000, isreflect=1), 256),
           ("cube60b_dspmxvw", cube60(nphoton=3000, isreflect=1, savedetflag="dspmxvw", issaveseed=1), 256),
           ("twod", twod(), 128)]
    for k in VARIANTS:
        if k not in NOT_PINNED:
            out.append((k, variant(k), 128))
    return out


def polarized(**kw):
    """small_two_media with Mie scatterers in both labels (polystyrene spheres
    of radius 0.5 and 0.3 um in water at 632.8 nm; prop's mus sets their
    density), a linearly polarised launch and the Stokes vector recorded with
    each detected photon."""
    cfg = small_two_media(
        prop=[[0, 0, 1, 1], [0.005, 1.0, 0.0, 1.33], [0.002, 2.0, 0.0, 1.33]],
        polprop=[[0.005, 0.5, 0.0, 1.59, 1.33], [0.002, 0.3, 0.0, 1.59, 1.33]],
        **{"lambda": 632.8}, srciquv=[1.0, 1.0, 0.0, 0.0], isreflect=0)
    cfg.update(kw)
    return cfg


def pol_inputs(cfg, mie):
    """The Mueller rows and the labels' properties mcx_prep_polarized derives
    (mcx_utils.c:1483-1519), in its float / double arithmetic; mie(x, m) gives
    (181 x 4 rows, qsca, g).  Returns a copy of cfg with 'smatrix' and the
    derived 'prop' for the oracle, which takes them as inputs."""
    f32 = np.float32
    prop = np.array(cfg["prop"], np.float32)
    pol = np.array(cfg["polprop"], np.float32).reshape(-1, 5)
    lam = f32(cfg["lambda"])
    rows = []
    for i, (mua, r, rho, nsph, nmed) in enumerate(pol):
        m = prop[i + 1]
        m[0] = mua
        m[3] = nmed
        x = float(f32(f32(6.28318530717959) * r * nmed)) / (float(lam) * 1e-3)
        A = float(f32(f32(3.1415926535897932) * r * r))
        sm, qsca, g = mie(x, float(f32(nsph / nmed)))
        if m[1] > f32(1e-10):
            target = f32(m[1])
            if m[2] < f32(1.0) - f32(1e-10):
                musp = f32(m[1] * (f32(1.0) - m[2]))
                target = f32(float(musp) / (1.0 - g))
            rho = f32(float(target) / qsca / A * 1e-3)
        m[1] = f32(qsca * A * float(rho) * 1e3)
        m[2] = f32(g)
        rows.append(np.asarray(sm, np.float32).reshape(181, 4))
    out = dict(cfg)
    out["prop"] = prop
    out["smatrix"] = np.stack(rows)
    return out


def replay_cfg(base, detp, seeds, **kw):
    """A replay of base's detected photons: detp [reclen, N] records and
    seeds [N, 2] uint64 (or [16, N] uint8) from a baseline run."""
    s = np.asarray(seeds)
    if s.dtype != np.uint8:
        s = np.ascontiguousarray(s, dtype=np.uint64).view(np.uint8).reshape(-1, 16).T
    cfg = dict(base, seed=np.asfortranarray(s), detphotons=np.asarray(detp, np.float32))
    cfg.pop("nphoton", None)
    cfg.update(kw)
    return cfg


# (name, baseline, replay keys, reference threads) -- replays pinned against the reference kernel
REPLAY_PINS = [
    ("replay_jacobian", dict(nphoton=3000), dict(outputtype="jacobian"), 128),
    ("replay_jacobian_perdet", dict(nphoton=3000), dict(outputtype="jacobian", replaydet=-1), 128),
    ("replay_jacobian_det1", dict(nphoton=3000), dict(outputtype="jacobian", replaydet=1), 128),
    ("replay_jacobian_fewthreads", dict(nphoton=3000), dict(outputtype="jacobian"), 16),
    ("replay_nscat", dict(nphoton=3000), dict(outputtype="nscat"), 128),
    ("replay_wm_perdet", dict(nphoton=3000), dict(outputtype="wm", replaydet=-1), 128),
    ("replay_wltof", dict(nphoton=3000), dict(outputtype="wltof"), 128),
    ("replay_wptof", dict(nphoton=3000), dict(outputtype="wptof"), 16),
    ("replay_flux", dict(nphoton=3000), dict(outputtype="flux"), 128),
    # frequency-domain replay outputs at 100 MHz (omega in rad/s)
    ("replay_rf", dict(nphoton=3000), dict(outputtype="rf", omega=2 * np.pi * 1e8), 128),
    ("replay_rf_perdet", dict(nphoton=3000), dict(outputtype="rf", omega=2 * np.pi * 1e8, replaydet=-1), 128),
    ("replay_rfmus", dict(nphoton=3000), dict(outputtype="rfmus", omega=2 * np.pi * 1e8), 128),
]
