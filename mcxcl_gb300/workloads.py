"""Named simulation inputs: the reference's built-in benchmarks and the
benchmark configurations this build is measured on.

Every entry is a ``run()`` dictionary.  Volumes are generated, never loaded.

* ``cube60``, ``cube60b``, ``cube60planar``, ``cubesph60b``: the reference's
  built-in benchmarks (src/mcx_bench.h:33-252, pmcxcl/pmcxcl/bench.py).
* ``config1`` .. ``config3``: the homogeneous cube, the cube with a
  scattering sphere (50 gates, four detectors) and the synthetic layered head
  used to measure this build (the head replaces the colin27 atlas, whose data
  is not used: nested ellipsoids of five tissue labels).
"""
import copy

import numpy as np


def sphere_volume(n=60, center=(30, 30, 30), radius=15, inner=2, outer=1):
    """A cube of label `outer` holding a sphere of label `inner`; a voxel is
    inside when its centre is (mcx_raster_sphere, src/mcx_shapes.c:234-293)."""
    idx = np.arange(n, dtype=np.float64) + 0.5
    x, y, z = np.meshgrid(idx, idx, idx, indexing="ij")
    d2 = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2
    vol = np.full((n, n, n), outer, dtype=np.uint8)
    vol[d2 < radius * radius] = inner
    return vol


def head_volume(shape=(181, 217, 181), axes=((88, 106, 88), (84, 102, 84), (79, 97, 79), (77, 95, 77),
                                             (60, 75, 60))):
    """Nested ellipsoids centred in the volume: label k+1 inside the k-th shell
    (innermost wins), 0 outside the head."""
    c = [(s - 1) / 2.0 for s in shape]
    x, y, z = np.meshgrid(*[np.arange(s, dtype=np.float32) for s in shape], indexing="ij")
    vol = np.zeros(shape, np.uint8)
    for label, (a, b, cc) in enumerate(axes, start=1):
        inside = ((x - c[0]) / a) ** 2 + ((y - c[1]) / b) ** 2 + ((z - c[2]) / cc) ** 2 <= 1.0
        vol[inside] = label
    return vol


def _cube60():
    return {
        "nphoton": 1000000,
        "vol": np.ones((60, 60, 60), dtype=np.uint8),
        "tstart": 0, "tend": 5e-9, "tstep": 5e-9,
        "srcpos": [29, 29, 0], "srcdir": [0, 0, 1],
        "prop": [[0, 0, 1, 1], [0.005, 1, 0.01, 1.37], [0.002, 5, 0.9, 1]],
        "isreflect": 0, "seed": 1648335518, "session": "cube60",
        "detpos": [[29, 19, 0, 1], [29, 39, 0, 1], [19, 29, 0, 1], [39, 29, 0, 1]],
        "issrcfrom0": 1,
    }


def builtin(name):
    """The reference's built-in benchmark of that name."""
    if name == "cube60":
        return _cube60()
    if name == "cube60b":
        return dict(_cube60(), isreflect=1, session="cube60b")
    if name == "cube60planar":
        return dict(_cube60(), isreflect=1, srctype="planar", srcpos=[10, 10, -10], srcparam1=[40, 0, 0, 0],
                    srcparam2=[0, 40, 0, 0], session="cube60planar")
    if name == "cubesph60b":
        return dict(_cube60(), isreflect=1, vol=sphere_volume(), session="cubesph60b")
    raise KeyError(name)


def config(n):
    """Benchmark configuration n (1-based): 1 homogeneous cube, 2 cube with
    sphere and detectors, 3 synthetic layered head."""
    if n == 1:
        cfg = _cube60()
        cfg.pop("detpos")
        cfg.update(issavedet=0, session="config1")
        return cfg
    if n == 2:
        cfg = _cube60()
        cfg.update(vol=sphere_volume(), prop=[[0, 0, 1, 1], [0.005, 1.0, 0.01, 1.37], [0.002, 5.0, 0.9, 1.0]],
                   isreflect=1, tstep=1e-10, nphoton=100000000,
                   detpos=[[30, 20, 0, 1], [30, 40, 0, 1], [20, 30, 0, 1], [40, 30, 0, 1]],
                   savedetflag="dsp", issaveseed=1, session="config2")
        return cfg
    if n == 3:
        vol = head_volume()
        cx, cy = 90, 108
        # source at the outer-shell apex on the minimum-z side, pointing +z
        ztop = int(np.argmax(vol[cx, cy, :] > 0))
        dets = []
        for k in range(16):
            ang = 2 * np.pi * k / 16
            dx, dy = 30 * np.cos(ang), 30 * np.sin(ang)
            ix, iy = int(round(cx + dx)), int(round(cy + dy))
            iz = int(np.argmax(vol[ix, iy, :] > 0))
            dets.append([ix, iy, iz, 2])
        return {
            "nphoton": 100000000, "vol": vol,
            "prop": [[0, 0, 1, 1], [0.019, 7.8, 0.89, 1.37], [0.019, 7.8, 0.89, 1.37], [0.004, 0.009, 0.89, 1.37],
                     [0.02, 9.0, 0.89, 1.37], [0.08, 40.9, 0.84, 1.37]],
            "tstart": 0, "tend": 5e-9, "tstep": 5e-10,
            "srcpos": [cx, cy, ztop], "srcdir": [0, 0, 1], "issrcfrom0": 1,
            "detpos": dets, "minenergy": 1e-4, "seed": 12345, "savedetflag": "dsp", "issaveseed": 1,
            "session": "config3",
        }
    raise KeyError(n)


def describe(n):
    """One line naming benchmark configuration n and its sizes."""
    return {
        1: "60^3 homogeneous cube (mua 0.005, mus 1.0, g 0.01, n 1.37), pencil (29,29,0) +z, one 0-5 ns gate, "
           "no reflection, no detectors",
        2: "60^3 cube + r15 sphere (label 2), Fresnel on, 50 gates x 0.1 ns, 4 r=1 detectors on z=0 saving "
           "detid/nscat/ppath + seeds, pencil (29,29,0) +z",
        3: "181x217x181 synthetic layered head (5 ellipsoid shells), 10 gates over 0-5 ns, 16 r=2 detectors on a "
           "30 mm ring, roulette at 1e-4, pencil on the top surface +z",
    }[n]


def gaussian_field(shape, corr, seed):
    """Unit-variance Gaussian random field: seeded white noise convolved
    (periodically, by FFT) with a Gaussian of standard deviation corr voxels."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal(shape)
    freqs = [np.fft.fftfreq(n) for n in shape]
    k2 = sum(np.meshgrid(*[f * f for f in freqs], indexing="ij"))
    kernel = np.exp(-2.0 * (np.pi ** 2) * (corr ** 2) * k2)
    z = np.real(np.fft.ifftn(np.fft.fftn(white) * kernel))
    z -= z.mean()
    return z / z.std()


def diff_config(n=100, nphoton=10000000, seed=2024):
    """Differentiation workload: an n^3 volume of per-voxel mua
    0.01 (1 + 0.2 z) per mm (z a unit-variance Gaussian random field of 5-voxel
    correlation length), mus 1/mm, g 0.9, n 1.37; pencil source at the centre
    of the z = 0 face pointing +z; 16 detectors of radius 1 mm on a 10 mm ring
    around it.  Returns (cfg without 'vol', mua, target mua): the target
    readings come from a second seeded field."""
    c = n / 2.0
    dets = [[c + 10 * np.cos(2 * np.pi * k / 16), c + 10 * np.sin(2 * np.pi * k / 16), 0, 1] for k in range(16)]
    cfg = {
        "nphoton": nphoton, "prop": [[0, 0, 1, 1], [0.01, 1.0, 0.9, 1.37]],
        "tstart": 0, "tend": 5e-9, "tstep": 5e-9, "srcpos": [c, c, 0], "srcdir": [0, 0, 1], "issrcfrom0": 1,
        "detpos": dets, "seed": seed, "isreflect": 1, "session": "diff",
    }
    shape = (n, n, n)
    mua = (0.01 * (1 + 0.2 * gaussian_field(shape, 5.0, 11))).astype(np.float32)
    target = (0.01 * (1 + 0.2 * gaussian_field(shape, 5.0, 12))).astype(np.float32)
    return cfg, np.maximum(mua, 1e-4), np.maximum(target, 1e-4)


def batch_configs(nsim=512, master_seed=7, edge=(32, 128), photons=(1e5, 1e7)):
    """Batch workload: nsim independent cubes with an integer edge uniform in
    [edge], with probability 0.5 a spherical inclusion of random centre and
    radius; mua log-uniform in [0.001, 0.1]/mm, mus uniform in [0.5, 2.0]/mm,
    g uniform in [0.6, 0.95], n uniform in [1.33, 1.45] (inclusion drawn the
    same way); photon counts log-uniform in [photons]; pencil source at the
    centre of the z = 0 face; one 5 ns gate.  Seeds come from numpy's
    SeedSequence(master_seed).spawn(nsim)."""
    seqs = np.random.SeedSequence(master_seed).spawn(nsim)
    out = []
    for k, ss in enumerate(seqs):
        rng = np.random.default_rng(ss)
        n = int(rng.integers(edge[0], edge[1] + 1))

        def medium():
            return [float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-1)))), float(rng.uniform(0.5, 2.0)),
                    float(rng.uniform(0.6, 0.95)), float(rng.uniform(1.33, 1.45))]
        prop = [[0, 0, 1, 1], medium()]
        vol = np.ones((n, n, n), np.uint8)
        if rng.random() < 0.5:
            r = float(rng.uniform(0.1, 0.3)) * n
            c = rng.uniform(r, n - r, size=3)
            idx = np.arange(n) + 0.5
            x, y, z = np.meshgrid(idx, idx, idx, indexing="ij")
            vol[(x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 < r * r] = 2
            prop.append(medium())
        nph = int(np.exp(rng.uniform(np.log(photons[0]), np.log(photons[1]))))
        out.append({
            "nphoton": nph, "vol": vol, "prop": prop, "tstart": 0, "tend": 5e-9, "tstep": 5e-9,
            "srcpos": [n / 2.0, n / 2.0, 0], "srcdir": [0, 0, 1], "issrcfrom0": 1, "isreflect": 1,
            "issavedet": 0, "seed": int(rng.integers(1, 2 ** 31 - 1)), "session": "batch%d" % k,
        })
    return out


def copy_cfg(cfg):
    return copy.deepcopy(cfg)
