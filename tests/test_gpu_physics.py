"""Physics checks on the benchmark workloads.

* Homogeneous cube (60^3, mua 0.005, mus 1, g 0.01, pencil at the centre of
  the z = 0 face, no boundary reflection): the CW fluence follows the
  semi-infinite diffusion solution of the reference's utils/cwdiffusion.m
  (Boas 2002, Haskell 1994; Reff = 0 as in demo_validation_homogeneous.m:111)
  away from the source and the lateral faces.
* Synthetic layered head (181x217x181, five tissues, 16 detectors, Russian
  roulette at 1e-4): the exact kernel reproduces the oracle bit for bit on a
  photon sample, and the fast kernel agrees with the exact one statistically.
"""
import numpy as np
import pytest

from mcxcl_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mcxcl_gb300
    info = mcxcl_gb300.gpuinfo()
    if not info:
        pytest.fail("no CUDA device visible to the transport library")
    return info[0]


def cwdiffusion(mua, musp, Reff, src, det):
    """Restatement of utils/cwdiffusion.m:25-36: dipole solution of the CW
    diffusion equation in a semi-infinite medium, fluence per unit power (1/mm^2)."""
    D = 1.0 / (3.0 * (mua + musp))
    zb = (1.0 + Reff) / (1.0 - Reff) * 2.0 * D
    z0 = 1.0 / (musp + mua)
    src = np.asarray(src, float)
    det = np.atleast_2d(np.asarray(det, float))
    r1 = np.linalg.norm(det - (src + [0, 0, z0]), axis=1)
    r2 = np.linalg.norm(det - (src + [0, 0, -z0 - 2 * zb]), axis=1)
    b = np.sqrt(3.0 * mua * musp)
    return 1.0 / (4 * np.pi * D) * (np.exp(-b * r1) / r1 - np.exp(-b * r2) / r2)


def test_homogeneous_cube_follows_cw_diffusion(gpu):
    import mcxcl_gb300
    cfg = workloads.config(1)
    cfg.update(nphoton=20000000, outputtype="fluence")
    r = mcxcl_gb300.run(cfg)
    phi = r["flux"][..., 0]                    # CW fluence per unit source weight, 1/mm^2
    src = np.array([29.0, 29.0, 0.0])
    mua, musp = 0.005, 1.0 * (1 - 0.01)
    # diffusion holds beyond ~10 transport mean free paths (1 mm here) from the
    # pencil beam's entry: a depth profile from 12 mm and a lateral profile
    # 8 mm deep, 8.5-14.5 mm from the entry point, well inside the lateral faces
    pts = []
    for z in range(12, 20):
        pts.append((29, 29, z))
    for x in range(31, 42):
        pts.append((x, 29, 8))
    pts = np.array(pts)
    centres = pts + 0.5
    mc = np.array([phi[tuple(p)] + phi[28 - (p[0] - 29) if p[0] != 29 else 28, p[1], p[2]] for p in pts]) / 2
    dif = cwdiffusion(mua, musp, 0.0, src, centres)
    ratio = mc / dif
    assert np.all(np.abs(ratio - 1) < 0.06), np.round(ratio, 3)
    assert abs(np.median(ratio) - 1) < 0.03, np.median(ratio)


def test_head_exact_kernel_matches_oracle_bits(gpu, oracle_mod):
    import mcxcl_gb300
    O = oracle_mod
    cfg = dict(workloads.config(3), nphoton=20000)
    g = mcxcl_gb300.run(dict(cfg, autopilot=0, nthread=4096, nblocksize=64, exactmath=1, savethreadenergy=1))
    r = O.run(cfg, nthread=4096, core=gpu["core"], mathmode=O.MATH_PMATH, fieldmode=O.FIELD_DOUBLE)
    assert np.array_equal(g["threadenergy"].view(np.uint32), np.asarray(r["energy"], np.float32).view(np.uint32))
    assert g["stat"]["detected"] == r["stat"]["detected"]
    assert g["stat"]["eventcount"]["step"] == r["stat"]["nstep"]
    ref = np.asarray(r["flux"], np.float64).reshape(g["flux"].shape, order="F")
    np.testing.assert_allclose(g["flux"], ref, rtol=1e-4, atol=1e-6 * np.abs(ref).max())


def test_head_fast_kernel_agrees_with_exact(gpu):
    import mcxcl_gb300
    cfg = dict(workloads.config(3), nphoton=2000000)
    f = mcxcl_gb300.run(cfg)
    e = mcxcl_gb300.run(dict(cfg, exactmath=1, seed=54321))
    af = f["stat"]["energyabs"] / f["stat"]["energytot"]
    ae = e["stat"]["energyabs"] / e["stat"]["energytot"]
    assert abs(af - ae) < 0.005, (af, ae)
    df, de = f["stat"]["detected"], e["stat"]["detected"]
    assert abs(df - de) <= 4 * np.sqrt(de) + 0.01 * de, (df, de)


def fddiffusion(mua, musp, n, omega, src, det):
    """Frequency-domain form of the same dipole solution: the decay constant
    sqrt(3 mua musp) becomes sqrt((mua + i omega n / c0) / D), the phase
    convention of the RF transport's weight update exp(-(mua + i omega n /
    c0) ds) (mcx_core.cl:2750-2760); zero internal reflection."""
    D = 1.0 / (3.0 * (mua + musp))
    zb = 2.0 * D
    z0 = 1.0 / (musp + mua)
    c0 = 299792458000.0                       # mm/s
    k = np.sqrt((mua + 1j * omega * n / c0) / D)
    src = np.asarray(src, float)
    det = np.atleast_2d(np.asarray(det, float))
    r1 = np.linalg.norm(det - (src + [0, 0, z0]), axis=1)
    r2 = np.linalg.norm(det - (src + [0, 0, -z0 - 2 * zb]), axis=1)
    return 1.0 / (4 * np.pi * D) * (np.exp(-k * r1) / r1 - np.exp(-k * r2) / r2)


def test_homogeneous_cube_rf_follows_fd_diffusion(gpu):
    """The RF transport (omega > 0, complex photon weights) on the homogeneous
    cube at 500 MHz: the complex fluence agrees in amplitude and phase with
    the frequency-domain diffusion solution, away from the entry point."""
    import mcxcl_gb300
    omega = 2 * np.pi * 5e8
    cfg = workloads.config(1)
    cfg.update(nphoton=20000000, outputtype="fluence", omega=omega)
    r = mcxcl_gb300.run(cfg)
    phi = r["flux"][..., 0]
    assert phi.dtype == np.complex64
    src = np.array([29.0, 29.0, 0.0])
    pts = np.array([(29, 29, z) for z in range(12, 20)] + [(x, 29, 8) for x in range(31, 42)])
    mc = np.array([phi[tuple(p)] + phi[28 - (p[0] - 29) if p[0] != 29 else 28, p[1], p[2]] for p in pts]) / 2
    fd = fddiffusion(0.005, 0.99, 1.37, omega, src, pts + 0.5)
    ratio = mc / fd
    assert np.all(np.abs(np.abs(ratio) - 1) < 0.08), np.round(np.abs(ratio), 3)
    assert np.all(np.abs(np.angle(ratio)) < 0.08), np.round(np.angle(ratio), 3)
    # the phase lag grows with depth below the source
    lag = -np.angle(mc[:8])
    assert np.all(np.diff(lag) > 0) and lag[-1] > 1.0, np.round(lag, 3)
