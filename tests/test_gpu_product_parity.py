"""The product (fast) kernel held to the parity bar on the measured workloads.

The fast instantiation is what ``run()`` and the benchmark use by default
(MUFU transcendentals, the GB300 autopilot's thread count).  Its RNG
decomposition differs from the exact instantiation's, so the comparison is
statistical.  The exact instantiation reproduces the CPU oracle bit for bit
(test_gpu_parity.py), and the oracle reproduces the reference kernel bit for
bit (test_oracle_pins.py), so this is the product kernel against the
reference's own arithmetic on:

* the cube + sphere workload (60^3, radius-15 sphere of a second medium,
  Fresnel at every boundary, 50 gates of 0.1 ns, four r = 1 disk detectors
  saving detector id, scatter counts and partial paths), 1e7 photons a seed;
* the synthetic layered head (181 x 217 x 181, five tissue labels, 16 r = 2
  detectors on a 30 mm ring, 10 gates, Russian roulette at 1e-4), 2e6 photons
  a seed.

Criteria (the reference's deposit and detection, mcx_core.cl:2815-2929 and
867-926): the total absorbed fraction and the detected-photon count agree
within 0.5 % (the count also within its Poisson band), and the per-voxel,
per-gate fluence agrees within 3 sigma of the Monte Carlo noise, sigma
estimated from 10 independent seeds on each side, wherever the relative
standard error of both sides is below 5 %.  With 10 + 10 samples the
statistic is close to Student's t with 18 degrees of freedom, of which about
0.8 % of independent elements exceed 3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Moments:
    """Per-element mean and variance of the runs' fluence, accumulated in
    FP64 without keeping every run."""

    def __init__(self):
        self.n = 0
        self.s = None
        self.s2 = None
        self.absorbed = []
        self.detected = 0
        self.launched = 0.0

    def add(self, res):
        f = np.asarray(res["flux"], np.float64).ravel(order="F")
        if self.s is None:
            self.s = np.zeros_like(f)
            self.s2 = np.zeros_like(f)
        self.s += f
        self.s2 += f * f
        self.n += 1
        st = res["stat"]
        self.absorbed.append(st["energyabs"] / st["energytot"])
        self.detected += int(st["detected"])
        self.launched += st["energytot"]

    def mean(self):
        return self.s / self.n

    def var_of_mean(self):
        m = self.mean()
        return np.maximum(self.s2 / self.n - m * m, 0.0) * self.n / (self.n - 1) / self.n


def _runs(cfg, seeds, **kw):
    import mcxcl_gb300
    m = Moments()
    for sd in seeds:
        m.add(mcxcl_gb300.run(dict(cfg, seed=int(sd), **kw)))
    return m


def _check(fast, exact, min_voxels):
    a_f, a_e = np.mean(fast.absorbed), np.mean(exact.absorbed)
    assert abs(a_f - a_e) <= 0.005 * a_e, ("absorbed fraction", a_f, a_e)
    d_f, d_e = fast.detected, exact.detected
    assert d_e > 1000, d_e
    assert abs(d_f - d_e) <= 0.005 * d_e + 3 * np.sqrt(d_f + d_e), ("detected photons", d_f, d_e)
    mf, me = fast.mean(), exact.mean()
    vf, ve = fast.var_of_mean(), exact.var_of_mean()
    ok = (me > 0) & (mf > 0) & (np.sqrt(ve) < 0.05 * me) & (np.sqrt(vf) < 0.05 * mf)
    z = np.abs(mf[ok] - me[ok]) / np.sqrt(vf[ok] + ve[ok])
    assert ok.sum() >= min_voxels, ok.sum()
    frac = float(np.mean(z > 3))
    assert frac < 0.02, ("fraction of elements beyond 3 sigma", frac, int(ok.sum()))
    return {"absorbed": (a_f, a_e), "detected": (d_f, d_e), "elements": int(ok.sum()), "beyond_3sigma": frac}


def test_fast_kernel_cube_sphere_workload_parity():
    """Cube + sphere, 50 gates, 4 detectors: 10 seeds x 1e7 photons each side."""
    from mcxcl_gb300 import workloads
    cfg = workloads.config(2)
    cfg["nphoton"] = 10_000_000
    fast = _runs(cfg, 5000 + np.arange(10))
    exact = _runs(cfg, 6000 + np.arange(10), exactmath=1)
    r = _check(fast, exact, min_voxels=50_000)
    print("cube + sphere:", r)


def test_fast_kernel_head_workload_parity():
    """Synthetic layered head, roulette, 16 detectors: 10 seeds x 2e6 photons each side."""
    from mcxcl_gb300 import workloads
    cfg = workloads.config(3)
    cfg["nphoton"] = 2_000_000
    fast = _runs(cfg, 7000 + np.arange(10))
    exact = _runs(cfg, 8000 + np.arange(10), exactmath=1)
    r = _check(fast, exact, min_voxels=5_000)
    print("head:", r)


def test_fluence_accumulation_error_against_fp64():
    """The precision contract on the homogeneous cube at 1e8 photons: every
    deposit of one run goes to the compensated field (the product: float high
    and low planes with an integer spill count), to an FP64 field, to a plain
    float field and to a float field with the reference's +-1000 spill
    (mcx_core.cl:2880-2886, merged in float as mcx_host.cpp:1252-1257 does),
    so all four hold exactly the same photons.  The compensated field's error
    against FP64 stays at or below 1e-6 (max and median over every non-zero
    element); the plain float field's is worse."""
    import ctypes
    from mcxcl_gb300 import _lib, pmcxcl, workloads
    L = _lib.load()
    cfg = workloads.config(1)
    cfg["nphoton"] = 100_000_000
    C = _lib.Config()
    try:
        pmcxcl.parse_config(cfg, C)
        L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
        pmcxcl._check(C)
        s = L.mcx_prepare_simulation(ctypes.byref(C))
        pmcxcl._check(C)
        ms = ctypes.c_float()
        assert L.mcxg_simulate(s, 128, ctypes.byref(ms)) == 0        # MCXG_VERIFY
        n = 60 * 60 * 60
        two = np.zeros(n, np.float64)
        f64 = np.zeros(n, np.float64)
        plain = np.zeros(n, np.float32)
        spill = np.zeros(n, np.float32)
        assert L.mcxg_get_field_f64(s, two.ctypes.data) == 0
        assert L.mcxg_get_verify(s, f64.ctypes.data, plain.ctypes.data, spill.ctypes.data) == 0
    finally:
        L.mcx_clearcfg(ctypes.byref(C))
    nz = f64 > 0
    assert nz.sum() > 100_000
    err = {}
    for name, x in (("compensated", two), ("plain float", plain.astype(np.float64)),
                    ("spill", spill.astype(np.float64))):
        r = np.abs(x[nz] - f64[nz]) / f64[nz]
        err[name] = (float(r.max()), float(np.median(r)))
    print("relative error against FP64 (max, median):", err)
    assert err["compensated"][0] <= 1e-6 and err["compensated"][1] <= 1e-6, err
    assert err["plain float"][0] > 10 * err["compensated"][0], err
    # the same photons: the totals agree to the FP64 sum's own rounding
    assert abs(two.sum() - f64.sum()) <= 1e-9 * f64.sum()
