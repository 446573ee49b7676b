"""The hot-voxel tile (mcxg_set_tile) against direct deposits.

With the tile on, a block's deposits into a box of voxels next to the source
(first gates) accumulate in shared memory and reach the field when the block
ends.  The tile and the direct-deposit kernels are different instantiations,
whose floating-point contractions may differ, so their photons need not be
bit-identical; what the tile must not do is lose or repeat a deposit.  With
the energy output every deposit is a piece of absorbed weight, so the field's
FP64 total equals the launched minus the escaped weight (per-thread float
sums: about 1e-6) for any path the photons took: a lost or repeated tile
element (each holds up to 1e-3 of the total) breaks that at once.  The two
kernels' absorbed fractions agree within the Monte Carlo noise.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(L, C, sess, tile):
    assert L.mcxg_set_tile(sess, tile) == 0
    ms = ctypes.c_float()
    rc = L.mcxg_simulate(sess, 0, ctypes.byref(ms))
    assert rc == 0, L.mcxg_error_string(rc)
    box = np.zeros(8, np.uint32)
    assert L.mcxg_get_tile(sess, box.ctypes.data) == 0
    n = int(C.maxgate) * C.dim.x * C.dim.y * C.dim.z
    cnt = np.zeros(n, np.int64)
    rem = np.zeros(n, np.float32)
    assert L.mcxg_get_field_planes(sess, cnt.ctypes.data, rem.ctypes.data) == 0
    f64 = np.zeros(n, np.float64)
    assert L.mcxg_get_field_f64(sess, f64.ctypes.data) == 0
    esc, lau = ctypes.c_double(), ctypes.c_double()
    assert L.mcxg_get_energy(sess, ctypes.byref(esc), ctypes.byref(lau)) == 0
    return dict(box=box, cnt=cnt, rem=rem, f64=f64, energy=(esc.value, lau.value))


@pytest.mark.parametrize("k,photons", [(1, 2e6), (2, 2e6), (3, 5e5)])
def test_tile_loses_no_deposit(k, photons):
    from mcxcl_gb300 import _lib, pmcxcl, workloads
    L = _lib.load()
    cfg = workloads.config(k)
    cfg.update(nphoton=int(photons), outputtype="energy", minenergy=0.0)   # no roulette: weight is conserved
    C = _lib.Config()
    pmcxcl.parse_config(cfg, C)
    L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    pmcxcl._check(C)
    sess = L.mcx_prepare_simulation(ctypes.byref(C))
    pmcxcl._check(C)
    try:
        runs = {t: _run(L, C, sess, t) for t in (0, 1024, 4096)}
        assert runs[0]["box"][7] == 0
        for t, r in runs.items():
            esc, lau = r["energy"]
            absorbed = lau - esc
            assert abs(r["f64"].sum() - absorbed) <= 1e-5 * absorbed, (t, r["f64"].sum(), absorbed)
            if t:
                x0, y0, z0, nx, ny, nz, ng, el = (int(v) for v in r["box"])
                assert 0 < el <= t and el == nx * ny * nz * ng
                assert x0 + nx <= C.dim.x and y0 + ny <= C.dim.y and z0 + nz <= C.dim.z and ng <= C.maxgate
                a0 = (runs[0]["energy"][1] - runs[0]["energy"][0]) / runs[0]["energy"][1]
                assert abs(absorbed / lau - a0) <= 0.01 * a0
    finally:
        L.mcxg_set_tile(sess, 0)
        L.mcx_clearcfg(ctypes.byref(C))
