"""The hot-voxel tile (mcxg_set_tile) against direct deposits.

With the tile on, a block's deposits into a box of voxels next to the source
(first gates) accumulate in shared memory and reach the field when the block
ends.  Each deposit is still split into an integer count of the problem's
fixed-point unit and a float remainder, and integer sums do not depend on
the order of the adds, so on the same seeds and launch shape the count
planes must be equal bit for bit to those of direct deposits; the float
remainders differ only by their summation order.  The photons themselves
(energies, detected records) do not depend on where deposits go.
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
def test_tile_keeps_the_exact_counts(k, photons):
    from mcxcl_gb300 import _lib, pmcxcl, workloads
    L = _lib.load()
    cfg = workloads.config(k)
    cfg["nphoton"] = int(photons)
    C = _lib.Config()
    pmcxcl.parse_config(cfg, C)
    L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    pmcxcl._check(C)
    sess = L.mcx_prepare_simulation(ctypes.byref(C))
    pmcxcl._check(C)
    try:
        a = _run(L, C, sess, 0)
        b = _run(L, C, sess, 4096)
        c = _run(L, C, sess, 1024)
        assert a["box"][7] == 0
        for r in (b, c):
            x0, y0, z0, nx, ny, nz, ng, el = (int(v) for v in r["box"])
            assert 0 < el <= (4096 if r is b else 1024) and el == nx * ny * nz * ng
            assert x0 + nx <= C.dim.x and y0 + ny <= C.dim.y and z0 + nz <= C.dim.z and ng <= C.maxgate
            assert np.array_equal(r["cnt"], a["cnt"])
            assert r["energy"] == a["energy"]
            nz_ = a["f64"] > 0
            rel = np.abs(r["f64"][nz_] - a["f64"][nz_]) / a["f64"][nz_]
            assert rel.max() < 1e-6, rel.max()
    finally:
        L.mcxg_set_tile(sess, 0)
        L.mcx_clearcfg(ctypes.byref(C))
