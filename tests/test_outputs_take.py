"""The output buffers pass from the Config to numpy without a copy.

pmcxcl._take hands a buffer the library allocated (the field, the detected
records, the seeds) to a numpy array: the Config's pointer becomes NULL, so
mcx_clearcfg leaves the buffer alone, and the array frees it through
mcx_free_buffer once its last view is gone.  Checked on the label volume
of a validated Config, a buffer of the same kind (malloc'd, freed by
mcx_clearcfg), with no GPU; on the GPU, a run whose outputs reuse the
buffers an earlier run gave back must hold only its own values.
"""
import ctypes
import gc

import numpy as np
import pytest


def test_take_moves_ownership_and_frees_once(monkeypatch):
    from mcxcl_gb300 import _lib, pmcxcl
    L = _lib.load()
    vol = np.zeros((6, 5, 4), np.uint8)
    vol[1:5, 1:4, 1:3] = 1
    cfg = {"nphoton": 1000, "vol": vol, "tstart": 0, "tend": 5e-9, "tstep": 5e-9,
           "srcpos": [2, 2, 0], "srcdir": [0, 0, 1], "prop": [[0, 0, 1, 1], [0.005, 1.0, 0.01, 1.37]]}
    C = _lib.Config()
    pmcxcl.parse_config(cfg, C)
    L.mcx_validatecfg(ctypes.byref(C), None, None, 0)
    pmcxcl._check(C)
    dims = (C.dim.x, C.dim.y, C.dim.z)
    n = dims[0] * dims[1] * dims[2]
    expect = np.ctypeslib.as_array(C.vol, shape=(n,)).copy()

    freed = []
    real = L.mcx_free_buffer

    def spy(p):
        freed.append(p)
        real(p)

    monkeypatch.setattr(L, "mcx_free_buffer", spy)
    arr = pmcxcl._take(C, "vol", ctypes.c_uint32, n)
    assert not C.vol                                  # the Config let go
    L.mcx_clearcfg(ctypes.byref(C))                   # must not free it
    view = arr.reshape(dims, order="F")
    del arr
    gc.collect()
    assert freed == []                                # a view keeps the buffer
    np.testing.assert_array_equal(view.reshape(-1, order="F"), expect)
    del view
    gc.collect()
    assert len(freed) == 1                            # freed once, by the array


@pytest.mark.gpu
def test_reused_output_buffers_hold_only_the_new_run():
    """A run's field and records may land in buffers an earlier run's arrays
    gave back (mcx_free_buffer keeps them): every element must be the new
    run's.  The second run's source sits in the opposite corner of a strongly
    absorbing cube, so the first run's hot voxels are nearly empty in it."""
    import mcxcl_gb300
    vol = np.ones((40, 40, 40), np.uint8)
    base = {"nphoton": 200000, "vol": vol, "tstart": 0, "tend": 5e-9, "tstep": 5e-10, "srcdir": [0, 0, 1],
            "prop": [[0, 0, 1, 1], [0.5, 2.0, 0.0, 1.0]], "issrcfrom0": 1, "seed": 7,
            "detpos": [[2, 2, 0, 2], [37, 37, 39, 2]], "savedetflag": "dp"}
    a = mcxcl_gb300.run(dict(base, srcpos=[2, 2, 0]))
    hot = a["flux"][:4, :4, :4].copy()
    na = a["detp"].shape[1]
    del a
    gc.collect()
    b = mcxcl_gb300.run(dict(base, srcpos=[37, 37, 39], srcdir=[0, 0, -1]))
    assert hot.sum() > 0
    assert b["flux"][:4, :4, :4].sum() < 1e-3 * hot.sum()
    assert np.isfinite(b["flux"]).all()
    assert b["detp"].shape[1] > 0 and na > 0
    assert (b["detp"][0] >= 1).all() and (b["detp"][0] <= 2).all()    # detector ids, not stale bytes
