"""The output buffers pass from the Config to numpy without a copy.

pmcxcl._take hands a buffer the library allocated (the field, the detected
records, the seeds) to a numpy array: the Config's pointer becomes NULL, so
mcx_clearcfg leaves the buffer alone, and the array frees it through
mcx_free_buffer once its last view is gone.  Checked here on the label volume
of a validated Config, a buffer of the same kind (malloc'd, freed by
mcx_clearcfg), with no GPU.
"""
import ctypes
import gc

import numpy as np


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
