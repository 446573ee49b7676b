"""The allocation-free energy sum (mcxg_energy_sum_noalloc) against the
session path (mcxg_get_energy, which reports stat.energytot/energyesc).

Callers that cannot let the library allocate device memory -- a service with
a device budget fixed at start-up, a framework that owns every buffer -- use
the allocation-free entry point on their own arrays.  This test hands it the
per-thread weights of two simulations in a row (torch owns the device
buffers) and checks both FP64 sums against the session path's.  The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def test_energy_sum_noalloc_matches_session_path_twice():
    import torch
    import mcxcl_gb300
    from mcxcl_gb300 import _lib
    L = _lib.load()
    assert torch.cuda.is_available()
    for seed in (4711, 4712):
        res = mcxcl_gb300.run(cases.cube60(nphoton=300000, issavedet=0, seed=seed, savethreadenergy=1))
        e = res["threadenergy"]
        d_energy = torch.from_numpy(np.ascontiguousarray(e)).cuda()
        d_sums = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.mcxg_energy_sum_noalloc(0, ctypes.c_void_p(d_energy.data_ptr()), e.shape[0],
                                       ctypes.c_void_p(d_sums.data_ptr()))
        assert rc == 0, L.mcxg_error_string(rc)
        esc, launched = d_sums.cpu().numpy()
        assert launched == pytest.approx(res["stat"]["energytot"], rel=1e-12)
        assert esc == pytest.approx(res["stat"]["energyesc"], rel=1e-12)
        assert launched == pytest.approx(300000, abs=10)


def test_energy_sum_noalloc_rejects_oversize():
    from mcxcl_gb300 import _lib
    L = _lib.load()
    rc = L.mcxg_energy_sum_noalloc(0, ctypes.c_void_p(1), 8388608 + 1, ctypes.c_void_p(1))
    assert rc == 4 and L.mcxg_error_string(rc) == b"input exceeds a compiled limit"
