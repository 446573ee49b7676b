"""Seed words made on the device from one generator window.

mcxg_set_seeds_window jumps every block of words ahead on the GPU (the
one-step matrix raised to the block length, then its powers of two) and
expands the blocks; the words must be the serial generator's
(mcx_rand_words: srand(seed) then rand(), src/mcx_host.cpp:696-700, 759-768),
word for word: one thread, ragged last blocks, one block per 1,024 words up to
16,384 blocks, the longer blocks of more than 67 M words, and a window taken
after a skip (a later repetition's seeds).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mcxcl_gb300
    info = mcxcl_gb300.gpuinfo()
    if not info:
        pytest.fail("no CUDA device visible to the transport library")
    return info[0]


@pytest.mark.parametrize("seed,skip,nthread", [(1648335518, 0, 1), (12345, 0, 7), (29012392, 0, 622592),
                                               (1, 0, 4194304), (77, 0, 17000003), (5, 2490368, 300001)])
def test_device_jump_ahead_gives_the_serial_words(gpu, seed, skip, nthread):
    from mcxcl_gb300 import _lib
    L = _lib.load()
    s = ctypes.c_void_p()
    assert L.mcxg_create(0, ctypes.byref(s)) == 0
    try:
        window = np.zeros(31, np.uint32)
        assert L.mcx_rand_blocks(seed, skip, 1, 1, window.ctypes.data) == 0
        assert L.mcxg_set_seeds_window(s, window.ctypes.data, nthread) == 0
        got = np.zeros(4 * nthread, np.uint32)
        assert L.mcxg_get_seeds(s, got.ctypes.data, nthread) == 0
        want = np.zeros(skip + 4 * nthread, np.uint32)
        L.mcx_rand_words(seed, want.ctypes.data, want.size)
        bad = np.flatnonzero(got != want[skip:])
        assert bad.size == 0, ("first differing word", int(bad[0]) if bad.size else None)
    finally:
        L.mcxg_destroy(s)
