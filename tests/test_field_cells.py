"""The field's count arithmetic, restated on the CPU.

A deposit's fixed-point count k (signed 64-bit) is added to an element as
two 32-bit words: the low word with an add that returns the old value, and
the high word plus the low add's carry-out to a separate word (both modulo
2^32).  Whatever the order of the adds, the two words must hold the signed
64-bit sum of the k's (mcx_kernel.cuh, field_commit; mcx_device.cu,
cell_value).
"""
import numpy as np

M32 = (1 << 32) - 1


def _commit(lo, hi, k):
    klo, khi = k & M32, (k >> 32) & M32
    up = khi
    if klo:
        old = lo
        lo = (lo + klo) & M32
        up += 1 if old + klo > M32 else 0
    hi = (hi + up) & M32
    return lo, hi


def _value(lo, hi):
    v = (hi << 32) | lo
    return v - (1 << 64) if v >> 63 else v


def test_words_hold_the_signed_sum_in_any_order():
    rng = np.random.default_rng(7)
    for trial in range(200):
        n = int(rng.integers(1, 400))
        scale = int(rng.choice([1 << 8, 1 << 31, 1 << 40, 1 << 52]))
        ks = [int(x) for x in rng.integers(-scale // 8, scale, n)]
        for order in (ks, ks[::-1], list(rng.permutation(ks))):
            lo = hi = 0
            for k in order:
                lo, hi = _commit(lo, hi, int(k))
            assert _value(lo, hi) == sum(ks)


def test_many_wraps_of_the_low_word():
    lo = hi = 0
    k = (1 << 32) - 3
    for _ in range(10000):
        lo, hi = _commit(lo, hi, k)
    assert _value(lo, hi) == 10000 * k
