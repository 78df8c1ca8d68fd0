"""Arithmetic of the shared-memory accumulator entries of the cycle kernels:
an entry is two 32-bit words {low: unsigned, high: signed}; a value q is
added as q & 0xffffffff to the low word (wrapping) and (q >> 32) + carry to
the high word, the carry being whether the low add wrapped.  Read as one
little-endian 64-bit word the entry must equal the sum of the values, in
any order, for up to 2^20 values of |q| <= 2^42 (the flush interval and the
quantum bound of the kernels).  Checked here with exact integers."""
import numpy as np

M32 = 1 << 32


def add(entry, q):
    lo, hi = entry
    qlo = q & (M32 - 1)
    new_lo = (lo + qlo) & (M32 - 1)
    carry = 1 if new_lo < lo else 0  # old + lo < old (unsigned wrap)
    hi = hi + (q >> 32) + carry
    assert -(1 << 31) <= hi < (1 << 31)
    return new_lo, hi


def as_i64(entry):
    lo, hi = entry
    u = ((hi & (M32 - 1)) << 32) | lo
    return u - (1 << 64) if u >= (1 << 63) else u


def test_random_orders_and_signs():
    rng = np.random.default_rng(5)
    for trial in range(20):
        n = int(rng.integers(1, 3000))
        qs = [int(x) for x in rng.integers(-(1 << 42), (1 << 42) + 1, size=n)]
        e = (0, 0)
        for q in qs:
            e = add(e, q)
        assert as_i64(e) == sum(qs)


def test_extremes_over_a_full_flush_interval():
    # 2^20 maximal values of one sign: the high word's largest magnitude
    for q in ((1 << 42), -(1 << 42)):
        n = 1 << 20
        e = (0, 0)
        # the same value n times: low words repeat, so add in closed form per
        # block of 2^10 and check the word bound on the way
        for _ in range(n >> 10):
            for _ in range(1 << 10):
                e = add(e, q)
        assert as_i64(e) == q * n


def test_alternating_carries():
    e = (0, 0)
    total = 0
    for k in range(5000):
        q = (M32 - 1) if k % 2 == 0 else -(M32 - 3)
        e = add(e, q)
        total += q
        assert as_i64(e) == total
