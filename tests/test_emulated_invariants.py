"""Host-side checks of the integer invariants the emulated-FP64 kernels rely
on, restated in Python: the balanced base-256 digit split (64-bit recurrence
and the 32-bit two-part form the split kernel uses give the same digits,
and the digits rebuild the fixed-point value), and the level restart
periods (every exact level stays within 2^24, restarting levels form one
run of adjacent levels)."""
import random

import pytest


def digits_64(fx, S):
    """d = ((v + 128) & 255) - 128, v = (v - d) >> 8, least significant first."""
    h = [0] * S
    for p in range(S - 1, 0, -1):
        d = ((fx + 128) & 255) - 128
        h[p] = d
        fx = (fx - d) >> 8
    h[0] = fx
    return h


def to_i32(x):
    x &= 0xFFFFFFFF
    return x - (1 << 32) if x >= 1 << 31 else x


def digits_32(fx, S):
    """The split kernel's form: all in 32 bits for S <= 3; otherwise the low
    three digits from the low 24 bits, their carry into the high part."""
    h = [0] * S

    def step(v):
        d = ((v + 128) & 255) - 128
        return d, (v - d) >> 8
    if S <= 3:
        v = to_i32(fx)
        for p in range(S - 1, 0, -1):
            h[p], v = step(v)
        h[0] = v
        return h
    if S <= 6:
        lo, hi = to_i32(fx & 0xFFFFFF), to_i32(fx >> 24)
        for p in range(S - 1, S - 4, -1):
            h[p], lo = step(lo)
        hi += lo
        for p in range(S - 4, 0, -1):
            h[p], hi = step(hi)
        h[0] = hi
        return h
    # S = 7 (|fx| <= 2^55): three 32-bit parts, the low two of 24 bits, each
    # part's carry joining the next
    lo, mid, top = to_i32(fx & 0xFFFFFF), to_i32((fx >> 24) & 0xFFFFFF), to_i32(fx >> 48)
    for p in range(S - 1, S - 4, -1):
        h[p], lo = step(lo)
    mid += lo
    for p in range(S - 4, S - 7, -1):
        h[p], mid = step(mid)
    top += mid
    for p in range(S - 7, 0, -1):
        h[p], top = step(top)
    h[0] = top
    return h


@pytest.mark.parametrize("S", [2, 3, 4, 5, 6, 7])
def test_digit_split_forms_agree(S):
    lim = 1 << (8 * S - 1)     # |fixed point| <= 2^(8S-1)
    rng = random.Random(S)
    edges = [0, 1, -1, 127, 128, -128, -129, 255, 256, -256, lim, -lim, lim - 1, -lim + 1,
             (1 << 24) - 1, 1 << 24, -(1 << 24), (1 << 24) + 128, -(1 << 24) - 128,
             (1 << 48) - 1, 1 << 48, -(1 << 48), (1 << 48) + (1 << 24) - 128, -(1 << 48) - 129]
    values = [v for v in edges if abs(v) <= lim] + [rng.randint(-lim, lim) for _ in range(20000)]
    for fx in values:
        d64, d32 = digits_64(fx, S), digits_32(fx, S)
        assert d64 == d32, fx
        assert all(abs(d) <= 128 for d in d64), fx          # exact in bf16, |d e| <= 2^14
        assert sum(d * 256 ** (S - 1 - p) for p, d in enumerate(d64)) == fx


def drain_period(t):
    return 32 if t <= 2 else 16 if t == 3 else 8 if t <= 5 else 4 if t <= 9 else 2 if t <= 17 else 1


def test_exact_levels_stay_within_2_24():
    # level t: t-1 products per k, |product| <= 2^14, 32 k per stage
    for t in range(2, 6):
        assert (t - 1) * 32 * drain_period(t) * 2 ** 14 <= 2 ** 24
        p = drain_period(t)
        assert p & (p - 1) == 0 and 2 * p * (t - 1) > 32     # the largest power of two


@pytest.mark.parametrize("S", [2, 3, 4, 5, 6])
def test_restarting_levels_form_one_run(S):
    top = min(S + 1, 5)
    for x in range(1, 4096):
        z = [t for t in range(2, top + 1) if x % drain_period(t) == 0]
        if z:
            assert z == list(range(z[0], top + 1)), (x, z)
            assert x % 8 == 0
