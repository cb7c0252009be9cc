"""Host-side checks of the integer invariants the emulated-FP64 kernels rely
on, restated in Python: the balanced base-256 digit split (the 64-bit
recurrence and the biased-byte form the split kernel uses give the same
digits, and the digits rebuild the fixed-point value), and the level restart
periods (every exact level stays within 2^24, restarting levels form one
run of adjacent levels), and the recombination's two integer conversions
(round to odd into a 64-bit window, float to int64 from its bits)."""
import math
import random
import struct

import numpy as np
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


def f32(x):
    """float32 rounding of a Python float (round to nearest even)."""
    return struct.unpack("<f", struct.pack("<f", x))[0]


def digits_bias(fx, S):
    """The split kernel's form: 128 added at each of the S - 1 lower digit
    positions of the 64-bit two's complement value; lower digit q is byte q
    of the sum minus 128, computed as the float (2^23 + byte) - (2^23 + 128)
    (a byte permute into 0x4B0000xx and one float add); the top digit is the
    sum shifted down arithmetically by 8 (S - 1)."""
    bias = 0x8080808080808080 >> (8 * (9 - S))
    u = (fx + bias) & 0xFFFFFFFFFFFFFFFF
    h = [0] * S
    for q in range(S - 1):
        byte = (u >> (8 * q)) & 255
        as_float = struct.unpack("<f", struct.pack("<I", 0x4B000000 | byte))[0]
        d = f32(as_float - 8388736.0)
        assert d == int(d)
        h[S - 1 - q] = int(d)
    top = u - (1 << 64) if u >= 1 << 63 else u
    h[0] = top >> (8 * (S - 1))
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
        d64, dk = digits_64(fx, S), digits_bias(fx, S)
        assert d64 == dk, fx
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


# --- the recombination's conversions -------------------------------------

def window_to_double(hi, lo, SH, e2):
    """The kernel's exact_to_double<SH>: W = hi * 2^SH + lo is cut to a signed
    64-bit window with the bits cut off ORed into its lowest bit (round to
    odd), the window rounded once to double, then scaled by 2^e2 (normal
    results only here)."""
    if SH == 0:
        y, scale = hi + lo, e2
    else:
        H = hi + (lo >> SH)
        r = lo & ((1 << SH) - 1)
        s = 63 - (H ^ (H >> 63)).bit_length()           # redundant sign bits of H (64-bit)
        if s >= SH:
            y, scale = (H << SH) | r, e2
        else:
            d = SH - s
            y = (H << s) | (r >> d) | (1 if r & ((1 << d) - 1) else 0)
            scale = e2 + d
    assert -(1 << 63) <= y < (1 << 63)
    return math.ldexp(float(y), scale) if y else 0.0


@pytest.mark.parametrize("SH", [0, 8, 16, 24, 32])
def test_round_to_odd_window_rounds_correctly(SH):
    """Rounding to odd at 55 bits or more, then to 53, equals one correct
    rounding of the exact value (checked against exact rational arithmetic;
    Python's int / int is correctly rounded)."""
    rng = random.Random(SH)
    for it in range(20000):
        mode = it % 5
        hi = rng.randint(-(1 << 57), 1 << 57) >> rng.randint(0, 57)
        lo = rng.randint(-(1 << 59), 1 << 59) >> rng.randint(0, 59)
        if mode == 1:                                    # cancellation
            hi = rng.randint(-(1 << 26), 1 << 26)
            lo = -(hi << SH) + rng.randint(-(1 << 30), 1 << 30)
        if mode == 2:                                    # ties in the low bits
            lo = (lo >> 12) << 12 | (1 << 11)
        if SH == 0:
            hi = 0 if mode == 3 else hi
        e2 = rng.randint(-900, 800)
        W = (hi << SH) + lo
        got = window_to_double(hi, lo, SH, e2)
        if W == 0:
            assert got == 0.0
            continue
        exact = float(W << e2) if e2 >= 0 else W / (1 << -e2)   # both correctly rounded
        assert got == exact, (hi, lo, e2)


def float_to_int64_from_bits(f32_bits, sh):
    """The 16-warp epilogue's float_to_ll_exact: f * 2^sh for an
    integer-valued float from its bits (mantissa shifted by its exponent)."""
    e = ((f32_bits >> 23) & 0xFF) - 150 + sh
    m = (f32_bits & 0x7FFFFF) | 0x800000
    v = m << e if e >= 0 else m >> min(-e, 31)
    return -v if f32_bits >> 31 else v


@pytest.mark.parametrize("sh", [0, 8, 16, 24, 32])
def test_float_to_int64_from_bits(sh):
    rng = np.random.default_rng(sh)
    # integer-valued floats across every exponent with |f| * 2^sh < 2^62
    mags = np.concatenate([rng.integers(1, 1 << 24, 4000).astype(np.float64),
                           np.ldexp(rng.integers(1 << 23, 1 << 24, 4000).astype(np.float64),
                                    rng.integers(0, 62 - 24 - sh + 1, 4000))])
    vals = np.concatenate([mags, -mags, [0.0, -0.0, 1.0, -1.0, 2.0 ** 24, -(2.0 ** 24)]])
    f32 = vals.astype(np.float32)
    assert np.array_equal(f32.astype(np.float64), vals)       # exactly representable
    for v, b in zip(vals, f32.view(np.uint32)):
        assert float_to_int64_from_bits(int(b), sh) == int(v) << sh, (v, sh)
