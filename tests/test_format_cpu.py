"""C's "%.<P>g" conversion that the attribute writer runs on the device, compiled for the host
(pg_format_g_host), against Python's own "%.<P>g" (correctly rounded, round-half-even at exact
ties, like the C library).  Covers random bit patterns over the whole double range (normal and
subnormal), the value ranges of the attribute columns (weights and alpha in (0, 1], fp32 fitness),
exact ties at the tenth digit, powers of ten and their neighbours, zero, infinities."""
import ctypes as C
import math
import struct

import numpy as np
import pytest

from paragraph_gb300 import load_library


@pytest.fixture(scope="module")
def fmt(built):
    lib = load_library()
    f = lib.pg_format_g_host
    f.restype = C.c_int32
    f.argtypes = [C.c_double, C.c_int32, C.c_char_p]
    buf = C.create_string_buffer(64)

    def run(x: float, p: int) -> str:
        n = f(x, p, buf)
        return buf.raw[:n].decode()
    return run


def _check(fmt, values, prec):
    bad = [(v, fmt(v, prec), f"%.{prec}g" % v) for v in values if fmt(v, prec) != f"%.{prec}g" % v]
    assert not bad, bad[:10]


def test_random_bit_patterns(fmt):
    rng = np.random.default_rng(1)
    bits = rng.integers(0, 2**63, size=40_000, dtype=np.uint64) | (rng.integers(0, 2, 40_000, dtype=np.uint64) << 63)
    vals = [v for v in bits.view(np.float64).tolist() if math.isfinite(v)]
    for p in (1, 6, 9, 10, 13):
        _check(fmt, vals[:8000], p)


def test_attribute_column_ranges(fmt):
    rng = np.random.default_rng(2)
    weights = rng.random(30_000)
    weights = np.concatenate([weights, weights / weights.sum(), rng.random(2000) ** 8, [1.0, 0.5, -1.0]])
    _check(fmt, weights.tolist(), 10)
    fit = rng.lognormal(0.0, 1.0, 30_000).astype(np.float32).astype(np.float64)
    _check(fmt, fit.tolist(), 9)
    _check(fmt, np.arange(1, 1001, dtype=np.float64).tolist(), 9)


def test_ties_powers_and_specials(fmt):
    ties = [1234567890.5, 1234567891.5, 0.5, 2.5, 1e10 + 0.5, 9999999999.5, 12345.678905, 1.5e-5, 2.5e-7]
    pows = []
    for k in range(-320, 309):
        x = float(f"1e{k}")
        pows += [x, math.nextafter(x, 0.0), math.nextafter(x, math.inf)]
    specials = [0.0, -0.0, math.inf, -math.inf, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                123456789012.0, 0.0001, 0.00009999999999, 1e-5, 99999.99999]
    for p in (9, 10):
        _check(fmt, ties + pows + specials, p)


def test_nan_prints_like_the_c_library(fmt):
    nan = struct.unpack("<d", struct.pack("<Q", 0x7FF8000000000000))[0]
    neg_nan = struct.unpack("<d", struct.pack("<Q", 0xFFF8000000000000))[0]
    assert fmt(nan, 10) == "nan" and fmt(neg_nan, 10) == "-nan"
