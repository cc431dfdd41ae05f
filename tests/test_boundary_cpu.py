"""CPU checks of the C-ABI boundary and of the shared building blocks (no GPU calls)."""
import re
from pathlib import Path

import numpy as np
import pytest

import oracle as O
import paragraph_gb300 as pg

ROOT = Path(__file__).resolve().parents[1]

# Random123 known-answer vectors for philox4x32_10 (counter, key, output).
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


def declared_symbols() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_loads_and_exports_every_declared_symbol(built):
    lib = pg.load_library()
    decl = declared_symbols()
    assert decl, "no declarations found"
    missing = [s for s in sorted(decl) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(pg.EXPORTED) == decl
    assert b"sm_103a" in lib.pg_version()


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(built, ctr, key, out):
    np.testing.assert_array_equal(O.philox(ctr, key), np.array(out, np.uint32))
    np.testing.assert_array_equal(pg.philox(ctr, key), np.array(out, np.uint32))


def test_philox_host_matches_oracle_random(built):
    rng = np.random.default_rng(0)
    for _ in range(200):
        c = rng.integers(0, 2**32, 4, dtype=np.uint64).astype(np.uint32)
        k = rng.integers(0, 2**32, 2, dtype=np.uint64).astype(np.uint32)
        np.testing.assert_array_equal(O.philox(c, k), pg.philox(c, k))


def _ulp_err32(a, b):
    b = np.float64(b)
    return abs(np.float64(a) - b) / (np.spacing(np.float32(abs(b) if b else 1.0)))


def test_elementary_functions_bit_identical_and_accurate(built):
    lib = pg.load_library()
    rng = np.random.default_rng(1)
    xs = np.exp(rng.uniform(-85, 85, 3000)).astype(np.float32)
    worst = 0.0
    for x in xs:
        a, b = lib.pg_logf_host(float(x)), O.logf(float(x))
        assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)
        worst = max(worst, _ulp_err32(a, np.log(np.float64(x))))
    assert worst <= 2.0, worst
    worst = 0.0
    for x in rng.uniform(-86, 87, 3000).astype(np.float32):
        a, b = lib.pg_expf_host(float(x)), O.expf(float(x))
        assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)
        worst = max(worst, _ulp_err32(a, np.exp(np.float64(x))))
    assert worst <= 2.0, worst
    for x in np.exp(rng.uniform(-700, 700, 2000)):
        a, b = lib.pg_log_host(float(x)), O.log(float(x))
        assert a == b
        assert abs(a - np.log(x)) <= 2 * np.spacing(abs(np.log(x)))
    for x in rng.uniform(-700, 700, 2000):
        a, b = lib.pg_exp_host(float(x)), O.exp(float(x))
        assert a == b
        assert abs(a - np.exp(x)) <= 2 * np.spacing(np.exp(x))
    # special values
    assert lib.pg_logf_host(0.0) == -np.inf and np.isnan(lib.pg_logf_host(-1.0))
    assert lib.pg_expf_host(-100.0) == 0.0 and lib.pg_expf_host(100.0) == np.inf
    assert lib.pg_log_host(1.0) == 0.0 and lib.pg_exp_host(0.0) == 1.0


@pytest.mark.parametrize("lam", [0.0, 1.0, 15.0, 20.0, 30.0, 120.0])
def test_poisson_table_matches_oracle_and_law(built, lam):
    t_pg, t_or = pg.poisson_table(lam), O.poisson_table(lam)
    np.testing.assert_array_equal(t_pg, t_or)
    assert np.all(np.diff(t_pg.astype(np.float64)) >= 0)
    from scipy.stats import poisson

    cdf = t_pg.astype(np.float64) / 2.0**64
    ref = poisson.cdf(np.arange(len(cdf)), lam) if lam > 0 else np.ones(len(cdf))
    assert np.max(np.abs(cdf[:-1] - ref[:-1])) < 1e-12


def test_create_rejects_bad_config_without_gpu_calls(built):
    lib = pg.load_library()
    import ctypes as C

    ctx = C.c_void_p()
    cfg = pg._Config(0, 0, 1, 0, 0, 0, 0)  # zero replicas
    assert lib.pg_create(C.byref(ctx), C.byref(cfg)) == pg.PG_ERR_ARG
    assert lib.pg_status_string(pg.PG_ERR_CAPACITY) == b"capacity exceeded"


def test_fp32_log_error_bound_holds_exhaustively(built):
    """The ER skip decides floor(log(u) / log(1 - p)) from an fp32 estimate whose error bound
    assumes the library's fp32 log is within 2 ulp on [2^-60, 1]; every float there is checked
    (the oracle's copy, which is bit-identical to the library's, computes the maximum)."""
    assert O._load().og_logf_max_ulp(2.0 ** -60, 1.0) < 2.0
    rng = np.random.default_rng(4)
    xs = np.concatenate([rng.random(2000), 2.0 ** -rng.uniform(0, 60, 2000)]).astype(np.float32)
    lib = pg.load_library()
    for x in xs.tolist():
        assert np.float32(lib.pg_logf_host(x)).view(np.uint32) == np.float32(O.logf(x)).view(np.uint32)
