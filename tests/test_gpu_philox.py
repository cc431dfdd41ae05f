"""The library's device Philox4x32-10 against the Random123 known answers and against cuRAND's
device generator of the same name (curand_kernel.h, built here from the toolkit's headers).

A small test helper (tests/philox_curand.cu) is compiled for sm_103a at test time: one kernel
draws block q of subsequence s under seed K from cuRAND (curand_init(K, s, 4 q) then curand4) and
the library's philox(counter = (q_lo, q_hi, s_lo, s_hi), key = (K_lo, K_hi)) in the same thread;
another runs the library's philox on the Random123 (counter, key) vectors.  Integer outputs:
compared exactly."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from test_boundary_cpu import PHILOX_KAT

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def helper(gpu, tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    so = tmp_path_factory.mktemp("philox") / "libphilox_xcheck.so"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-o", str(so), str(ROOT / "tests" / "philox_curand.cu")],
                   check=True, capture_output=True)
    return C.CDLL(str(so))


def _p(a):
    return C.c_void_p(a.ctypes.data)


def test_device_philox_known_answers(helper):
    ck = np.array([c + k for c, k, _ in PHILOX_KAT], np.uint32)
    out = np.zeros((len(ck), 4), np.uint32)
    assert helper.philox_raw(len(ck), _p(ck), _p(out)) == 0
    np.testing.assert_array_equal(out, np.array([o for _, _, o in PHILOX_KAT], np.uint32))


def test_device_philox_matches_curand(helper):
    rng = np.random.default_rng(11)
    n = 1 << 14
    seed = rng.integers(0, 1 << 63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n, dtype=np.uint64)
    sub = rng.integers(0, 1 << 63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n, dtype=np.uint64)
    blk = rng.integers(0, 1 << 60, n, dtype=np.uint64)
    # small and edge values too: the engine's counters hold small draw indices
    seed[:4] = [0, 42, (1 << 32) - 1, (1 << 64) - 1]
    sub[:4] = [0, 1, 1 << 32, (1 << 64) - 1]
    blk[:4] = [0, 1, 2, (1 << 32) + 5]
    out_c = np.zeros((n, 4), np.uint32)
    out_p = np.zeros((n, 4), np.uint32)
    assert helper.philox_xcheck(n, _p(seed), _p(sub), _p(blk), _p(out_c), _p(out_p)) == 0
    np.testing.assert_array_equal(out_p, out_c)
