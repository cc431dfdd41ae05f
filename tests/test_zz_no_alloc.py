"""The allocation-free ER entry point, called through the C ABI.

pg_er_generate_noalloc serves callers that cannot allocate device memory when they call the
library (a program that must not call cudaMalloc while it times or captures other GPU work, or a
runtime that only hands out pre-sized buffers).  Its scratch is a fixed array inside the library,
so this test checks that two calls in a row -- the second one reusing the scratch the first one
left behind -- produce exactly the edges the ordinary pg_er_epoch path appends.  Edges are integer
ids, so the comparison is exact.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import paragraph_gb300 as pg
from paragraph_gb300 import GrowthEngine
from paragraph_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _reference_edges(seed, n0, delta, p):
    s = W.er_seed(n0)
    with GrowthEngine(seed=seed) as eng:
        eng.load_graph(s.pub, s.fitness, s.src, s.dst)
        eng.er_epoch(delta, p)
        return eng.last_epoch_edges()


def _noalloc(lib, seed, n0, delta, p, cap):
    torch = pytest.importorskip("torch")
    src = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    dst = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    count = C.c_int64(-1)
    st = lib.pg_er_generate_noalloc(seed, 0, n0, delta, p, C.c_void_p(src.data_ptr()),
                                    C.c_void_p(dst.data_ptr()), cap, C.byref(count), None)
    return st, count.value, src[: max(count.value, 0)].cpu().numpy(), dst[: max(count.value, 0)].cpu().numpy()


def test_noalloc_matches_er_epoch_twice(gpu):
    lib = pg.load_library()
    cases = [(17, 150_000, 3000, 1e-3), (5, 70_000, 1200, 1e-4)]  # second call reuses the scratch
    for seed, n0, delta, p in cases:
        ref_src, ref_dst = _reference_edges(seed, n0, delta, p)
        st, cnt, src, dst = _noalloc(lib, seed, n0, delta, p, cap=len(ref_src) + 1024)
        assert st == pg.PG_OK
        assert cnt == len(ref_src)
        np.testing.assert_array_equal(src, ref_src)
        np.testing.assert_array_equal(dst, ref_dst)


def test_noalloc_allocates_no_device_memory(gpu):
    """After a first call (which looks up the scratch array's address), a call of another shape
    changes neither the device's free memory nor torch's reserved pool: nothing is allocated."""
    torch = pytest.importorskip("torch")
    lib = pg.load_library()
    cap = 400_000
    src = torch.empty(cap, dtype=torch.int32, device="cuda")
    dst = torch.empty(cap, dtype=torch.int32, device="cuda")
    count = C.c_int64(-1)

    def call(seed, n0, delta, p):
        st = lib.pg_er_generate_noalloc(seed, 0, n0, delta, p, C.c_void_p(src.data_ptr()),
                                        C.c_void_p(dst.data_ptr()), cap, C.byref(count), None)
        assert st == pg.PG_OK and 0 < count.value <= cap

    call(9, 90_000, 1500, 1e-3)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    call(10, 260_000, 700, 2e-3)  # more chunks per node, a different task count
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_rejects_oversized_and_small_capacity(gpu):
    lib = pg.load_library()
    count = C.c_int64(-1)
    # delta * ceil(n / 65536) above the scratch limit
    st = lib.pg_er_generate_noalloc(1, 0, 1 << 20, pg_max_tasks() + 1, 1e-6, None, None, 0,
                                    C.byref(count), None)
    assert st == pg.PG_ERR_CAPACITY
    # capacity too small: reports the count and writes nothing
    st, cnt, _, _ = _noalloc(lib, 3, 20_000, 100, 1e-2, cap=10)
    assert st == pg.PG_ERR_CAPACITY and cnt > 10


def pg_max_tasks() -> int:
    return 1 << 18
