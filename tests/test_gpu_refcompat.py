"""Refcompat functor (ParAGraph's own per-paper model) on the GPU against the CPU restatement.

The scores use exact 128-bit integer sums, the keys and the uniform fill the same Philox streams,
so the bar is bit-exact: both CSRs, in-degrees, new-paper attributes, citations in arrival order,
the per-paper draws (weights, alpha, generator, out-degree) and the counters."""
import re
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import PG_WEIGHTS_REFCOMPAT, GrowthEngine, PAParams, PGError, RCParams
from paragraph_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run_both(g, rc, bag, rec, epochs, seed=77, planted=None):
    eng = GrowthEngine(seed=seed, record_trace=True, weight_model=PG_WEIGHTS_REFCOMPAT)
    eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(growth_rate=rc.growth_rate),
                   planned_epochs=epochs)
    eng.rc_configure(rc, bag, rec)
    og = O.OracleGraph(seed, 0)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.rc_configure(rc, bag, rec)
    if planted is not None:
        first, lag, peak, dur = planted
        eng.rc_set_nodes(first, lag, peak, dur)
        og.rc_set_nodes(first, lag, peak, dur)
    return eng, og


def _engine_constant(name):
    src = (Path(__file__).resolve().parents[1] / "paragraph_gb300" / "csrc" / "pg_engine.cuh").read_text()
    return int(re.search(rf"constexpr int {name} = (\d+);", src).group(1))


# cut-offs of the CTA-wide 2-hop pass: generator row entries, entries of the generator's rows' rows
_BIG_GD, _BIG_STREAM = _engine_constant("kRcBigGd"), _engine_constant("kRcBigStream")


def _row_stats(og):
    """Per node of the current graph: row entries and the length of its 2-hop stream."""
    ind, outd = og.degrees()
    deg = (ind + outd).astype(np.int64)
    stream = np.zeros(len(deg), np.int64)
    for which in (0, 1):
        off, col = og.csr(which)
        np.add.at(stream, np.repeat(np.arange(len(off) - 1), np.diff(off)), deg[col])
    return deg, stream


def _compare(eng, og):
    assert eng.counts() == (og.n, og.m)
    for which in (0, 1):
        a, b = eng.csr(which), og.csr(which)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(eng.degrees()[0], og.degrees()[0])
    pg_, fg = eng.nodes()
    po, fo = og.nodes()
    np.testing.assert_array_equal(pg_, po)
    np.testing.assert_array_equal(fg.view(np.uint32), fo.view(np.uint32))


@pytest.mark.parametrize("case", [
    dict(n0=3000, growth=0.05, same_year=0.1, w=(-1, -1, -1), alpha=-1.0, epochs=3),
    dict(n0=3000, growth=0.1, same_year=0.0, w=(1.0, 1.0, 1.0), alpha=0.5, epochs=2),
    dict(n0=400, growth=0.25, same_year=0.3, w=(2.0, 0.0, 1.0), alpha=1.0, epochs=3),
    dict(n0=40, growth=0.5, same_year=0.5, w=(-1, -1, -1), alpha=0.0, epochs=4),
])
def test_refcompat_bit_exact(gpu, case):
    g = W.rc_seed(case["n0"], 10, seed=3)
    bag, rec = W.rc_tables(seed=5)
    rc = RCParams(pa_weight=case["w"][0], rec_weight=case["w"][1], fit_weight=case["w"][2],
                  alpha=case["alpha"], same_year=case["same_year"], growth_rate=case["growth"])
    eng, og = _run_both(g, rc, bag, rec, case["epochs"])
    routes = np.zeros(2, np.int64)  # agents with a 2-hop stream: one warp, a CTA
    with eng:
        for _ in range(case["epochs"]):
            deg, stream = _row_stats(og)
            nn, ne = eng.grow_epoch()
            og.rc_epoch()
            ag = og.rc_agents()
            gen = ag[ag[:, 5] >= 2, 4].astype(np.int64)
            cta = (deg[gen] >= _BIG_GD) | (stream[gen] >= _BIG_STREAM)
            routes += (int((~cta).sum()), int(cta.sum()))
            assert ne == og.epoch_edges()[1]
            np.testing.assert_array_equal(eng.arrivals(), og.arrivals())
            np.testing.assert_array_equal(eng.rc_agents(), og.rc_agents())
            st, so = eng.stats(), og.stats()
            for k in ("rows_expanded", "elems_streamed", "draws", "nodes_weighted"):
                assert st[k] == so[k], k
            _compare(eng, og)
    if case["n0"] >= 400:
        assert routes.min() > 0, routes  # both routes of the 2-hop walk were checked


def test_refcompat_long_generator_rows_bit_exact(gpu):
    """Generators with 32 or more row entries, or whose rows' rows hold 1024 or more entries: their
    agents' 2-hop streams are walked by a whole CTA (warps splitting each group's stream by 32-entry
    chunks, their top lists merged) before the agent kernel."""
    base = W.rc_seed(3000, 10, seed=4)
    rng = np.random.default_rng(8)
    pop = rng.choice(3000, 400, replace=False)
    extra = rng.integers(60, 260, size=400)
    src = np.concatenate([base.src] + [rng.integers(0, 3000, size=d).astype(np.int32) for d in extra])
    dst = np.concatenate([base.dst] + [np.full(d, v, np.int32) for v, d in zip(pop, extra)])
    keep = src != dst
    g = W.SeedGraph(base.pub, base.fitness, src[keep], dst[keep])
    bag, rec = W.rc_tables(seed=6, bag_mean=30.0)
    rc = RCParams(growth_rate=0.08, same_year=0.1)
    eng, og = _run_both(g, rc, bag, rec, 3)
    with eng:
        for _ in range(3):
            eng.grow_epoch()
            og.rc_epoch()
            np.testing.assert_array_equal(eng.arrivals(), og.arrivals())
            np.testing.assert_array_equal(eng.rc_agents(), og.rc_agents())
            st, so = eng.stats(), og.stats()
            for k in ("rows_expanded", "elems_streamed", "draws"):
                assert st[k] == so[k], k
            _compare(eng, og)
        ind, outd = eng.degrees()
        gens = eng.rc_agents()[:, 4].astype(np.int64)
        assert ((ind + outd)[gens] >= _BIG_GD).sum() > 10  # the CTA-wide path was taken


def test_refcompat_planted_papers_and_checkpoint(gpu):
    g = W.rc_seed(2000, 8, seed=9)
    bag, rec = W.rc_tables(seed=2, bag_mean=20.0)
    rc = RCParams(growth_rate=0.05, same_year=0.2)
    planted = (100, np.full(50, 1, np.int32), np.full(50, 900, np.int32), np.full(50, 2, np.int32))
    eng, og = _run_both(g, rc, bag, rec, 4, planted=planted)
    with eng:
        eng.grow_epoch()
        og.rc_epoch()
        eng.checkpoint()
        for _ in range(2):
            eng.grow_epoch()
            og.rc_epoch()
        _compare(eng, og)
        first = eng.csr(0)
        eng.restore()
        for _ in range(2):
            eng.grow_epoch()
        again = eng.csr(0)
        np.testing.assert_array_equal(first[1], again[1])


def test_refcompat_needs_configuration(gpu):
    g = W.rc_seed(500, 5, seed=1)
    with GrowthEngine(seed=1, weight_model=PG_WEIGHTS_REFCOMPAT) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(growth_rate=0.1), planned_epochs=1)
        with pytest.raises(PGError):
            eng.grow_epoch()
        with pytest.raises(PGError):
            eng.rc_configure(RCParams(gamma=7), [10, 12], [1.0])
