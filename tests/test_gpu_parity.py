"""GPU engine vs CPU oracle, through the C ABI.

Everything here is integer or index work on the same Philox streams and the same fixed-point CDF,
so the bar is bit-exact: forward/backward CSR, in-degrees, new-node attributes, citation choices
(sorted rows and arrival order) and the byte-model counters must be identical.
"""
import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import (PG_ERR_CAPACITY, PG_SAMPLER_ENUMERATE, PG_SAMPLER_THINNING, GrowthEngine, PGError,
                             PAParams, ReplicaInput)
from paragraph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
SAMPLERS = [PG_SAMPLER_THINNING, PG_SAMPLER_ENUMERATE]


def _oracle_for(g, params: PAParams, seed: int, replica: int = 0, sampler: int = 0):
    og = O.OracleGraph(seed, replica)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.set_params(**params.__dict__)
    og.set_sampler(sampler)
    return og


def _compare_state(eng: GrowthEngine, og: O.OracleGraph, replica: int = 0):
    n, m = eng.counts(replica)
    assert (n, m) == (og.n, og.m)
    for which in (0, 1):
        off_g, col_g = eng.csr(which, replica)
        off_o, col_o = og.csr(which)
        np.testing.assert_array_equal(off_g, off_o, err_msg=f"offsets which={which}")
        np.testing.assert_array_equal(col_g, col_o, err_msg=f"columns which={which}")
    ig, og_ = eng.degrees(replica)
    io, oo = og.degrees()
    np.testing.assert_array_equal(ig, io)
    np.testing.assert_array_equal(og_, oo)
    pg_, fg = eng.nodes(replica)
    po, fo = og.nodes()
    np.testing.assert_array_equal(pg_, po)
    np.testing.assert_array_equal(fg.view(np.uint32), fo.view(np.uint32))


@pytest.mark.parametrize("sampler", SAMPLERS)
@pytest.mark.parametrize("n0,delta,lam,beta", [(300, 40, 4.0, 4.0), (2000, 500, 15.0, 4.0),
                                               (2000, 500, 15.0, 1.0), (64, 64, 30.0, 8.0),
                                               (12, 30, 60.0, 8.0)])
def test_pa_small_bit_exact(gpu, sampler, n0, delta, lam, beta):
    g = W.plain_pa_seed(n0, 10, seed=7)
    prm = PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=beta, mean_out_degree=lam,
                   growth_rate=0.0, fixed_new_nodes=delta, num_anchors=3)
    with GrowthEngine(seed=1234, record_trace=True, sampler=sampler) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=3)
        og = _oracle_for(g, prm, 1234, sampler=sampler)
        for _ in range(3):
            nn, ne = eng.grow_epoch()
            og.pa_epoch()
            assert nn == delta
            assert ne == og.epoch_edges()[1]
            np.testing.assert_array_equal(eng.arrivals(), og.arrivals())
            st, so = eng.stats(), og.stats()
            for k in ("nodes_weighted", "rows_expanded", "elems_streamed", "draws"):
                assert st[k] == so[k], k
            if sampler == PG_SAMPLER_THINNING:
                assert st["adj_scanned"] == so["adj_scanned"]
            _compare_state(eng, og)


@pytest.mark.parametrize("sampler", SAMPLERS)
def test_plain_pa_config_bit_exact(gpu, sampler):
    """Plain PA growth: 10k seed DAG, 3 epochs x 5,000 agents, Poisson(15), 3 anchors."""
    g = W.plain_pa_seed(10_000, 10, seed=42)
    prm = W.plain_pa_params()
    with GrowthEngine(seed=42, sampler=sampler) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=3)
        og = _oracle_for(g, prm, 42, sampler=sampler)
        for _ in range(3):
            eng.grow_epoch()
            og.pa_epoch()
            s_g, d_g = eng.last_epoch_edges()
            s_o, d_o = og.last_epoch_edges()
            np.testing.assert_array_equal(s_g, s_o)
            np.testing.assert_array_equal(d_g, d_o)
        _compare_state(eng, og)


# at n0 = 20,000 these p give 0.2 .. 20 expected successes per chunk: every lane-group width of
# the walk (1, 2, 4, 8, 16, 32 lanes per task) is exercised
@pytest.mark.parametrize("p", [1e-5, 1e-4, 2e-4, 4e-4, 7e-4, 1e-3, 0.0, 1.0])
def test_er_bit_exact(gpu, p):
    n0, delta = (20_000, 2000) if p < 1.0 else (3000, 50)
    s = W.er_seed(n0)
    with GrowthEngine(seed=99) as eng:
        eng.load_graph(s.pub, s.fitness, s.src, s.dst)
        og = O.OracleGraph(99, 0)
        og.load(s.pub, s.fitness, s.src, s.dst)
        for _ in range(2):
            ne = eng.er_epoch(delta, p)
            og.er_epoch(delta, p)
            assert ne == og.epoch_edges()[1]
        _compare_state(eng, og)
        if p == 1.0:
            assert og.m == delta * n0 + delta * (n0 + delta)


@pytest.mark.parametrize("p", [2e-4, 1e-3, 5e-3])
def test_er_overflow_pass_bit_exact(gpu, p):
    """Each ER walk writes its edges into slots reserved for its binomial count; with the
    reservation cut to one standard deviation (er_slot_sigmas=1) a few per cent of the walks have
    more edges than slots and finish in the overflow pass.  The edges are still the oracle's, bit
    for bit, and this test checks that walks did overflow."""
    n0, delta = 100_000, 2000
    s = W.er_seed(n0)
    with GrowthEngine(seed=17) as eng:
        eng.load_graph(s.pub, s.fitness, s.src, s.dst)
        eng.set_tuning(er_slot_sigmas=1)
        og = O.OracleGraph(17, 0)
        og.load(s.pub, s.fitness, s.src, s.dst)
        over = 0
        for _ in range(2):
            n = og.n
            ne = eng.er_epoch(delta, p)
            og.er_epoch(delta, p)
            assert ne == og.epoch_edges()[1]
            src, dst = og.last_epoch_edges()
            np.testing.assert_array_equal(eng.last_epoch_edges()[1], dst)
            # the slots of each (new node, 2^16-id chunk) walk, as the engine reserves them
            chunk = 1 << 16
            lens = np.minimum(chunk, n - chunk * np.arange((n + chunk - 1) // chunk))
            mu = lens * p
            slots = np.minimum(lens, np.ceil(mu + np.sqrt(mu * (1 - p))) + 8)
            per = np.zeros((delta, len(lens)), np.int64)
            np.add.at(per, (src - n, dst // chunk), 1)
            over += int((per > slots[None, :]).sum())
        _compare_state(eng, og)
    assert over > 0


def _popular_seed(n: int, popular: int, lo: int, hi: int, seed: int) -> W.SeedGraph:
    """Sparse background (4 random citations per node) plus `popular` nodes cited by lo..hi
    random others: more than 256 nodes with rows longer than the shared frontier, so many are
    not hubs."""
    rng = np.random.default_rng(seed)
    src = [rng.integers(0, n, size=4 * n)]
    dst = [rng.integers(0, n, size=4 * n)]
    for v, d in zip(rng.choice(n, popular, replace=False), rng.integers(lo, hi, size=popular)):
        src.append(rng.integers(0, n, size=d))
        dst.append(np.full(d, v))
    src, dst = np.concatenate(src), np.concatenate(dst)
    keep = src != dst
    return W.SeedGraph(rng.integers(-5, 0, size=n).astype(np.int32),
                       rng.lognormal(0.0, 1.0, size=n).astype(np.float32),
                       src[keep].astype(np.int32), dst[keep].astype(np.int32))


@pytest.mark.parametrize("small_hash", [0, 1])
def test_large_anchor_rows_bit_exact(gpu, small_hash):
    """Agents whose anchors' rows overflow the shared frontier (1,024 entries, 512 with the small
    hash): membership in those rows is a binary search of the CSR rows; such agents are also the
    ones the setup lists first."""
    g = _popular_seed(6000, 2000, 1000, 3000, seed=5)
    prm = PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=20.0,
                   growth_rate=0.0, fixed_new_nodes=300, num_anchors=3)
    with GrowthEngine(seed=77, record_trace=True) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=2)
        eng.set_tuning(small_hash=small_hash)
        og = _oracle_for(g, prm, 77, sampler=PG_SAMPLER_THINNING)
        over = 0
        for _ in range(2):
            ind, outd = eng.degrees()
            deg = ind.astype(np.int64) + outd
            eng.grow_epoch()
            og.pa_epoch()
            anc = eng.anchors()[:, :3]
            over += int((deg[anc].sum(axis=1) > 1024).sum())
            st, so = eng.stats(), og.stats()
            assert st["adj_scanned"] == so["adj_scanned"]
            np.testing.assert_array_equal(eng.arrivals(), og.arrivals())
            _compare_state(eng, og)
        assert over > 0  # some agents' anchor rows exceed the shared frontier


def test_er_reserve_keeps_results(gpu):
    """Capacity reserved up front (no arena growth between epochs) changes no edge."""
    s = W.er_seed(20_000)
    runs = []
    for reserve in (False, True):
        with GrowthEngine(seed=7) as eng:
            eng.load_graph(s.pub, s.fitness, s.src, s.dst)
            n0, m0 = eng.counts()
            if reserve:
                eng.reserve(n0 + 3 * 2000, m0 + 3 * 2000 * 26_000)
                eng.reserve(10, 10)  # already large enough: no-op
            for _ in range(3):
                eng.er_epoch(2000, 1e-3)
            runs.append(eng.csr(0))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])


def test_run_epochs_graph_matches_sequential(gpu):
    g = W.plain_pa_seed(3000, 10, seed=3)
    prm = PAParams(mean_out_degree=12.0, growth_rate=0.05, fixed_new_nodes=0)
    with GrowthEngine(seed=5) as a, GrowthEngine(seed=5) as b:
        a.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=6)
        b.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=6)
        for _ in range(6):
            a.grow_epoch()
        b.run_epochs(6, use_graph=True)
        for which in (0, 1):
            for x, y in zip(a.csr(which), b.csr(which)):
                np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("epoch_kernel", [0, 1])
def test_replicas_match_independent_oracles(gpu, epoch_kernel):
    """Replicas of one context, grown by the sequence of stage kernels or by one persistent kernel
    per epoch, each equal the oracle grown alone."""
    reps = W.ensemble_inputs(replicas=5, lo=500, hi=4000, epochs=3, seed=11)
    with GrowthEngine(seed=77, replicas=len(reps)) as eng:
        eng.load_replicas(reps)
        eng.set_tuning(epoch_kernel=epoch_kernel)
        ogs = []
        for r, ri in enumerate(reps):
            og = O.OracleGraph(77, r)
            og.load(ri.pub_epoch, ri.fitness, ri.src, ri.dst)
            og.set_params(**ri.params.__dict__)
            ogs.append(og)
        for _ in range(3):
            eng.grow_epoch()
            for og in ogs:
                og.pa_epoch()
        for r, og in enumerate(ogs):
            _compare_state(eng, og, replica=r)


def test_hub_index_carried_over_epochs(gpu):
    """The hub index is kept from epoch to epoch and only the hubs that change are moved.  On this
    seed (300k nodes, Pareto(1.5) in-degrees, 5 % growth) nodes pass degree 1024 and join the hub
    set every epoch, and at epoch 5 more than 256 nodes have passed it, so the threshold doubles and
    about 170 hubs leave at once.  Every epoch's counters, arrivals and CSRs equal the oracle's; a
    restore at epoch 3 (which makes the next epoch rebuild the index) regrows the same graph."""
    g = W.pareto_seed(300_000, 1.5, 16.0, seed=3)
    prm = PAParams(mean_out_degree=30.0, growth_rate=0.05, fixed_new_nodes=0)
    counts = []
    with GrowthEngine(seed=5, record_trace=True) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=7)
        og = _oracle_for(g, prm, 5, sampler=PG_SAMPLER_THINNING)
        for e in range(7):
            ind, outd = eng.degrees()
            deg = ind.astype(np.int64) + outd
            counts.append(int((deg >= 1024).sum()))
            if e == 3:
                eng.checkpoint()
            eng.grow_epoch()
            og.pa_epoch()
            st, so = eng.stats(), og.stats()
            for k in ("nodes_weighted", "rows_expanded", "draws", "adj_scanned"):
                assert st[k] == so[k], (e, k)
            np.testing.assert_array_equal(eng.arrivals(), og.arrivals())
        _compare_state(eng, og)
        final = [eng.csr(w) for w in (0, 1)]
        eng.restore()
        eng.run_epochs(4, use_graph=True)
        for (o1, c1), (o2, c2) in zip(final, [eng.csr(w) for w in (0, 1)]):
            np.testing.assert_array_equal(o1, o2)
            np.testing.assert_array_equal(c1, c2)
        og.close()
    assert counts[0] < counts[1] < counts[4] <= 256 < counts[5], counts


def test_checkpoint_restore_regrows_identically(gpu):
    g = W.plain_pa_seed(4000, 10, seed=9)
    prm = PAParams(mean_out_degree=20.0, growth_rate=0.03, fixed_new_nodes=0)
    with GrowthEngine(seed=8) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=8)
        eng.checkpoint()
        e1 = eng.run_epochs(8, use_graph=True)
        a = [eng.csr(w) for w in (0, 1)]
        eng.restore()
        assert eng.counts() == (g.n, len(set(zip(g.src.tolist(), g.dst.tolist()))))
        e2 = eng.run_epochs(8, use_graph=True)  # replays the captured graph
        assert e1 == e2
        for (o1, c1), (o2, c2) in zip(a, [eng.csr(w) for w in (0, 1)]):
            np.testing.assert_array_equal(o1, o2)
            np.testing.assert_array_equal(c1, c2)
        st = eng.stats()
        assert st["run_epochs"] == 8 and st["run_new_edges"] == e2
        assert st["run_kernel_launches"] == 8 * (18 + 8)  # thinning adds the guide table and hub index
        # the same run as one persistent kernel per epoch: same graph, one launch per epoch
        eng.set_tuning(epoch_kernel=1)
        eng.restore()
        assert eng.run_epochs(8, use_graph=True) == e1
        for (o1, c1), (o2, c2) in zip(a, [eng.csr(w) for w in (0, 1)]):
            np.testing.assert_array_equal(o1, o2)
            np.testing.assert_array_equal(c1, c2)
        assert eng.stats()["run_kernel_launches"] == 8


def test_tuning_never_changes_results(gpu):
    """Every launch shape the tuner may pick gives the same graph, and autotune leaves the graph
    exactly as it found it."""
    reps = W.ensemble_inputs(replicas=6, lo=2000, hi=20000, epochs=4, seed=21)
    tunings = [dict(), dict(agent_ctas_per_sm=2), dict(small_hash=1),
               dict(small_hash=1, agent_ctas_per_sm=3, copy_ctas_per_sm=4),
               dict(copy_ctas_per_sm=16), dict(epoch_kernel=1)]
    ref = None
    with GrowthEngine(seed=31, replicas=len(reps)) as eng:
        eng.load_replicas(reps)
        eng.checkpoint()
        for t in tunings:
            eng.restore()
            eng.set_tuning(**t)
            eng.run_epochs(4, use_graph=True)
            got = [eng.csr(w, r) for r in range(len(reps)) for w in (0, 1)]
            if ref is None:
                ref = got
                continue
            for (o1, c1), (o2, c2) in zip(ref, got):
                np.testing.assert_array_equal(o1, o2)
                np.testing.assert_array_equal(c1, c2)
        eng.restore()
        before = [eng.csr(0, r) for r in range(len(reps))]
        best, ms = eng.autotune(2)
        assert ms > 0 and best["small_hash"] in (0, 1)
        assert eng.tuning() == best
        for r, (o1, c1) in enumerate(before):
            o2, c2 = eng.csr(0, r)
            np.testing.assert_array_equal(o1, o2)
            np.testing.assert_array_equal(c1, c2)
        # the caller's checkpoint survives the tuner
        eng.run_epochs(4, use_graph=True)
        eng.restore()
        for r, (o1, c1) in enumerate(before):
            np.testing.assert_array_equal(eng.csr(0, r)[1], c1)


def test_single_replica_context_reproduces_batched_replica(gpu):
    """replica_base lets a one-replica context draw as replica i of a batched one, so the serial
    loop and the batched ensemble grow identical graphs."""
    reps = W.ensemble_inputs(replicas=4, lo=1000, hi=8000, epochs=3, seed=5)
    with GrowthEngine(seed=13, replicas=len(reps)) as batched:
        batched.load_replicas(reps)
        batched.run_epochs(3, use_graph=True)
        for i, ri in enumerate(reps):
            with GrowthEngine(seed=13, replica_base=i) as one:
                one.load_replicas([ri])
                one.run_epochs(3, use_graph=True)
                for w in (0, 1):
                    for x, y in zip(batched.csr(w, i), one.csr(w, 0)):
                        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("n", [1500, 50_000, 300_001])
def test_device_seed_load_matches_host_construction(gpu, n):
    """The seed CSRs are built on the device (radix sort, duplicate removal, transpose); they equal
    the oracle's host construction, including duplicate edges, self-loops and isolated nodes, node
    counts whose id width is not a multiple of the 8-bit digit, and graphs larger than one sort
    tile per pass."""
    rng = np.random.default_rng(5)
    src = rng.integers(0, n, 6 * n).astype(np.int32)
    dst = rng.integers(0, n, 6 * n).astype(np.int32)
    src = np.concatenate([src, src[:1000], np.arange(10, dtype=np.int32)])   # duplicates, self-loops
    dst = np.concatenate([dst, dst[:1000], np.arange(10, dtype=np.int32)])
    pub = rng.integers(-5, 0, n).astype(np.int32)
    fit = rng.lognormal(0, 1, n).astype(np.float32)
    with GrowthEngine(seed=1) as eng:
        eng.load_graph(pub, fit, src, dst, PAParams(fixed_new_nodes=100), planned_epochs=1)
        og = O.OracleGraph(1, 0)
        og.load(pub, fit, src, dst)
        _compare_state(eng, og)
        tiny = GrowthEngine(seed=1)
        tiny.load_graph(pub[:3], fit[:3], np.zeros(0, np.int32), np.zeros(0, np.int32),
                        PAParams(fixed_new_nodes=2), planned_epochs=1)
        assert tiny.counts() == (3, 0)
        tiny.close()
        before = eng.counts()
        with pytest.raises(PGError, match="out of range at index 1"):
            eng.load_graph(pub, fit, np.array([0, n], np.int32), np.array([1, 2], np.int32))
        # the rejected edge list left the loaded graph as it was
        assert eng.counts() == before
        _compare_state(eng, og)


def test_bad_edge_in_one_replica_leaves_the_loaded_replicas(gpu):
    """All replicas' raw edges are staged and checked on the device before the arena is rebuilt: an
    endpoint out of range in one replica is reported with its index and replica, and the replicas
    loaded before stay as they were."""
    import dataclasses

    reps = W.ensemble_inputs(replicas=3, lo=500, hi=2000, epochs=1, seed=4)
    with GrowthEngine(seed=2, replicas=3) as eng:
        eng.load_replicas(reps)
        before = [eng.csr(w, r) for r in range(3) for w in (0, 1)]
        dst = reps[1].dst.copy()
        dst[5] = len(reps[1].pub_epoch)  # one past the last node
        bad = list(reps)
        bad[1] = dataclasses.replace(reps[1], dst=dst)
        with pytest.raises(PGError, match="out of range at index 5 of replica 1"):
            eng.load_replicas(bad)
        for (o1, c1), (o2, c2) in zip(before, [eng.csr(w, r) for r in range(3) for w in (0, 1)]):
            np.testing.assert_array_equal(o1, o2)
            np.testing.assert_array_equal(c1, c2)
        eng.run_epochs(1)  # still usable


def test_page_locked_edge_lists_load_like_pageable_ones(gpu):
    """Edge lists in page-locked host memory are read by the device directly (the others are
    copied first): a mix of both loads to the same CSRs as pageable lists, and a bad endpoint in a
    page-locked list is reported with its index and replica."""
    import dataclasses

    torch = pytest.importorskip("torch")

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    reps = W.ensemble_inputs(replicas=4, lo=500, hi=3000, epochs=1, seed=8)
    mixed = [dataclasses.replace(r, src=pinned(r.src), dst=pinned(r.dst)) if i % 2 == 0 else r
             for i, r in enumerate(reps)]
    with GrowthEngine(seed=2, replicas=4) as a, GrowthEngine(seed=2, replicas=4) as b:
        a.load_replicas(reps)
        b.load_replicas(mixed)
        for r in range(4):
            for w in (0, 1):
                (o1, c1), (o2, c2) = a.csr(w, r), b.csr(w, r)
                np.testing.assert_array_equal(o1, o2)
                np.testing.assert_array_equal(c1, c2)
        dst = mixed[2].dst.copy()  # a page-locked copy of replica 2's targets
        dst = pinned(dst)
        dst[7] = -1
        bad = list(mixed)
        bad[2] = dataclasses.replace(mixed[2], dst=dst)
        with pytest.raises(PGError, match="out of range at index 7 of replica 2"):
            b.load_replicas(bad)
        b.run_epochs(1)  # the loaded replicas are still usable


@pytest.mark.parametrize("pinned,replicas,epoch_kernel", [(True, 1, 0), (False, 3, 0), (True, 3, 1)])
def test_run_epochs_out_streams_every_citation(gpu, pinned, replicas, epoch_kernel):
    """pg_run_epochs_out delivers every new citation, epoch by epoch and replica by replica, into
    the caller's buffers: written from the device during the run when they are page-locked, read
    back after the run otherwise.  Each (epoch, replica) block equals that replica's new forward
    rows of the epoch."""
    reps = W.ensemble_inputs(replicas=replicas, lo=2000, hi=8000, epochs=4, seed=12)
    cap = 400_000
    if pinned:
        torch = pytest.importorskip("torch")
        out = (torch.empty(cap, dtype=torch.int32).pin_memory().numpy(),
               torch.empty(cap, dtype=torch.int32).pin_memory().numpy())
    else:
        out = (np.empty(cap, np.int32), np.empty(cap, np.int32))
    with GrowthEngine(seed=6, replicas=replicas) as eng:
        eng.load_replicas(reps)
        eng.set_tuning(epoch_kernel=epoch_kernel)
        n0 = [eng.counts(r)[0] for r in range(replicas)]
        m0 = [eng.counts(r)[1] for r in range(replicas)]
        ne, counts = eng.run_epochs_out(4, out)
        assert ne == counts.sum() > 0
        pos = 0
        done = list(m0)
        for e in range(4):
            for r in range(replicas):
                k = int(counts[e, r])
                s_ref, d_ref = eng.edges(done[r], k, r)
                np.testing.assert_array_equal(out[0][pos:pos + k], s_ref)
                np.testing.assert_array_equal(out[1][pos:pos + k], d_ref)
                assert (s_ref >= n0[r]).all()
                done[r] += k
                pos += k
        assert pos == ne
        assert done == [eng.counts(r)[1] for r in range(replicas)]


def test_run_epochs_out_reports_short_buffers(gpu):
    """Buffers too small for the run: the epochs that fit are written, the rest are grown but not
    written, the call reports PG_ERR_CAPACITY, and the context stays usable."""
    g = W.plain_pa_seed(4000, 10, seed=2)
    prm = PAParams(mean_out_degree=20.0, growth_rate=0.05, fixed_new_nodes=0)
    out = (np.empty(5000, np.int32), np.empty(5000, np.int32))  # about one epoch's citations
    with GrowthEngine(seed=3) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=5)
        m0 = eng.counts()[1]
        with pytest.raises(PGError) as err:
            eng.run_epochs_out(4, out)
        assert err.value.status == PG_ERR_CAPACITY
        m1 = eng.counts()[1]
        assert m1 > m0 + 5000  # all four epochs were grown
        first = eng.edges(m0, 2000)
        np.testing.assert_array_equal(out[0][:2000], first[0])
        np.testing.assert_array_equal(out[1][:2000], first[1])
        eng.grow_epoch()  # not poisoned
        assert eng.counts()[1] > m1


def test_edges_into_caller_buffers(gpu):
    g = W.plain_pa_seed(2000, 5, seed=2)
    with GrowthEngine(seed=3) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(fixed_new_nodes=300), planned_epochs=1)
        eng.grow_epoch()
        f, c = eng.epoch_edges()
        a = eng.edges(f, c)
        buf = (np.empty(c + 7, np.int32), np.empty(c + 7, np.int32))
        b = eng.edges(f, c, out=buf)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


def test_format_edges_text(gpu):
    """The device text writer prints every edge as "ids[source],ids[target]\\n" in forward-CSR
    order, for large, small and negative ids."""
    g = W.plain_pa_seed(3000, 5, seed=8)
    with GrowthEngine(seed=4) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(fixed_new_nodes=500), planned_epochs=1)
        eng.grow_epoch()
        n, m = eng.counts()
        ids = 10**12 + 7 * np.arange(n, dtype=np.int64) - 5
        ids[0], ids[3], ids[7] = 0, -42, 9
        txt = eng.format_edges(ids)
        off, col = eng.csr(0)
        src = np.repeat(np.arange(n), np.diff(off))
        expect = "".join(f"{ids[s]},{ids[d]}\n" for s, d in zip(src, col)).encode()
        assert txt == expect
        with pytest.raises(PGError):
            eng.format_edges(ids[:-1])


@pytest.mark.parametrize("peak_integer", [False, True])
def test_format_attributes_text(gpu, peak_integer):
    """The device attribute writer prints the same bytes as C's printf with the reference's row
    format (Python's %-formatting follows the same rules and rounding)."""
    g = W.plain_pa_seed(3000, 5, seed=8)
    rng = np.random.default_rng(3)
    with GrowthEngine(seed=4, record_trace=True) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(fixed_new_nodes=700), planned_epochs=2)
        eng.grow_epoch()
        eng.grow_epoch()
        n, _ = eng.counts()
        n0 = g.n
        ids = 10**12 + 7 * np.arange(n, dtype=np.int64) - 5
        ids[0] = -3
        draws = np.where(np.arange(n)[:, None] < n0, -1.0, rng.random((n, 4)) ** rng.integers(1, 30, (n, 4)))
        draws[n0 + 1] = [0.0, 1.0, 0.5, 1e-300]
        ints = rng.integers(-1, 3000, (n, 4)).astype(np.int32)
        gens = np.where(rng.random((n, 4)) < 0.5, -1, rng.integers(0, 10**13, (n, 4)))
        gens[n0 + 2] = -1
        txt = eng.format_attributes(ids, draws, ints, gens, n0, peak_integer).decode()
        pub, fit = eng.nodes()
        ind, outd = eng.degrees()
    lines = []
    for v in range(n):
        peak = "%d" % int(fit[v]) if peak_integer else "%.9g" % float(fit[v])
        gen = ("no_generators" if v < n0 else
               (";".join(str(x) for x in gens[v] if x >= 0) or "-1"))
        lines.append("%d,%s,%d,%.10g,%.10g,%.10g,%d,%s,%d,%.10g,%d,%d,%d,%d,%s\n" % (
            ids[v], "seed" if v < n0 else "agent", pub[v], draws[v, 0], draws[v, 1], draws[v, 2],
            ints[v, 0], peak, ints[v, 1], draws[v, 3], ind[v], outd[v], ints[v, 2], ints[v, 3], gen))
    assert txt == "".join(lines)


@pytest.mark.parametrize("p", [1e-5, 1e-3])
def test_run_er_epochs_matches_single_epochs(gpu, p):
    """Ten ER epochs enqueued without host synchronisation grow the same graph as ten single-epoch
    calls, and the last epoch's edges are reported the same way."""
    s = W.er_seed(100_000)
    res = []
    for multi in (False, True):
        with GrowthEngine(seed=42) as eng:
            eng.load_graph(s.pub, s.fitness, s.src, s.dst)
            if multi:
                ne = eng.run_er_epochs(10, 10_000, p)
            else:
                ne = sum(eng.er_epoch(10_000, p) for _ in range(10))
            res.append((ne, eng.counts(), [eng.csr(w) for w in (0, 1)], eng.last_epoch_edges(),
                        eng.degrees()[0]))
    (n1, c1, csr1, last1, ind1), (n2, c2, csr2, last2, ind2) = res
    assert n1 == n2 and c1 == c2
    for (o1, k1), (o2, k2) in zip(csr1, csr2):
        np.testing.assert_array_equal(o1, o2)
        np.testing.assert_array_equal(k1, k2)
    for x, y in zip(last1, last2):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(ind1, ind2)
