"""Failure paths on the GPU, made without faulting or hanging it.

The reference turns any CUDA error into exit status 1 (src/kernel.cu:1761-1764) and only prints
device-side overflows.  Here kernels never trap: they set bits of a device error word that later
kernels check before they write, the host turns the word into a status, and a context whose epoch
failed refuses further growth until it is restored or reloaded.

* Timeout: the first bounded wait on every staged copy of the thinning agent kernel is cut to zero
  polls (pg_set_wait_limit), so each gives up at once; the warp then drains its copies in flight
  with the full bound and stops.  The epoch must return PG_ERR_TIMEOUT, the context must refuse the
  next epoch, and pg_restore must bring back a context that grows exactly as the oracle does.
* Capacity: one replica of a batched context is given a mean out-degree far beyond what its edge
  region was planned for; the device check before the agent kernels must stop the epoch with
  PG_ERR_CAPACITY before anything is written, and the same restore path must recover."""
import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import (PG_ERR_CAPACITY, PG_ERR_STATE, PG_ERR_TIMEOUT, GrowthEngine, PAParams,
                             PGError, ReplicaInput)
from paragraph_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _same_csr(eng, og, replica=0):
    assert eng.counts(replica) == (og.n, og.m)
    for which in (0, 1):
        for x, y in zip(eng.csr(which, replica), og.csr(which)):
            np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(eng.degrees(replica)[0], og.degrees()[0])


def test_timed_out_wait_is_reported_and_restore_recovers(gpu):
    # a popular-node seed: agents test long candidate rows, so every agent stages copies
    g = W.pareto_seed(60_000, 2.5, 16.0, seed=3)
    prm = PAParams(mean_out_degree=20.0, growth_rate=0.0, fixed_new_nodes=2000)
    with GrowthEngine(seed=21) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=2)
        eng.checkpoint()
        before = eng.counts()
        eng.set_wait_limit(0)
        with pytest.raises(PGError) as err:
            eng.grow_epoch()
        assert err.value.status == PG_ERR_TIMEOUT
        assert "bounded wait" in str(err.value)
        with pytest.raises(PGError) as again:  # the failed epoch left the context inconsistent
            eng.grow_epoch()
        assert again.value.status == PG_ERR_STATE
        with pytest.raises(PGError):
            eng.run_epochs(1, use_graph=True)
        eng.set_wait_limit(-1)
        eng.restore()
        assert eng.counts() == before
        og = O.OracleGraph(21, 0)
        og.load(g.pub, g.fitness, g.src, g.dst)
        og.set_params(**prm.__dict__)
        for _ in range(2):
            eng.grow_epoch()
            og.pa_epoch()
            np.testing.assert_array_equal(eng.last_epoch_edges()[1], og.last_epoch_edges()[1])
        _same_csr(eng, og)


def test_device_capacity_overflow_is_reported_and_writes_nothing(gpu):
    reps = []
    for r, n in enumerate((3000, 5000)):
        g = W.plain_pa_seed(n, 10, seed=40 + r)
        reps.append(ReplicaInput(g.pub, g.fitness, g.src, g.dst,
                                 PAParams(mean_out_degree=5.0, growth_rate=0.0, fixed_new_nodes=400),
                                 planned_epochs=1))
    with GrowthEngine(seed=8, replicas=2) as eng:
        eng.load_replicas(reps)
        eng.checkpoint()
        seed_csr = [[eng.csr(w, r) for w in (0, 1)] for r in range(2)]
        # replica 1 now asks for ~40x the citations its edge region was planned for
        eng.set_params(PAParams(mean_out_degree=200.0, growth_rate=0.0, fixed_new_nodes=400), replica=1)
        with pytest.raises(PGError) as err:
            eng.grow_epoch()
        assert err.value.status == PG_ERR_CAPACITY
        for r in range(2):  # the check stopped the epoch before any write
            for w in (0, 1):
                for x, y in zip(eng.csr(w, r), seed_csr[r][w]):
                    np.testing.assert_array_equal(x, y)
        with pytest.raises(PGError) as again:
            eng.grow_epoch()
        assert again.value.status == PG_ERR_STATE
        eng.restore()
        eng.set_params(reps[1].params, replica=1)
        eng.grow_epoch()
        for r, ri in enumerate(reps):
            og = O.OracleGraph(8, r)
            og.load(ri.pub_epoch, ri.fitness, ri.src, ri.dst)
            og.set_params(**ri.params.__dict__)
            og.pa_epoch()
            _same_csr(eng, og, replica=r)
