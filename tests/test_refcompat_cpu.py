"""Refcompat functor on the CPU: the library's host tables against the oracle's independent ones,
and the oracle restatement's per-paper budget rule on small graphs (no GPU)."""
import numpy as np

import oracle as O
from paragraph_gb300 import RCParams, rc_bag_table, rc_fitness_table
from paragraph_gb300 import workloads as W


def test_bag_and_fitness_tables_match_oracle(built):
    bag, _ = W.rc_tables(seed=11)
    np.testing.assert_array_equal(rc_bag_table(bag), O.rc_bag_table(bag))
    np.testing.assert_array_equal(rc_fitness_table(), O.rc_fitness_table())
    t = rc_bag_table([3, 3, 5, 300])
    assert t[2] == 0 and t[3] == 1 << 63 and t[5] == 3 << 62 and t[256] == (1 << 64) - 1
    f = rc_fitness_table()
    assert np.all(np.diff(f.astype(np.float64)) >= 0) and f[-1] == (1 << 64) - 1


def test_oracle_budget_rule(built):
    g = W.rc_seed(800, 6, seed=4)
    bag, rec = W.rc_tables(seed=6, bag_mean=12.0)
    rc = RCParams(growth_rate=0.1, same_year=0.25, fully_random=0.1)
    og = O.OracleGraph(5, 0)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.rc_configure(rc, bag, rec)
    n0 = og.n
    og.rc_epoch()
    delta = og.n - n0
    assert delta == int(np.ceil(n0 * 0.1))
    info = og.rc_agents()
    arr = og.arrivals()
    off, col = og.csr(0)
    pos = 0
    same_year = 0
    for a in range(delta):
        d = int(info[a, 5])
        cites = arr[pos:pos + d]
        pos += d
        assert cites[0] == int(info[a, 4])                     # the generator comes first
        assert len(set(cites.tolist())) == d                   # distinct
        row = col[off[n0 + a]:off[n0 + a + 1]]
        np.testing.assert_array_equal(np.sort(cites), row)     # the forward row is the sorted set
        new = cites[cites >= n0]
        assert len(new) <= 1 and np.all(new < n0 + delta)      # at most one same-year citation
        same_year += len(new)
        assert np.isclose(info[a, :3].sum(), 1.0)
    # exactly floor(delta * same_year) citers, less those whose out-degree of 1 leaves room only
    # for the generator
    S = int(np.floor(delta * 0.25))
    assert S - int(np.sum(info[:, 5] < 2)) <= same_year <= S
    assert pos == len(arr)
