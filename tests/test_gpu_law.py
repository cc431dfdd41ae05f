"""Distribution-level parity of the GPU growth step with the reference's sampling law.

* Plain PA growth (10k seed DAG, 3 epochs x 5,000 agents, Poisson(15), 3 anchors, beta = 4): the
  default thinning sampler and the enumeration sampler -- the reference's Efraimidis-Spirakis top-k
  over the enumerated 2-hop ball (src/abm.cu:461-565) -- each grow the configuration on the GPU
  under independent seeds; a two-sample KS test compares the final in-degree distributions (and
  the in-degree gained during growth) at p > 0.01, for three seed pairs.
* Refcompat (ParAGraph's own model) on the GPU: the 1-hop and 2-hop choices of one epoch against
  the ES law and a numpy restatement of MakePopulateCitations' top-k of log(u)/score, as in
  tests/test_law_cpu.py but with the GPU's own output.
The p-values are printed in pytest's terminal summary."""
import numpy as np
import pytest

import law
from paragraph_gb300 import (PG_SAMPLER_ENUMERATE, PG_SAMPLER_THINNING, PG_WEIGHTS_REFCOMPAT,
                             GrowthEngine, PAParams, RCParams)
from paragraph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
P_KS = 0.01


def _grow_config1(seed: int, sampler: int):
    g = W.plain_pa_seed(10_000, 10, seed=42)
    with GrowthEngine(seed=seed, sampler=sampler) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, W.plain_pa_params(), planned_epochs=3)
        ind0, _ = eng.degrees()
        for _ in range(3):
            eng.grow_epoch()
        ind, _ = eng.degrees()
    return ind0, ind


@pytest.mark.parametrize("pair", [(101, 202), (303, 404), (505, 606)])
def test_in_degree_ks_thinning_vs_enumeration(gpu, pair):
    seed_t, seed_e = pair
    ind0, ind_t = _grow_config1(seed_t, PG_SAMPLER_THINNING)
    _, ind_e = _grow_config1(seed_e, PG_SAMPLER_ENUMERATE)
    assert len(ind_t) == len(ind_e) == 25_000
    n0 = len(ind0)
    pv = {
        "final in-degree": law.ks_2samp(ind_t, ind_e),
        "in-degree gained by seed nodes": law.ks_2samp(ind_t[:n0] - ind0, ind_e[:n0] - ind0),
        "in-degree of grown nodes": law.ks_2samp(ind_t[n0:], ind_e[n0:]),
    }
    for name, v in pv.items():
        law.record(f"KS plain PA config, thinning seed {seed_t} vs enumeration seed {seed_e}: {name}", v)
    assert ind_t.sum() > ind0.sum() and ind_e.sum() > ind0.sum()
    assert min(pv.values()) > P_KS, pv


def test_in_degree_ks_detects_a_different_beta(gpu):
    """Power check: the same KS test tells beta = 4 from beta = 1 (no neighbourhood boost)."""
    g = W.plain_pa_seed(10_000, 10, seed=42)
    out = []
    for beta in (4.0, 1.0):
        prm = W.plain_pa_params()
        prm.beta = beta
        with GrowthEngine(seed=7) as eng:
            eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=3)
            ind0, _ = eng.degrees()
            for _ in range(3):
                eng.grow_epoch()
            out.append(eng.degrees()[0][:len(ind0)] - ind0)
    assert law.ks_2samp(out[0], out[1]) < 1e-6


def test_refcompat_gpu_choices_follow_the_reference_rule(gpu):
    n0, seed = 3000, 9
    g = W.rc_seed(n0, 6, seed=seed)
    bag, rec = W.rc_tables(seed=seed, bag_mean=12.0)
    rc = RCParams(pa_weight=-1.0, rec_weight=-1.0, fit_weight=-1.0, alpha=-1.0,
                  fully_random=0.1, same_year=0.0, growth_rate=0.5)
    with GrowthEngine(seed=seed + 1000, weight_model=PG_WEIGHTS_REFCOMPAT, record_trace=True) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(growth_rate=rc.growth_rate),
                       planned_epochs=1)
        eng.rc_configure(rc, bag, rec)
        ind0, _ = eng.degrees()
        pub0, peak0 = eng.nodes()
        eng.grow_epoch()
        info, arr = eng.rc_agents(), eng.arrivals()
    scores = law.rc_scores(ind0, pub0, peak0, np.zeros(n0, np.int64), np.full(n0, 1000, np.int64),
                           rec, t=0)
    u = law.rc_choice_pits(n0, g, rc, info, arr, scores, np.random.Generator(np.random.PCG64(78)))
    pv = {}
    for part in ("in", "out"):
        assert len(u[(part, "engine")]) > 1000
        pv[f"{part}: PIT of the GPU's choices under the ES law (KS vs uniform)"] = law.ks_uniform(u[(part, "engine")])
        pv[f"{part}: GPU vs numpy top-k of log(u)/score (two-sample KS)"] = law.ks_2samp(u[(part, "engine")],
                                                                                       u[(part, "numpy")])
    for name, v in pv.items():
        law.record(f"law refcompat GPU {name}", v)
    assert min(pv.values()) > 1e-3, pv
