"""The samplers' law against the law itself, on the CPU (oracle restatement; no GPU).

Bit-exact GPU <-> oracle parity says the kernels compute what the oracle computes; these tests say
that what the oracle computes is the reference's law.  On graphs small enough to write the law
down (64 or 96 nodes, sparse, so an agent's 2-hop ball is a fifth to a third of the nodes and beta
matters), one epoch of 20,000 agents is drawn by each baseline sampler, and the first and second
citations of every agent are compared with the successive-sampling law W_j = q_j beta^[j in B2]:
Pearson chi-square against the exact expected counts, a homogeneity test against draws of a plain
numpy successive sampler, and a KS test of the randomised probability integral transform (PIT) of
each choice under its own agent's law.  The refcompat model's 1-hop and 2-hop choices are compared
with MakePopulateCitations' top-k of log(u)/score (src/abm.cu:461-565) the same way: the PIT of the
first two choices of each part under the ES law, and a numpy restatement drawn with the oracle's
per-paper draws held fixed.  A test passes when every p-value is above 0.001; the p-values are
printed in the terminal summary."""
import numpy as np
import pytest

import law
import oracle as O
from paragraph_gb300 import PAParams, RCParams
from paragraph_gb300 import workloads as W

P_MIN = 1e-3
THINNING, ENUMERATE = 0, 1
# (nodes, citations per seed node, anchors): balls of about 30 % and 20 % of the nodes
GRAPHS = {"64n-1a": (64, 2, 1), "96n-3a": (96, 1, 3)}


def _seed(shape: str, skew: bool) -> W.SeedGraph:
    n, c, _ = GRAPHS[shape]
    g = W.plain_pa_seed(n, c, seed=11)
    if skew:
        # one node holds about 99 % of the weight: the thinning sampler's event cap is reached and
        # its exact continuation without replacement takes over
        g.fitness[7] = 5.0e3
    return g


def _grow_one_epoch(g, prm: PAParams, seed: int, sampler: int):
    og = O.OracleGraph(seed, 0)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.set_params(**prm.__dict__)
    og.set_sampler(sampler)
    n0 = og.n
    og.pa_epoch()
    _, cdf, _ = og.weights()
    q = np.diff(cdf.astype(np.float64), prepend=0.0)
    off, _ = og.csr(0)
    k = np.diff(off[n0:og.n + 1])
    arr = og.arrivals()
    starts = np.concatenate([[0], np.cumsum(k)[:-1]])
    anchors = O.agent_anchors(seed, 0, 0, n0, og.n - n0, prm.num_anchors)
    st = og.stats()
    og.close()
    return q, k, arr, starts, anchors, st


def _pit_first_two(rng, p: np.ndarray, first: np.ndarray, second: np.ndarray, two: np.ndarray):
    """PIT of every agent's first choice under p[a], and of its second under p[a] without the first."""
    u1 = np.array([law.pit(rng, p[a], first[a]) for a in range(len(p))])
    u2 = []
    for a in np.nonzero(two)[0]:
        r = p[a].copy()
        r[first[a]] = 0.0
        u2.append(law.pit(rng, r / r.sum(), second[a]))
    return u1, np.array(u2)


@pytest.mark.parametrize("sampler", [THINNING, ENUMERATE])
@pytest.mark.parametrize("shape,skew", [("64n-1a", False), ("96n-3a", False), ("64n-1a", True)])
def test_first_and_second_choice_follow_successive_sampling(built, sampler, shape, skew):
    n0, _, na = GRAPHS[shape]
    agents, beta = 20_000, 4.0
    g = _seed(shape, skew)
    prm = PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=beta, mean_out_degree=20.0 if skew else 3.0,
                   growth_rate=0.0, fixed_new_nodes=agents, num_anchors=na)
    q, k, arr, starts, anchors, st = _grow_one_epoch(g, prm, 1000 + sampler, sampler)
    ball = law.ball_masks(n0, g.src, g.dst, anchors)
    p = law.first_choice_probs(q, beta, ball)
    tag = f"{'thinning' if sampler == THINNING else 'enumeration'} {shape}{' skewed' if skew else ''}"
    pv = {}

    first = arr[starts]
    two = k >= 2
    second = np.where(two, arr[np.minimum(starts + 1, len(arr) - 1)], -1)
    pv["first citation vs exact law (chi2)"] = law.chi2_gof(np.bincount(first, minlength=n0),
                                                            p.sum(axis=0))[2]
    pairs = np.zeros((n0, n0))
    np.add.at(pairs, (first[two], second[two]), 1.0)
    pv["ordered first two citations vs exact law (chi2)"] = law.chi2_gof(
        pairs, law.pair_expectation(p[two]))[2]

    rng = np.random.Generator(np.random.PCG64(5 + sampler + 2 * skew + 4 * na))
    u1, u2 = _pit_first_two(rng, p, first, second, two)
    pv["PIT of the first citation (KS vs uniform)"] = law.ks_uniform(u1)
    pv["PIT of the second citation given the first (KS vs uniform)"] = law.ks_uniform(u2)

    # the same two draws from a plain numpy successive sampler over the same agents
    idx = np.nonzero(two)[0]
    ref = np.array([law.successive_sample(rng, p[a], 2) for a in idx])
    pv["first citation vs numpy successive sampler (chi2)"] = law.chi2_homogeneity(
        np.bincount(first[two], minlength=n0), np.bincount(ref[:, 0], minlength=n0))[2]
    ref_pairs = np.zeros((n0, n0))
    np.add.at(ref_pairs, (ref[:, 0], ref[:, 1]), 1.0)
    pv["ordered pairs vs numpy successive sampler (chi2)"] = law.chi2_homogeneity(pairs, ref_pairs)[2]

    for name, v in pv.items():
        law.record(f"law {tag}: {name}", v)
    if skew and sampler == THINNING:
        assert st["draws"] > (64 * k + 256).sum(), "the continuation path was not exercised"
    assert 0.15 < ball.mean() < 0.4
    assert min(pv.values()) > P_MIN, pv


def test_law_tests_detect_a_wrong_beta(built):
    """Power check: the same tests reject the law when it is stated with beta = 2 (the oracle
    samples with beta = 4)."""
    n0, _, na = GRAPHS["64n-1a"]
    g = _seed("64n-1a", False)
    prm = PAParams(beta=4.0, mean_out_degree=3.0, growth_rate=0.0, fixed_new_nodes=20_000,
                   num_anchors=na)
    q, k, arr, starts, anchors, _ = _grow_one_epoch(g, prm, 1000, THINNING)
    ball = law.ball_masks(n0, g.src, g.dst, anchors)
    wrong = law.first_choice_probs(q, 2.0, ball)
    first = arr[starts]
    assert law.chi2_gof(np.bincount(first, minlength=n0), wrong.sum(axis=0))[2] < 1e-6
    u = [law.pit(np.random.Generator(np.random.PCG64(1)), wrong[a], first[a]) for a in range(len(first))]
    assert law.ks_uniform(np.array(u)) < 1e-6


# ---------------------------------------------------------------- refcompat (the reference's own model)
def _rc_epoch(n0: int, seed: int):
    g = W.rc_seed(n0, 6, seed=seed)
    bag, rec = W.rc_tables(seed=seed, bag_mean=12.0)
    rc = RCParams(pa_weight=-1.0, rec_weight=-1.0, fit_weight=-1.0, alpha=-1.0,
                  fully_random=0.1, same_year=0.0, growth_rate=0.5)
    og = O.OracleGraph(seed, 0)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.rc_configure(rc, bag, rec)
    indeg0, _ = og.degrees()
    pub0, peak0 = og.nodes()
    og.rc_epoch()
    info, arr = og.rc_agents(), og.arrivals()
    og.close()
    scores = law.rc_scores(indeg0, pub0, peak0, np.zeros(n0, np.int64), np.full(n0, 1000, np.int64),
                           rec, t=0)
    return g, rc, info, arr, scores


def test_refcompat_neighbourhood_choices_follow_the_reference_rule(built):
    n0 = 3000
    g, rc, info, arr, scores = _rc_epoch(n0, 9)
    u = law.rc_choice_pits(n0, g, rc, info, arr, scores, np.random.Generator(np.random.PCG64(77)))
    pv = {}
    for part in ("in", "out"):
        assert len(u[(part, "engine")]) > 1000
        pv[f"{part}: PIT of the engine's choices under the ES law (KS vs uniform)"] = law.ks_uniform(u[(part, "engine")])
        pv[f"{part}: PIT of numpy top-k of log(u)/score (KS vs uniform)"] = law.ks_uniform(u[(part, "numpy")])
        pv[f"{part}: engine vs numpy restatement (two-sample KS)"] = law.ks_2samp(u[(part, "engine")],
                                                                                u[(part, "numpy")])
    for name, v in pv.items():
        law.record(f"law refcompat {name}", v)
    assert min(pv.values()) > P_MIN, pv
