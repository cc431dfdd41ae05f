"""Sampling-law helpers for the distribution tests (not a test module).

The growth step's citations are a weighted sample without replacement.  These helpers state that
law directly in numpy, independently of the samplers under test:

* baseline model: successive sampling (Poisson sampling without replacement) with weights
  W_j = q_j * beta^[j in B2(A)], q_j the epoch's quantised weights and B2(A) the undirected 2-hop
  ball of the agent's anchors -- the law of the reference's Efraimidis-Spirakis top-k over the
  neighbourhood (src/abm.cu:461-565, gpu-std/device_min_heap.cuh:71-145);
* refcompat model: a plain numpy restatement of MakePopulateCitations (src/abm.cu:461-565): every
  candidate gets the key log(u)/score with u uniform on (0, 1], and the k largest keys are cited.

Every p-value a test computes is recorded with `record` and printed in pytest's terminal summary
(tests/conftest.py), so a quiet run still shows them.
"""
from __future__ import annotations

import numpy as np
from scipy import stats

PVALUES: list[tuple[str, float]] = []


def record(name: str, p: float) -> float:
    PVALUES.append((name, float(p)))
    return float(p)


# ---------------------------------------------------------------- graphs
def undirected_rows(n: int, src: np.ndarray, dst: np.ndarray) -> list[np.ndarray]:
    """Sorted unique neighbours of every node, edges taken in both directions."""
    s = np.concatenate([src, dst]).astype(np.int64)
    d = np.concatenate([dst, src]).astype(np.int64)
    key = np.unique(s * n + d)
    s, d = key // n, key % n
    cut = np.searchsorted(s, np.arange(n + 1))
    return [d[cut[v]:cut[v + 1]] for v in range(n)]


def ball_masks(n: int, src: np.ndarray, dst: np.ndarray, anchors: np.ndarray) -> np.ndarray:
    """[agents, n] bool: node j is within two undirected hops of one of the agent's anchors
    (anchors, their neighbours, and the neighbours of those).  anchors: [agents, m], -1 unused."""
    a = np.zeros((n, n), bool)
    a[src, dst] = True
    a[dst, src] = True
    one = a | np.eye(n, dtype=bool)
    two = (one.astype(np.int64) @ one.astype(np.int64)) > 0
    out = np.zeros((len(anchors), n), bool)
    for i in range(anchors.shape[1]):
        x = anchors[:, i]
        ok = x >= 0
        out[ok] |= two[x[ok]]
    return out


# ---------------------------------------------------------------- successive-sampling law
def first_choice_probs(q: np.ndarray, beta: float, ball: np.ndarray) -> np.ndarray:
    """[agents, n] probability that node j is an agent's first citation: W_j / sum W."""
    w = q[None, :] * np.where(ball, beta, 1.0)
    return w / w.sum(axis=1, keepdims=True)


def pair_expectation(p: np.ndarray) -> np.ndarray:
    """Expected counts of ordered (first, second) citation pairs over agents with p[a] their
    first-choice probabilities: P(j1, j2) = p(j1) p(j2) / (1 - p(j1)), j1 != j2."""
    e = (p / (1.0 - p)).T @ p
    np.fill_diagonal(e, 0.0)
    return e


def successive_sample(rng: np.random.Generator, p: np.ndarray, k: int) -> np.ndarray:
    """First k draws of successive sampling without replacement from one agent's p (numpy RNG)."""
    w = p.astype(np.float64).copy()
    out = np.empty(k, np.int64)
    for i in range(k):
        j = rng.choice(len(w), p=w / w.sum())
        out[i] = j
        w[j] = 0.0
    return out


# ---------------------------------------------------------------- tests of fit and of homogeneity
def chi2_gof(obs: np.ndarray, exp: np.ndarray, min_exp: float = 5.0) -> tuple[float, int, float]:
    """Pearson goodness of fit; cells with expectation below min_exp are pooled into one."""
    obs = np.asarray(obs, np.float64).ravel()
    exp = np.asarray(exp, np.float64).ravel()
    big = exp >= min_exp
    o = np.append(obs[big], obs[~big].sum())
    e = np.append(exp[big], exp[~big].sum())
    if e[-1] < min_exp and len(e) > 2:
        # a small pooled cell joins the last large one (with a single large cell it stays apart)
        o, e = o[:-1], e[:-1]
        o[-1] += obs[~big].sum()
        e[-1] += exp[~big].sum()
    stat = float(((o - e) ** 2 / e).sum())
    dof = len(o) - 1
    return stat, dof, float(stats.chi2.sf(stat, dof))


def chi2_homogeneity(a: np.ndarray, b: np.ndarray, min_total: float = 10.0) -> tuple[float, int, float]:
    """Two samples of counts over the same cells (equal or unequal totals): Pearson's test that
    they come from one distribution; cells with fewer than min_total counts in all are pooled."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    tot = a + b
    big = tot >= min_total
    ta = np.append(a[big], a[~big].sum())
    tb = np.append(b[big], b[~big].sum())
    keep = (ta + tb) > 0
    table = np.stack([ta[keep], tb[keep]])
    stat, p, dof, _ = stats.chi2_contingency(table, correction=False)
    return float(stat), int(dof), float(p)


def ks_2samp(x: np.ndarray, y: np.ndarray) -> float:
    return float(stats.ks_2samp(np.asarray(x), np.asarray(y)).pvalue)


def ks_uniform(u: np.ndarray) -> float:
    return float(stats.kstest(np.asarray(u), "uniform").pvalue)


def pit(rng: np.random.Generator, p: np.ndarray, j: int) -> float:
    """Randomised probability integral transform of outcome j under the discrete law p (over
    cells 0..len(p)-1): F(j-) + V p_j with V uniform, which is uniform on (0, 1) when j ~ p."""
    return float(p[:j].sum() + rng.random() * p[j])


# ---------------------------------------------------------------- refcompat model in numpy
def rc_scores(indeg: np.ndarray, pub: np.ndarray, peak: np.ndarray, lag: np.ndarray,
              dur: np.ndarray, rec: np.ndarray, t: int, gamma: int = 3, decay: int = 3):
    """Score components of ParAGraph's model at epoch t (FillInDegreeArr, FillFitnessArr,
    FillRecencyArr, src/abm.cu:112-208): pa_j = (indeg^gamma + 1) / sum, fit_j likewise with the
    fitness f_j(t) of the paper's window, rec_j = P(age_j) / (papers of that age * sum of P over
    the ages present)."""
    pub = pub.astype(np.int64)
    start = pub + lag
    f = np.where(start > t, 1.0,
                 np.where(start + dur >= t, peak.astype(np.float64),
                          np.floor(peak / np.maximum(t - start - dur + 1, 1).astype(np.float64) ** decay)))
    a = indeg.astype(np.float64) ** gamma + 1.0
    b = f ** gamma + 1.0
    age = t - pub
    ok = (age >= 0) & (age < len(rec))
    cnt = np.bincount(age[ok], minlength=len(rec)).astype(np.float64)
    U = rec[cnt > 0].sum()
    r = np.zeros(len(pub))
    r[ok] = rec[age[ok]] / (cnt[age[ok]] * U)
    return a / a.sum(), r, b / b.sum()


def rc_topk_keys(rng: np.random.Generator, cand: np.ndarray, score: np.ndarray, k: int) -> np.ndarray:
    """MakePopulateCitations' choice among distinct candidates: key log(u)/score (u uniform on
    (0, 1]; a zero score gets the smallest key), the k largest keys, largest first."""
    if k <= 0 or len(cand) == 0:
        return np.zeros(0, np.int64)
    u = 1.0 - rng.random(len(cand))
    s = score[cand]
    key = np.where(s != 0.0, np.log(u) / np.where(s != 0.0, s, 1.0), -np.inf)
    order = np.argsort(-key, kind="stable")
    return cand[order[:min(k, len(cand))]]


def rc_budget(d: int, alpha: float, fully_random: float, same_year: int) -> tuple[int, int]:
    """Per-paper budget split of the refcompat rule (src/kernel.cu:244-256,320-326): the share of
    the neighbourhood citations asked of the 1-hop set, and the reserve for uniform citations."""
    rsv = int(np.floor(fully_random * d))
    rem1 = d - 1 - same_year - rsv
    in_t = int(np.ceil(rem1 * alpha)) if rem1 > 0 else 0
    in_t = min(in_t, max(rem1, 0))
    return in_t, rsv


def rc_choice_pits(n0, g, rc, info, arr, scores, rng):
    """Per part (1-hop "in", 2-hop "out"): PIT values of the first two choices of every paper under
    the ES law (successive sampling with weights score_j over the part's candidates), for the
    engine's choices and for the numpy restatement's, drawn with the same per-paper draws."""
    rows = undirected_rows(n0, g.src, g.dst)
    pa, rec, fit = scores
    out = {(part, who): [] for part in ("in", "out") for who in ("engine", "numpy")}
    pos = 0
    for a in range(len(info)):
        w3, alpha, gen, d = info[a, :3], info[a, 3], int(info[a, 4]), int(info[a, 5])
        cites = arr[pos:pos + d]
        pos += d
        assert cites[0] == gen
        score = w3[0] * pa + w3[1] * rec + w3[2] * fit
        n1 = rows[gen][rows[gen] != gen]
        n2 = (np.setdiff1d(np.unique(np.concatenate([rows[y] for y in n1])), np.append(n1, gen))
              if len(n1) else n1)
        in_t, rsv = rc_budget(d, alpha, rc.fully_random, 0)
        n_in = min(in_t, len(n1))
        rem2 = d - 1 - rsv - n_in
        n_out = min(rem2, len(n2)) if rem2 > 0 else 0
        parts = (("in", n1, cites[1:1 + n_in]), ("out", n2, cites[1 + n_in:1 + n_in + n_out]))
        for part, cand, got in parts:
            if len(got) == 0 or len(got) == len(cand):
                continue  # no choice was made, or all candidates were taken
            p = score[cand] / score[cand].sum()
            mine = rc_topk_keys(rng, cand, score, len(got))
            for who, picks in (("engine", got), ("numpy", mine)):
                idx = np.searchsorted(cand, picks[:2])
                out[(part, who)].append(pit(rng, p, idx[0]))
                if len(idx) > 1:
                    r = p.copy()
                    r[idx[0]] = 0.0
                    out[(part, who)].append(pit(rng, r / r.sum(), idx[1]))
    return {key: np.array(v) for key, v in out.items()}
