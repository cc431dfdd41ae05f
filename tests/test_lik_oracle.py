"""The FP64 trace log-likelihood of the oracle: against a plain-Python restatement of the density
on a tiny trace, and its gradient against central finite differences (h = 1e-4).

The density is that of successive sampling without replacement with weights
W_j = f_j^gamma (indeg_e(j)+1)^alpha exp(-(t_e - t_j)/tau) beta^[j in N_a] over the nodes that existed
when the agent's epoch began (the law the growth samplers draw from)."""
import math

import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import PAParams
from paragraph_gb300 import workloads as W

THETA_STAR = np.array([1.0, 5.0, 1.0, 4.0])


def _trace(n0, epochs, seed=5, lam=20.0, growth=0.03, fixed=0):
    g = W.plain_pa_seed(n0, 10, seed=3)
    prm = PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=lam,
                   growth_rate=growth, fixed_new_nodes=fixed, num_anchors=3)
    return O.grow_trace(g, prm, epochs, seed=seed)


def _brute_loglik(tr, theta):
    """Plain-Python density: sets for the balls, sums in the order written."""
    al, tau, ga, be = theta
    n = tr.num_nodes
    n0 = int(tr.epoch_nodes[0])
    out = [set() for _ in range(n)]
    inn = [set() for _ in range(n)]
    for s, d in zip(tr.seed_src.tolist(), tr.seed_dst.tolist()):
        out[s].add(d)
        inn[d].add(s)
    for a in range(tr.agents):
        for c in tr.cites[tr.cite_off[a]:tr.cite_off[a + 1]].tolist():
            out[n0 + a].add(c)
            inn[c].add(n0 + a)
    total = 0.0
    for a in range(tr.agents):
        v = n0 + a
        e = int(np.searchsorted(tr.epoch_nodes, v, side="right")) - 1
        ne, te = int(tr.epoch_nodes[e]), int(tr.epoch_t[e])

        def nb(x):
            return {y for y in out[x] if y < ne} | {y for y in inn[x] if y < ne}

        anchors = [int(x) for x in tr.anchors[a] if x >= 0]
        ball = set(anchors)
        hop1 = set()
        for x in anchors:
            hop1 |= nb(x)
        ball |= hop1
        for y in hop1:
            ball |= nb(y)

        def w(j):
            d = sum(1 for s in inn[j] if s < ne)
            x = ga * math.log(float(tr.fitness[j])) + al * math.log(d + 1.0) - (te - int(tr.pub[j])) / tau
            return math.exp(x) * (be if j in ball else 1.0)

        ws = [w(j) for j in range(ne)]
        z = sum(ws)
        p = 0.0
        for c in tr.cites[tr.cite_off[a]:tr.cite_off[a + 1]].tolist():
            total += math.log(ws[c]) - math.log(z - p)
            p += ws[c]
    return total


def test_oracle_loglik_matches_plain_python():
    tr = _trace(120, 3, lam=4.0, growth=0.0, fixed=12)
    assert tr.agents == 36
    thetas = np.array([THETA_STAR, [0.6, 2.5, 1.7, 7.0], [1.4, 9.0, 0.6, 1.0]])
    ll = O.loglik(tr, thetas, grad=False, threads=1)
    for b in range(len(thetas)):
        ref = _brute_loglik(tr, thetas[b])
        assert abs(ll[b] - ref) <= 1e-11 * abs(ref), (b, ll[b], ref)


def _fd_grad(tr, theta, h=1e-4):
    pts = []
    for k in range(4):
        for sgn in (1.0, -1.0):
            t = theta.copy()
            t[k] += sgn * h
            pts.append(t)
    ll = O.loglik(tr, np.array(pts), grad=False)
    return (ll[0::2] - ll[1::2]) / (2 * h)


def test_oracle_gradient_matches_central_differences():
    """FP64 adjoint-free gradient vs central differences, h = 1e-4: relative error (2-norm over
    the four components) <= 1e-6 at points from the calibration ranges.  At theta* the gradient is
    close to zero (the trace was drawn there), so the finite-difference truncation error
    (h^2/6 d3 logL) is a larger share of it; there the bound is 1e-5."""
    tr = _trace(3000, 10)
    pts = W.theta_batch(8, seed=11)
    _, g = O.loglik(tr, pts)
    for b in range(len(pts)):
        fd = _fd_grad(tr, pts[b])
        rel = np.linalg.norm(fd - g[b]) / np.linalg.norm(g[b])
        assert rel <= 1e-6, (b, pts[b], g[b], fd, rel)
    _, gs = O.loglik(tr, THETA_STAR[None])
    fd = _fd_grad(tr, THETA_STAR)
    assert np.linalg.norm(fd - gs[0]) / np.linalg.norm(gs[0]) <= 1e-5


def test_loglik_peaks_near_the_generating_parameters():
    tr = _trace(3000, 10)
    pts = W.theta_batch(16, seed=3)
    ll = O.loglik(tr, np.vstack([THETA_STAR, pts]), grad=False)
    assert ll[0] > ll[1:].max()
