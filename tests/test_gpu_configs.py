"""Bit-exact parity at the benchmark configurations' stated sizes (GPU engine vs CPU oracle).

* ER G(n,p): 100,000-node seed, 10 epochs of 10,000 new nodes, p in {1e-5, 1e-4, 1e-3}.
* PA at scale: 1,000,000-node seed with Pareto(2.5) in-degrees, Poisson(30), 3 % growth; the first
  three epochs (the oracle's thinning sampler takes about a second per epoch on 16 cores).  This is
  the skewed graph whose hubs exercise the hub masks and the hub-pair rows.
* Batched ensemble: all 256 replicas (seeds log-uniform in [5,000, 200,000], per-replica alpha,
  tau, gamma, beta) grown 10 epochs in one context, one persistent kernel per epoch, from one
  captured graph; the replicas with the
  largest and smallest seeds and with the extreme values of each parameter are compared with
  oracles grown alone.
* Calibration trace: 200,000-node seed, 10 epochs at theta* = (1, 5, 1, 4); the GPU trace equals
  the oracle's, and the log-likelihood and its gradient at theta* and 8 points of the parameter
  ranges agree with the FP64 oracle (tolerances as in tests/test_gpu_lik.py).
Every integer result is compared bit for bit: both CSRs, in-degrees, new-node attributes and the
citations of every epoch in arrival order."""
import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import GrowthEngine
from paragraph_gb300 import workloads as W

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _compare_state(eng: GrowthEngine, og: O.OracleGraph, replica: int = 0):
    assert eng.counts(replica) == (og.n, og.m)
    for which in (0, 1):
        off_g, col_g = eng.csr(which, replica)
        off_o, col_o = og.csr(which)
        np.testing.assert_array_equal(off_g, off_o, err_msg=f"offsets which={which}")
        np.testing.assert_array_equal(col_g, col_o, err_msg=f"columns which={which}")
    for x, y in zip(eng.degrees(replica), og.degrees()):
        np.testing.assert_array_equal(x, y)
    pg_, fg = eng.nodes(replica)
    po, fo = og.nodes()
    np.testing.assert_array_equal(pg_, po)
    np.testing.assert_array_equal(fg.view(np.uint32), fo.view(np.uint32))


@pytest.mark.parametrize("p", [1e-5, 1e-4, 1e-3])
def test_er_config_full_size(gpu, p):
    s = W.er_seed(100_000)
    with GrowthEngine(seed=42) as eng:
        eng.load_graph(s.pub, s.fitness, s.src, s.dst)
        og = O.OracleGraph(42, 0)
        og.load(s.pub, s.fitness, s.src, s.dst)
        total = 0
        for _ in range(10):
            ne = eng.er_epoch(10_000, p)
            og.er_epoch(10_000, p)
            assert ne == og.epoch_edges()[1]
            s_g, d_g = eng.last_epoch_edges()
            s_o, d_o = og.last_epoch_edges()
            np.testing.assert_array_equal(s_g, s_o)
            np.testing.assert_array_equal(d_g, d_o)
            total += ne
        _compare_state(eng, og)
    # expected edges: 10,000 x sum over epochs of (100,000 + 10,000 t) x p
    mu = 1e4 * sum(1e5 + 1e4 * t for t in range(10)) * p
    assert abs(total - mu) < 6 * np.sqrt(mu)


def test_pa_scale_config_first_epochs(gpu):
    g = W.pareto_seed(1_000_000, 2.5, 16.0, seed=42)
    prm = W.scale_pa_params()
    with GrowthEngine(seed=42, record_trace=True) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=3)
        og = O.OracleGraph(42, 0)
        og.load(g.pub, g.fitness, g.src, g.dst)
        og.set_params(**prm.__dict__)
        og.set_sampler(0)
        ind, outd = eng.degrees()
        assert (ind.astype(np.int64) + outd >= 1024).sum() > 0  # hubs: the hub masks are in play
        for _ in range(3):
            nn, ne = eng.grow_epoch()
            og.pa_epoch()
            assert ne == og.epoch_edges()[1]
            np.testing.assert_array_equal(eng.arrivals(), og.arrivals())
            st, so = eng.stats(), og.stats()
            for k in ("nodes_weighted", "rows_expanded", "draws", "adj_scanned"):
                assert st[k] == so[k], k
        _compare_state(eng, og)


def test_ensemble_config_full_size(gpu):
    reps = W.ensemble_inputs(256, 5_000, 200_000, 10, seed=42)
    sizes = np.array([len(r.pub_epoch) for r in reps])
    prm = np.array([[r.params.alpha, r.params.tau, r.params.gamma, r.params.beta] for r in reps])
    pick = {int(sizes.argmax()), int(sizes.argmin())}
    for c in range(4):
        pick |= {int(prm[:, c].argmax()), int(prm[:, c].argmin())}
    with GrowthEngine(seed=42, replicas=len(reps)) as eng:
        eng.load_replicas(reps)
        eng.set_tuning(epoch_kernel=1)  # one persistent kernel per epoch over all 256 replicas
        eng.run_epochs(10, use_graph=True)
        for r in sorted(pick):
            ri = reps[r]
            og = O.OracleGraph(42, r)
            og.load(ri.pub_epoch, ri.fitness, ri.src, ri.dst)
            og.set_params(**ri.params.__dict__)
            for _ in range(10):
                og.pa_epoch()
            _compare_state(eng, og, replica=r)
            og.close()
    assert len(pick) >= 8 and sizes.max() > 150_000


def test_calibration_config_full_size(gpu):
    g = W.plain_pa_seed(200_000, 10, seed=42)
    prm = W.calibration_params()
    tg = W.grow_trace(g, prm, 10, seed=42)
    to = O.grow_trace(g, prm, 10, seed=42)
    for f in ("epoch_nodes", "epoch_t", "anchors", "cite_off", "cites", "pub"):
        np.testing.assert_array_equal(getattr(tg, f), getattr(to, f), err_msg=f)
    np.testing.assert_array_equal(tg.fitness.view(np.uint32), to.fitness.view(np.uint32))
    pts = np.vstack([[1.0, 5.0, 1.0, 4.0], W.theta_batch(8, seed=3)])
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(tg)
        ll = eng.loglik(pts)
        gr = eng.loglik_grad(pts)
        eng.set_lik_exact_exp2(True)
        lx = eng.loglik(pts)
        gx = eng.loglik_grad(pts)
    llo, gro = O.loglik(to, pts)
    rel_ll = np.abs(ll - llo) / np.abs(llo)
    rel_g = np.linalg.norm(gr - gro, axis=1) / np.linalg.norm(gro, axis=1)
    rel_lx = np.abs(lx - llo) / np.abs(llo)
    rel_gx = np.linalg.norm(gx - gro, axis=1) / np.linalg.norm(gro, axis=1)
    msg = (f"loglik {rel_ll.max():.3g}, grad (8 points) {rel_g[1:].max():.3g}, grad (theta*) {rel_g[0]:.3g}; "
           f"exact: loglik {rel_lx.max():.3g}, grad (8 points) {rel_gx[1:].max():.3g}, grad (theta*) {rel_gx[0]:.3g}")
    print(msg)
    assert rel_ll.max() <= 1e-7 and rel_lx.max() <= 1e-7, msg
    assert rel_g[1:].max() <= 1e-6, msg
    assert rel_g[0] <= 1e-5, msg
    # the exact arithmetic meets the gradient bound at the generating point too
    assert rel_gx.max() <= 1e-6, msg
