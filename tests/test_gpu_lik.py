"""GPU log-likelihood forward pass and adjoint against the FP64 oracle.

The GPU computes each weight in fp32 (one exp2 of an exponent carried as an fp32 pair) and every
normaliser and log-sum in FP64 or compensated fp32; the oracle is FP64 throughout.  Tolerances:
log-likelihood relative error <= 1e-7 (fp32 weights carry about 1e-7 relative error into each of
the ~1e5 terms); gradient relative error (2-norm over the four components) <= 1e-6 at the 64
points drawn from the parameter ranges.  At the generating point theta* the gradient is close to
zero -- the trace was drawn there -- so errors that do not average out over the trace are a larger
share of it: the default arithmetic (special-function-unit exp2, pairwise ball sums) is held to
1e-5 there, the exact arithmetic (pg_lik_set_exact_exp2) to 1e-6 like every other point."""
import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import GrowthEngine, PGError
from paragraph_gb300 import workloads as W

pytestmark = pytest.mark.gpu
THETA_STAR = np.array([1.0, 5.0, 1.0, 4.0])


@pytest.fixture(scope="module")
def trace_mid(gpu):
    g = W.plain_pa_seed(20_000, 10, seed=3)
    return W.grow_trace(g, W.calibration_params(), 10, seed=5)


def test_gpu_trace_equals_oracle_trace(gpu):
    """Anchors and draw-order citations recorded by the GPU growth step match the oracle's."""
    g = W.plain_pa_seed(4000, 10, seed=4)
    prm = W.calibration_params()
    tg = W.grow_trace(g, prm, 4, seed=9)
    to = O.grow_trace(g, prm, 4, seed=9)
    for f in ("epoch_nodes", "epoch_t", "anchors", "cite_off", "cites", "pub"):
        np.testing.assert_array_equal(getattr(tg, f), getattr(to, f), err_msg=f)
    np.testing.assert_array_equal(tg.fitness.view(np.uint32), to.fitness.view(np.uint32))


def test_loglik_and_gradient_match_fp64_oracle(trace_mid):
    pts = np.vstack([THETA_STAR, W.theta_batch(64, seed=1)])
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(trace_mid)
        ll = eng.loglik(pts)
        gr = eng.loglik_grad(pts)
    llo, gro = O.loglik(trace_mid, pts)
    rel_ll = np.abs(ll - llo) / np.abs(llo)
    rel_g = np.linalg.norm(gr - gro, axis=1) / np.linalg.norm(gro, axis=1)
    msg = f"loglik {rel_ll.max():.3g}, grad (64 points) {rel_g[1:].max():.3g}, grad (theta*) {rel_g[0]:.3g}"
    print(msg)
    assert rel_ll.max() <= 1e-7, msg
    assert rel_g[1:].max() <= 1e-6, msg
    assert rel_g[0] <= 1e-5, msg


def test_exact_arithmetic_meets_1e6_at_the_generating_point(trace_mid):
    """The exact arithmetic (fp32 exp2 to ~2 ulp, every ball weight and product summed on its own)
    holds the gradient within 1e-6 of the FP64 oracle at theta* as well, in batches of one point
    (the sliced ball walk) and of nine (one lane per point)."""
    pts = np.vstack([THETA_STAR, W.theta_batch(8, seed=11)])
    llo, gro = O.loglik(trace_mid, pts)
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(trace_mid)
        eng.set_lik_exact_exp2(True)
        ll = eng.loglik(pts)
        gr = eng.loglik_grad(pts)
        l1 = eng.loglik(pts[:1])
        g1 = eng.loglik_grad(pts[:1])
    rel_ll = np.abs(ll - llo) / np.abs(llo)
    rel_g = np.linalg.norm(gr - gro, axis=1) / np.linalg.norm(gro, axis=1)
    rel_1 = np.linalg.norm(g1[0] - gro[0]) / np.linalg.norm(gro[0])
    msg = f"loglik {rel_ll.max():.3g}, grad (theta*) {rel_g[0]:.3g} / alone {rel_1:.3g}, others {rel_g[1:].max():.3g}"
    assert rel_ll.max() <= 1e-7 and abs(l1[0] - llo[0]) <= 1e-7 * abs(llo[0]), msg
    assert rel_g.max() <= 1e-6 and rel_1 <= 1e-6, msg


def test_arithmetic_modes_switch_cleanly(trace_mid):
    """The feature rows follow the arithmetic of each forward pass and the adjoint keeps the
    forward's: default results after exact passes, with the mode switched again before the adjoint,
    equal a fresh context's default results bit for bit."""
    pts = W.theta_batch(3, seed=13)
    with GrowthEngine(seed=1) as a, GrowthEngine(seed=1) as b:
        a.load_trace(trace_mid)
        b.load_trace(trace_mid)
        l0 = a.loglik(pts)
        g0 = a.loglik_grad(pts)
        b.set_lik_exact_exp2(True)
        lx = b.loglik(pts)
        b.loglik_grad(pts)
        b.set_lik_exact_exp2(False)
        l1 = b.loglik(pts)
        b.set_lik_exact_exp2(True)
        g1 = b.loglik_grad(pts)
    np.testing.assert_array_equal(l0, l1)
    np.testing.assert_array_equal(g0, g1)
    assert not np.array_equal(l0, lx)


def test_batch_groups_and_single_points_agree(trace_mid):
    """70 points run as two launches of <= 64; every point alone gives the same values.  A single
    point splits the ball sums over more threads than a batch, so the compensated fp32 partial
    sums differ in order: agreement is to 1e-9 (log-likelihood) and 1e-7 (gradient), not bitwise."""
    pts = W.theta_batch(70, seed=2)
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(trace_mid)
        ll = eng.loglik(pts)
        gr = eng.loglik_grad(pts, dloglik=np.full(70, 2.0))
        for b in (0, 33, 64, 69):
            l1 = eng.loglik(pts[b:b + 1])
            g1 = eng.loglik_grad(pts[b:b + 1])
            assert abs(l1[0] - ll[b]) <= 1e-9 * abs(ll[b])
            assert np.linalg.norm(2.0 * g1[0] - gr[b]) <= 1e-7 * np.linalg.norm(gr[b])


def test_adjoint_matches_gpu_central_differences(trace_mid):
    """Central differences of the GPU's own log-likelihood (h = 1e-4).  The fp32 weights make the
    log-likelihood accurate to about 1e-8 relative, about 1e-2 absolute here, and that rounding
    changes from one point to the next, so the differences carry up to 1e-2 / 2e-4 = 50 units of
    noise on gradients of 1e4: the check is at 1e-3 relative.  The FP64 gradient of the oracle
    meets central differences at 1e-6 (tests/test_lik_oracle.py) and the GPU adjoint meets that
    FP64 gradient at 1e-6 (above)."""
    pts = W.theta_batch(4, seed=5)
    h = 1e-4
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(trace_mid)
        eng.loglik(pts)
        gr = eng.loglik_grad(pts)
        for b in range(len(pts)):
            shifted = []
            for k in range(4):
                for s in (1.0, -1.0):
                    t = pts[b].copy()
                    t[k] += s * h
                    shifted.append(t)
            l = eng.loglik(np.array(shifted))
            fd = (l[0::2] - l[1::2]) / (2 * h)
            assert np.linalg.norm(fd - gr[b]) / np.linalg.norm(gr[b]) <= 1e-3


def test_adjoint_needs_the_forward_points(trace_mid):
    pts = W.theta_batch(3, seed=8)
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(trace_mid)
        with pytest.raises(PGError):
            eng.loglik_grad(pts)
        eng.loglik(pts)
        with pytest.raises(PGError):
            eng.loglik_grad(pts[:2])
        eng.loglik_grad(pts)


def test_ball_bitmap_in_several_passes(gpu):
    """A seed of 900k nodes needs two shared-memory bitmap passes (786,432 ids each)."""
    g = W.plain_pa_seed(900_000, 10, seed=6)
    prm = W.calibration_params()
    prm.growth_rate = 0.0
    prm.fixed_new_nodes = 3000
    tr = W.grow_trace(g, prm, 1, seed=2)
    pts = np.vstack([THETA_STAR, [0.7, 3.0, 1.5, 6.0]])
    with GrowthEngine(seed=1) as eng:
        eng.load_trace(tr)
        ll = eng.loglik(pts)
        gr = eng.loglik_grad(pts)
    llo, gro = O.loglik(tr, pts)
    assert (np.abs(ll - llo) / np.abs(llo)).max() <= 1e-7
    rel = np.linalg.norm(gr - gro, axis=1) / np.linalg.norm(gro, axis=1)
    assert rel[0] <= 1e-5 and rel[1] <= 1e-6, rel


def test_ball_chunks_rebuilt_per_pass_give_identical_results(trace_mid):
    """Balls kept for all agents at once, or rebuilt chunk by chunk in every pass (what a trace too
    large for memory does): the per-agent arithmetic is the same, so the results are bitwise equal."""
    pts = W.theta_batch(5, seed=4)
    with GrowthEngine(seed=1) as a, GrowthEngine(seed=1) as b:
        a.load_trace(trace_mid)
        b.set_tuning(lik_chunk_agents=700)
        b.load_trace(trace_mid)
        la, lb = a.loglik(pts), b.loglik(pts)
        ga, gb = a.loglik_grad(pts), b.loglik_grad(pts)
    np.testing.assert_array_equal(la, lb)
    np.testing.assert_array_equal(ga, gb)
