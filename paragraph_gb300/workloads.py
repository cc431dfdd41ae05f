"""Seeded synthetic seed graphs with the shapes of the benchmark configurations.

The reference grows real citation graphs read from edge/node lists (drivers/*.sh pass the "sj"
graph, which is not distributed with it); these generators stand in for them with the sizes and
distributions the benchmark configurations name.  All draws come from numpy's PCG64, so a seed
fixes the graph.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import PAParams, ReplicaInput


@dataclass
class SeedGraph:
    pub: np.ndarray      # int32 publication epoch
    fitness: np.ndarray  # float32 > 0
    src: np.ndarray      # int32 citing node
    dst: np.ndarray      # int32 cited node

    @property
    def n(self) -> int:
        return len(self.pub)

    @property
    def m(self) -> int:
        return len(self.src)


def _distinct_earlier(rng: np.random.Generator, n: int, k: int) -> tuple[np.ndarray, np.ndarray]:
    """Node i cites min(k, i) distinct uniformly random earlier nodes."""
    srcs, dsts = [], []
    small = min(n, k + 1)
    for i in range(1, small):  # nodes 1..k cite every earlier node
        srcs.append(np.full(i, i, np.int32))
        dsts.append(np.arange(i, dtype=np.int32))
    if n > k + 1:
        ids = np.arange(k + 1, n, dtype=np.int64)
        draws = np.floor(rng.random((len(ids), k)) * ids[:, None]).astype(np.int64)
        draws.sort(axis=1)
        dup = np.any(draws[:, 1:] == draws[:, :-1], axis=1)
        for row in np.nonzero(dup)[0]:  # redraw the few rows with a repeated target
            i = int(ids[row])
            draws[row] = np.sort(rng.choice(i, size=k, replace=False))
        srcs.append(np.repeat(ids, k).astype(np.int32))
        dsts.append(draws.reshape(-1).astype(np.int32))
    if not srcs:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    return np.concatenate(srcs), np.concatenate(dsts)


def plain_pa_seed(n: int = 10_000, cites: int = 10, seed: int = 42) -> SeedGraph:
    """Seed DAG: node i cites min(cites, i) earlier nodes; publication epochs uniform over the five
    prior epochs (-5..-1); fitness lognormal(0, 1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    src, dst = _distinct_earlier(rng, n, cites)
    pub = rng.integers(-5, 0, size=n).astype(np.int32)
    fit = rng.lognormal(0.0, 1.0, size=n).astype(np.float32)
    return SeedGraph(pub, fit, src, dst)


def pareto_seed(n: int = 1_000_000, shape: float = 2.5, mean_indeg: float = 16.0,
                seed: int = 42) -> SeedGraph:
    """Seed with Pareto(shape) target in-degrees wired from later nodes.

    Node i draws a target in-degree floor(x_m U^(-1/shape)) (x_m set for the requested mean) and
    receives that many citations from uniformly chosen later nodes; repeated pairs collapse when
    the graph is loaded.  Publication epochs follow id order over the five prior epochs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xm = mean_indeg * (shape - 1.0) / shape
    u = 1.0 - rng.random(n)
    target = np.floor(xm * u ** (-1.0 / shape)).astype(np.int64)
    later = (n - 1) - np.arange(n, dtype=np.int64)
    target = np.minimum(target, later)
    dst = np.repeat(np.arange(n, dtype=np.int64), target)
    span = np.repeat(later, target)
    src = dst + 1 + np.floor(rng.random(len(dst)) * span).astype(np.int64)
    pub = (-5 + (np.arange(n) * 5) // n).astype(np.int32)
    fit = rng.lognormal(0.0, 1.0, size=n).astype(np.float32)
    return SeedGraph(pub, fit, src.astype(np.int32), dst.astype(np.int32))


def er_seed(n: int = 100_000) -> SeedGraph:
    """ER seed: n nodes, no edges."""
    return SeedGraph(np.full(n, -1, np.int32), np.ones(n, np.float32), np.zeros(0, np.int32),
                     np.zeros(0, np.int32))


# ---------------------------------------------------------------- configuration presets
def plain_pa_params() -> PAParams:
    """Plain PA growth: 3 epochs x 5,000 agents, Poisson(15) out-degree, alpha=1, tau=5, gamma=1,
    beta=4, 3 anchors."""
    return PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=15.0,
                    growth_rate=0.0, fixed_new_nodes=5000, num_anchors=3)


def scale_pa_params() -> PAParams:
    """PA at scale: 3 % growth per epoch, Poisson(30) out-degree."""
    return PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=30.0,
                    growth_rate=0.03, fixed_new_nodes=0, num_anchors=3)


def ensemble_inputs(replicas: int = 256, lo: int = 5_000, hi: int = 200_000, epochs: int = 10,
                    seed: int = 42) -> list[ReplicaInput]:
    """Batched ensemble: seed sizes log-uniform in [lo, hi]; per-replica alpha~U[0.5,1.5],
    tau~U[2,10], gamma~U[0.5,2], beta~U[1,8]; Poisson(20) out-degree; 3 % growth."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), replicas)).astype(np.int64)
    out = []
    for r in range(replicas):
        g = plain_pa_seed(int(sizes[r]), 10, seed=seed * 1000 + r)
        p = PAParams(alpha=float(rng.uniform(0.5, 1.5)), tau=float(rng.uniform(2, 10)),
                     gamma=float(rng.uniform(0.5, 2.0)), beta=float(rng.uniform(1, 8)),
                     mean_out_degree=20.0, growth_rate=0.03, fixed_new_nodes=0, num_anchors=3)
        out.append(ReplicaInput(g.pub, g.fitness, g.src, g.dst, p, planned_epochs=epochs))
    return out


def grow_trace(g: SeedGraph, params: PAParams, epochs: int, seed: int = 42,
               device: int = 0) -> "TraceInput":
    """Grow `epochs` PA epochs from seed graph g on the GPU and record the trace (each agent's
    anchors and its citations in draw order)."""
    from . import GrowthEngine, TraceInput

    ep_nodes, ep_t, anchors, cites, counts = [g.n], [], [], [], []
    with GrowthEngine(seed=seed, device=device, record_trace=True) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, params, planned_epochs=epochs)
        for e in range(epochs):
            n_e = eng.counts()[0]
            nn, _ = eng.grow_epoch()
            ep_t.append(e)
            anchors.append(eng.anchors(nn))
            first, cnt = eng.epoch_edges()
            off, _ = eng.csr(0)
            counts.append(np.diff(off[n_e:n_e + nn + 1]))
            cites.append(eng.arrivals())
            ep_nodes.append(n_e + nn)
        pub, fit = eng.nodes()
    cnt = np.concatenate(counts)
    return TraceInput(pub=pub, fitness=fit, seed_src=g.src, seed_dst=g.dst,
                      epoch_nodes=np.array(ep_nodes), epoch_t=np.array(ep_t),
                      anchors=np.concatenate(anchors), cite_off=np.concatenate([[0], np.cumsum(cnt)]),
                      cites=np.concatenate(cites), num_anchors=params.num_anchors)


def calibration_params() -> PAParams:
    """Trace for calibration: theta* = (alpha, tau, gamma, beta) = (1, 5, 1, 4), Poisson(20)
    out-degree, 3 % growth, 3 anchors."""
    return PAParams(alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=20.0,
                    growth_rate=0.03, fixed_new_nodes=0, num_anchors=3)


def theta_batch(points: int = 64, seed: int = 7) -> np.ndarray:
    """Parameter points from the ensemble ranges: alpha~U[0.5,1.5], tau~U[2,10], gamma~U[0.5,2],
    beta~U[1,8]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.stack([rng.uniform(0.5, 1.5, points), rng.uniform(2, 10, points),
                     rng.uniform(0.5, 2.0, points), rng.uniform(1, 8, points)], axis=1)


# ---------------------------------------------------------------- refcompat inputs
def rc_seed(n: int = 10_000, cites: int = 10, seed: int = 42, years: int = 10) -> SeedGraph:
    """Seed for ParAGraph's own model: node i cites min(cites, i) earlier nodes, publication years
    spread over the `years` prior epochs, integer peak fitness drawn from P(v) ~ v^-1.634 over
    1..1000 (the reference's InitializeFitness, src/abm.cu:124-150)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    src, dst = _distinct_earlier(rng, n, cites)
    pub = np.sort(rng.integers(-years, 0, size=n)).astype(np.int32)
    v = np.arange(1, 1001, dtype=np.float64)
    p = v ** -1.634
    fit = rng.choice(v, size=n, p=p / p.sum()).astype(np.float32)
    return SeedGraph(pub, fit, src, dst)


def rc_tables(seed: int = 42, bag_mean: float = 15.0, bag_len: int = 1000,
              ages: int = 40) -> tuple[np.ndarray, np.ndarray]:
    """An out-degree bag (Poisson-like counts, as a list of observed out-degrees) and recency
    probabilities by age (geometric decay), the two input files of the reference's abm driver."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bag = np.clip(rng.poisson(bag_mean, size=bag_len), 0, 300).astype(np.int32)
    rec = 0.8 ** np.arange(ages, dtype=np.float64)
    return bag, rec / rec.sum()
