"""ctypes wrapper of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the GPU growth engine and the timed CPU baseline.  The
product package (paragraph_gb300) never imports this module; tests/, __graft_entry__.smoke() and
bench.py's CPU legs do.  Parity of this restatement against the reference itself is unpinned (the
reference has no tests, golden vectors or fixed seeds and cannot be built here).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
LIB = _DIR / "_build" / "liboracle.so"
_lib = None


class _Trace(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("pub", C.c_void_p), ("fitness", C.c_void_p),
                ("num_seed_edges", C.c_int64), ("seed_src", C.c_void_p), ("seed_dst", C.c_void_p),
                ("num_epochs", C.c_int32), ("num_anchors", C.c_int32), ("epoch_nodes", C.c_void_p),
                ("epoch_t", C.c_void_p), ("anchors", C.c_void_p), ("cite_off", C.c_void_p),
                ("cites", C.c_void_p)]


def _load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        import sys

        sys.path.insert(0, str(_DIR.parent))
        from paragraph_gb300.build import build_oracle

        build_oracle()
    lib = C.CDLL(str(LIB))
    vp, i32, i64, u64, u32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_uint32
    sig = {
        "og_philox": (None, [vp, vp, vp]),
        "og_logf": (C.c_float, [C.c_float]),
        "og_logf_max_ulp": (C.c_double, [C.c_float, C.c_float]),
        "og_expf": (C.c_float, [C.c_float]),
        "og_log": (C.c_double, [C.c_double]),
        "og_exp": (C.c_double, [C.c_double]),
        "og_poisson_table": (None, [C.c_double, vp]),
        "og_fitness": (C.c_float, [u64, u32, u32, u32]),
        "og_create": (vp, [u64, u32]),
        "og_destroy": (None, [vp]),
        "og_load": (i32, [vp, i64, vp, vp, i64, vp, vp]),
        "og_set_params": (i32, [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, i64, i32]),
        "og_set_epoch": (None, [vp, i64]),
        "og_set_sampler": (None, [vp, i32]),
        "og_epoch": (i64, [vp]),
        "og_pa_epoch": (i32, [vp, i32]),
        "og_er_epoch": (i32, [vp, i64, C.c_double, i32]),
        "og_num_nodes": (i64, [vp]),
        "og_num_edges": (i64, [vp]),
        "og_copy_csr": (None, [vp, i32, vp, vp]),
        "og_copy_degrees": (None, [vp, vp, vp]),
        "og_copy_nodes": (None, [vp, vp, vp]),
        "og_epoch_edges": (None, [vp, C.POINTER(i64), C.POINTER(i64)]),
        "og_copy_arrivals": (None, [vp, vp]),
        "og_stats": (None, [vp, vp]),
        "og_copy_weights": (i64, [vp, vp, vp, C.POINTER(i32)]),
        "og_agent_anchors": (None, [u64, u32, u32, i64, i64, i32, vp]),
        "og_loglik": (i32, [C.POINTER(_Trace), i32, vp, vp, vp, i32]),
        "og_rc_configure": (i32, [vp, vp, vp, i64, vp, i32]),
        "og_rc_bag_table": (None, [vp, i64, vp]),
        "og_rc_fitness_table": (None, [vp]),
        "og_rc_set_nodes": (None, [vp, i64, i64, vp, vp, vp]),
        "og_rc_epoch": (i32, [vp, i32]),
        "og_rc_copy_agents": (None, [vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def philox(counter, key) -> np.ndarray:
    lib = _load()
    c = np.ascontiguousarray(counter, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib.og_philox(_p(c), _p(k), _p(o))
    return o


def logf(x: float) -> float:
    return _load().og_logf(x)


def expf(x: float) -> float:
    return _load().og_expf(x)


def log(x: float) -> float:
    return _load().og_log(x)


def exp(x: float) -> float:
    return _load().og_exp(x)


def poisson_table(lam: float) -> np.ndarray:
    t = np.zeros(257, np.uint64)
    _load().og_poisson_table(lam, _p(t))
    return t


def rc_bag_table(bag) -> np.ndarray:
    b = np.ascontiguousarray(bag, np.int32)
    t = np.zeros(257, np.uint64)
    _load().og_rc_bag_table(_p(b), len(b), _p(t))
    return t


def rc_fitness_table() -> np.ndarray:
    t = np.zeros(1000, np.uint64)
    _load().og_rc_fitness_table(_p(t))
    return t


def fitness(seed: int, replica: int, epoch: int, unit: int) -> float:
    return _load().og_fitness(seed, replica, epoch & 0xFFFFFFFF, unit)


class OracleGraph:
    """One replica's graph state, stepped on the CPU."""

    def __init__(self, seed: int = 42, replica: int = 0):
        self._lib = _load()
        self._g = self._lib.og_create(seed, replica)

    def close(self):
        if self._g:
            self._lib.og_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, pub, fit, src, dst) -> None:
        pub = np.ascontiguousarray(pub, np.int32)
        fit = np.ascontiguousarray(fit, np.float32)
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        st = self._lib.og_load(self._g, len(pub), _p(pub), _p(fit), len(src), _p(src), _p(dst))
        if st:
            raise ValueError(f"og_load failed ({st})")

    def set_params(self, alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=15.0,
                   growth_rate=0.0, fixed_new_nodes=5000, num_anchors=3) -> None:
        st = self._lib.og_set_params(self._g, alpha, tau, gamma, beta, mean_out_degree,
                                     growth_rate, int(fixed_new_nodes), int(num_anchors))
        if st:
            raise ValueError(f"og_set_params failed ({st})")

    def set_epoch(self, e: int) -> None:
        self._lib.og_set_epoch(self._g, e)

    # ---- refcompat functor (ParAGraph's own per-paper model)
    def rc_configure(self, rc, bag, recency) -> None:
        """rc: an object with the fields of paragraph_gb300.RCParams; bag: out-degree bag;
        recency[dy]: recency probability of age dy."""
        prm = np.array([rc.pa_weight, rc.rec_weight, rc.fit_weight, rc.alpha, rc.fully_random,
                        rc.same_year, rc.growth_rate, rc.gamma, rc.decay], np.float64)
        bag = np.ascontiguousarray(bag, np.int32)
        rec = np.ascontiguousarray(recency, np.float64)
        st = self._lib.og_rc_configure(self._g, _p(prm), _p(bag), len(bag), _p(rec), len(rec))
        if st:
            raise ValueError(f"og_rc_configure failed ({st})")

    def rc_set_nodes(self, first: int, lag, peak, dur) -> None:
        lag = np.ascontiguousarray(lag, np.int32)
        peak = np.ascontiguousarray(peak, np.int32)
        dur = np.ascontiguousarray(dur, np.int32)
        self._lib.og_rc_set_nodes(self._g, first, len(lag), _p(lag), _p(peak), _p(dur))

    def rc_epoch(self, threads: int = 0) -> None:
        st = self._lib.og_rc_epoch(self._g, threads)
        if st:
            raise ValueError(f"og_rc_epoch failed ({st})")

    def rc_agents(self) -> np.ndarray:
        """Last refcompat epoch, per agent: pa, rec, fit weights, alpha, generator, out-degree."""
        k = self.n - self.stats()["nodes_weighted"]
        out = np.zeros((k, 6), np.float64)
        self._lib.og_rc_copy_agents(self._g, _p(out))
        return out

    def set_sampler(self, sampler: int) -> None:
        """0: thinning sampler (default); 1: full 2-hop neighbourhood enumeration."""
        self._lib.og_set_sampler(self._g, sampler)

    def pa_epoch(self, threads: int = 0) -> None:
        st = self._lib.og_pa_epoch(self._g, threads)
        if st:
            raise ValueError(f"og_pa_epoch failed ({st})")

    def er_epoch(self, delta: int, p: float, threads: int = 0) -> None:
        st = self._lib.og_er_epoch(self._g, delta, p, threads)
        if st:
            raise ValueError(f"og_er_epoch failed ({st})")

    @property
    def n(self) -> int:
        return self._lib.og_num_nodes(self._g)

    @property
    def m(self) -> int:
        return self._lib.og_num_edges(self._g)

    def csr(self, which: int = 0):
        off = np.empty(self.n + 1, np.int64)
        col = np.empty(max(self.m, 1), np.int32)
        self._lib.og_copy_csr(self._g, which, _p(off), _p(col))
        return off, col[: self.m]

    def degrees(self):
        i = np.empty(self.n, np.int32)
        o = np.empty(self.n, np.int32)
        self._lib.og_copy_degrees(self._g, _p(i), _p(o))
        return i, o

    def nodes(self):
        p = np.empty(self.n, np.int32)
        f = np.empty(self.n, np.float32)
        self._lib.og_copy_nodes(self._g, _p(p), _p(f))
        return p, f

    def epoch_edges(self):
        f, c = C.c_int64(), C.c_int64()
        self._lib.og_epoch_edges(self._g, C.byref(f), C.byref(c))
        return f.value, c.value

    def last_epoch_edges(self):
        first, cnt = self.epoch_edges()
        off, col = self.csr(0)
        src = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(off))
        return src[first:first + cnt], col[first:first + cnt]

    def arrivals(self):
        _, c = self.epoch_edges()
        a = np.empty(max(c, 1), np.int32)
        self._lib.og_copy_arrivals(self._g, _p(a))
        return a[:c]

    def stats(self) -> dict:
        s = np.zeros(6, np.int64)
        self._lib.og_stats(self._g, _p(s))
        return dict(nodes_weighted=int(s[0]), rows_expanded=int(s[1]), elems_streamed=int(s[2]),
                    draws=int(s[3]), new_edges=int(s[4]), adj_scanned=int(s[5]))

    def weights(self):
        n = self._lib.og_copy_weights(self._g, None, None, None)
        w = np.empty(n, np.float32)
        cdf = np.empty(n, np.uint64)
        sh = C.c_int32()
        self._lib.og_copy_weights(self._g, _p(w), _p(cdf), C.byref(sh))
        return w, cdf, sh.value


# ---------------------------------------------------------------- growth traces and their likelihood
class Trace:
    """A growth trace: seed graph, then epochs of agents (agent a is node epoch_nodes[0] + a) with
    anchors ([agents, 4], -1 unused) and citations in draw order (cites[cite_off[a]:cite_off[a+1]])."""

    FIELDS = ("pub", "fitness", "seed_src", "seed_dst", "epoch_nodes", "epoch_t", "anchors",
              "cite_off", "cites")
    DTYPES = (np.int32, np.float32, np.int32, np.int32, np.int64, np.int32, np.int32, np.int64,
              np.int32)

    def __init__(self, num_anchors: int, **arrays):
        self.num_anchors = int(num_anchors)
        for f, dt in zip(self.FIELDS, self.DTYPES):
            setattr(self, f, np.ascontiguousarray(arrays[f], dt))

    @property
    def num_nodes(self) -> int:
        return len(self.pub)

    @property
    def num_epochs(self) -> int:
        return len(self.epoch_t)

    @property
    def agents(self) -> int:
        return len(self.cite_off) - 1


def agent_anchors(seed: int, replica: int, epoch: int, n: int, agents: int, num_anchors: int):
    out = np.empty((agents, 4), np.int32)
    _load().og_agent_anchors(seed, replica, epoch & 0xFFFFFFFF, n, agents, num_anchors, _p(out))
    return out


def grow_trace(g, params, epochs: int, seed: int, sampler: int = 0, replica: int = 0,
               threads: int = 0) -> Trace:
    """Grow `epochs` PA epochs on the CPU from seed graph g and record the trace."""
    og = OracleGraph(seed, replica)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.set_params(**params.__dict__)
    og.set_sampler(sampler)
    ep_nodes, ep_t, anchors, cites, counts = [og.n], [], [], [], []
    for _ in range(epochs):
        n_e, t = og.n, og._lib.og_epoch(og._g)
        og.pa_epoch(threads)
        d = og.n - n_e
        ep_t.append(t)
        anchors.append(agent_anchors(seed, replica, t, n_e, d, params.num_anchors))
        off, _ = og.csr(0)
        counts.append(np.diff(off[n_e:n_e + d + 1]))
        cites.append(og.arrivals())
        ep_nodes.append(og.n)
    pub, fit = og.nodes()
    og.close()
    cnt = np.concatenate(counts)
    return Trace(params.num_anchors, pub=pub, fitness=fit, seed_src=g.src, seed_dst=g.dst,
                 epoch_nodes=np.array(ep_nodes), epoch_t=np.array(ep_t),
                 anchors=np.concatenate(anchors), cite_off=np.concatenate([[0], np.cumsum(cnt)]),
                 cites=np.concatenate(cites))


def loglik(trace, theta, grad: bool = True, threads: int = 0):
    """FP64 log-likelihood (and gradient) of a trace at each row (alpha, tau, gamma, beta) of
    theta.  Returns ll[B] or (ll[B], grad[B, 4])."""
    th = np.ascontiguousarray(np.atleast_2d(theta), np.float64)
    B = th.shape[0]
    ll = np.zeros(B)
    gr = np.zeros((B, 4)) if grad else None
    T = _Trace(trace.num_nodes, _p(trace.pub), _p(trace.fitness), len(trace.seed_src),
               _p(trace.seed_src), _p(trace.seed_dst), trace.num_epochs, trace.num_anchors,
               _p(trace.epoch_nodes), _p(trace.epoch_t), _p(trace.anchors), _p(trace.cite_off),
               _p(trace.cites))
    st = _load().og_loglik(C.byref(T), B, _p(th), _p(ll), _p(gr), threads)
    if st:
        raise ValueError(f"og_loglik failed ({st})")
    return (ll, gr) if grad else ll
