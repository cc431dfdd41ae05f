"""paragraph_gb300 -- GB300-native per-epoch citation-graph growth (ParAGraph's hot path).

Python mirror of the C ABI in include/paragraph_gb300.h.  The compute path is the in-tree CUDA
library paragraph_gb300/_lib/libparagraph_gb300.so (sm_103a); there is no CPU fallback: if the
library is missing, importing the engine raises.

Reference correspondence (paths inside the ParAGraph project):
  GrowthEngine.load_graph   Graph(edgelist, nodelist) -> ParseNodelist/ParseEdgelist (src/graph.cu:336-447)
  GrowthEngine.grow_epoch   one iteration of execute()'s epoch loop around buildOneNodeConnections_timed
                            (src/kernel.cu:1682-1845, 1125-1586)
  GrowthEngine.er_epoch     the ER G(n,p) step (results/slurm-8634746.out:60-73)
  GrowthEngine.edges        new_edges_vec / WriteGraph rows (src/graph.cu:909-1003)
  GrowthEngine.stats        EpochTiming (includes/epoch_profiler.cuh:56-103)
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libparagraph_gb300.so"

PG_OK, PG_ERR_CUDA, PG_ERR_CAPACITY, PG_ERR_ARG, PG_ERR_TIMEOUT, PG_ERR_IO, PG_ERR_STATE = range(7)
PG_WEIGHTS_BASELINE, PG_WEIGHTS_REFCOMPAT = 0, 1
PG_SAMPLER_THINNING, PG_SAMPLER_ENUMERATE = 0, 1
MAX_OUT_DEGREE = 256

# Every entry point the header declares; tests check the library exports each of them.
EXPORTED = [
    "pg_create", "pg_destroy", "pg_last_error", "pg_status_string", "pg_load_graph",
    "pg_load_replicas", "pg_set_params", "pg_default_params", "pg_set_epoch", "pg_grow_epoch",
    "pg_run_epochs", "pg_run_epochs_out", "pg_er_epoch", "pg_reserve", "pg_get_counts", "pg_epoch_edges", "pg_copy_edges",
    "pg_copy_degrees", "pg_copy_nodes", "pg_copy_csr", "pg_copy_arrivals", "pg_set_timing",
    "pg_get_stats", "pg_sync", "pg_check_device", "pg_philox4x32_10", "pg_poisson_table",
    "pg_logf_host", "pg_expf_host", "pg_log_host", "pg_exp_host", "pg_version",
    "pg_timer_start", "pg_timer_stop", "pg_checkpoint", "pg_restore", "pg_er_generate_noalloc",
    "pg_set_tuning", "pg_get_tuning", "pg_autotune", "pg_copy_anchors", "pg_trace_load",
    "pg_loglik_fwd", "pg_loglik_bwd", "pg_rc_configure", "pg_rc_set_nodes", "pg_rc_copy_agents",
    "pg_rc_bag_table", "pg_rc_fitness_table", "pg_format_edges", "pg_set_wait_limit",
    "pg_format_attributes", "pg_format_g_host", "pg_run_er_epochs", "pg_lik_set_exact_exp2",
]


class PGError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class _Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("num_replicas", C.c_int32), ("seed", C.c_uint64),
                ("weight_model", C.c_int32), ("record_trace", C.c_int32), ("sampler", C.c_int32),
                ("replica_base", C.c_int32)]


class _Params(C.Structure):
    _fields_ = [("alpha", C.c_double), ("tau", C.c_double), ("gamma", C.c_double),
                ("beta", C.c_double), ("mean_out_degree", C.c_double), ("growth_rate", C.c_double),
                ("fixed_new_nodes", C.c_int64), ("num_anchors", C.c_int32), ("reserved", C.c_int32)]


class _RcParams(C.Structure):
    _fields_ = [("pa_weight", C.c_double), ("rec_weight", C.c_double), ("fit_weight", C.c_double),
                ("alpha", C.c_double), ("fully_random", C.c_double), ("same_year", C.c_double),
                ("growth_rate", C.c_double), ("gamma", C.c_int32), ("decay", C.c_int32)]


@dataclass
class RCParams:
    """Parameters of the refcompat functor -- ParAGraph's own model, with the abm driver's
    defaults (src/main.cu:29-114; gamma and decay are constants of the reference,
    includes/abm.cuh:543-553).  A weight or alpha below 0 is drawn per agent."""
    pa_weight: float = -1.0
    rec_weight: float = -1.0
    fit_weight: float = -1.0
    alpha: float = -1.0
    fully_random: float = 0.05
    same_year: float = 0.0
    growth_rate: float = 0.03
    gamma: int = 3
    decay: int = 3


class _ReplicaDesc(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("pub_epoch", C.c_void_p), ("fitness", C.c_void_p),
                ("num_edges", C.c_int64), ("src", C.c_void_p), ("dst", C.c_void_p),
                ("node_capacity", C.c_int64), ("edge_capacity", C.c_int64),
                ("planned_epochs", C.c_int32), ("reserved", C.c_int32), ("params", _Params)]


class _Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "epoch", "new_nodes", "new_edges", "nodes_weighted", "rows_expanded", "elems_streamed",
        "draws", "bwd_moved", "bytes_alg", "bytes_alg_agents")] + [
        (n, C.c_double) for n in ("ms_total", "ms_weights", "ms_setup", "ms_agents", "ms_csr", "ms_er")] + [
        (n, C.c_int64) for n in (
        "run_epochs", "run_new_nodes", "run_new_edges", "run_rows_expanded", "run_elems_streamed",
        "run_draws", "run_bwd_moved", "run_nodes_weighted", "run_bytes_alg", "run_bytes_alg_agents")] + [
        (n, C.c_double) for n in ("run_ms_weights", "run_ms_setup", "run_ms_agents", "run_ms_csr")] + [
        ("run_kernel_launches", C.c_int64), ("adj_scanned", C.c_int64),
        ("run_adj_scanned", C.c_int64), ("lik_ball_elems", C.c_int64),
        ("lik_adj_entries", C.c_int64), ("lik_citations", C.c_int64), ("lik_ms_fwd", C.c_double),
        ("lik_ms_bwd", C.c_double)]


class _AttrRows(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_seed", C.c_int64), ("ids", C.c_void_p),
                ("draws", C.c_void_p), ("ints", C.c_void_p), ("generators", C.c_void_p),
                ("peak_integer", C.c_int32), ("reserved", C.c_int32)]


class _Tuning(C.Structure):
    _fields_ = [("agent_ctas_per_sm", C.c_int32), ("small_hash", C.c_int32),
                ("copy_ctas_per_sm", C.c_int32), ("lik_chunk_agents", C.c_int32),
                ("epoch_kernel", C.c_int32), ("er_slot_sigmas", C.c_int32)]


class _TraceDesc(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("pub_epoch", C.c_void_p), ("fitness", C.c_void_p),
                ("num_seed_edges", C.c_int64), ("seed_src", C.c_void_p), ("seed_dst", C.c_void_p),
                ("num_epochs", C.c_int32), ("num_anchors", C.c_int32), ("epoch_nodes", C.c_void_p),
                ("epoch_t", C.c_void_p), ("anchors", C.c_void_p), ("cite_off", C.c_void_p),
                ("cites", C.c_void_p)]


@dataclass
class PAParams:
    """Baseline weight functor w_j = f_j^gamma (indeg_j+1)^alpha exp(-(t-t_j)/tau) beta^[j in N_a]."""
    alpha: float = 1.0
    tau: float = 5.0
    gamma: float = 1.0
    beta: float = 4.0
    mean_out_degree: float = 15.0
    growth_rate: float = 0.0
    fixed_new_nodes: int = 5000
    num_anchors: int = 3

    def _c(self) -> _Params:
        return _Params(self.alpha, self.tau, self.gamma, self.beta, self.mean_out_degree,
                       self.growth_rate, int(self.fixed_new_nodes), int(self.num_anchors), 0)


@dataclass
class ReplicaInput:
    pub_epoch: np.ndarray
    fitness: np.ndarray
    src: np.ndarray
    dst: np.ndarray
    params: PAParams = field(default_factory=PAParams)
    planned_epochs: int = 1
    node_capacity: int = 0
    edge_capacity: int = 0


@dataclass
class TraceInput:
    """A growth trace: seed graph, then epochs of agents (agent a is node epoch_nodes[0] + a) with
    anchors ([agents, 4], unused -1) and citations in draw order (cites[cite_off[a]:cite_off[a+1]])."""
    pub: np.ndarray
    fitness: np.ndarray
    seed_src: np.ndarray
    seed_dst: np.ndarray
    epoch_nodes: np.ndarray
    epoch_t: np.ndarray
    anchors: np.ndarray
    cite_off: np.ndarray
    cites: np.ndarray
    num_anchors: int = 3

    def __post_init__(self):
        for f, dt in (("pub", np.int32), ("fitness", np.float32), ("seed_src", np.int32),
                      ("seed_dst", np.int32), ("epoch_nodes", np.int64), ("epoch_t", np.int32),
                      ("anchors", np.int32), ("cite_off", np.int64), ("cites", np.int32)):
            setattr(self, f, np.ascontiguousarray(getattr(self, f), dt))

    @property
    def num_nodes(self) -> int:
        return len(self.pub)

    @property
    def num_epochs(self) -> int:
        return len(self.epoch_t)

    @property
    def agents(self) -> int:
        return len(self.cite_off) - 1


_lib = None


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the CUDA library; raises if it has not been built (no fallback path exists)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -m paragraph_gb300.build` "
            "(the growth engine has no CPU fallback)")
    lib = C.CDLL(str(p))
    vp, i32, i64, u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64
    P = C.POINTER
    sig = {
        "pg_create": (i32, [P(vp), P(_Config)]),
        "pg_destroy": (None, [vp]),
        "pg_last_error": (C.c_char_p, [vp]),
        "pg_status_string": (C.c_char_p, [i32]),
        "pg_load_graph": (i32, [vp, i64, vp, vp, i64, vp, vp]),
        "pg_load_replicas": (i32, [vp, P(_ReplicaDesc), i32]),
        "pg_set_params": (i32, [vp, i32, P(_Params)]),
        "pg_default_params": (i32, [P(_Params)]),
        "pg_set_epoch": (i32, [vp, i64]),
        "pg_grow_epoch": (i32, [vp, P(i64), P(i64)]),
        "pg_run_epochs": (i32, [vp, i32, i32, P(i64)]),
        "pg_run_epochs_out": (i32, [vp, i32, i32, vp, vp, i64, vp, P(i64)]),
        "pg_er_epoch": (i32, [vp, i64, C.c_double, P(i64)]),
        "pg_reserve": (i32, [vp, i64, i64]),
        "pg_get_counts": (i32, [vp, i32, P(i64), P(i64)]),
        "pg_epoch_edges": (i32, [vp, i32, P(i64), P(i64)]),
        "pg_copy_edges": (i32, [vp, i32, i64, i64, vp, vp]),
        "pg_copy_degrees": (i32, [vp, i32, vp, vp]),
        "pg_copy_nodes": (i32, [vp, i32, vp, vp]),
        "pg_copy_csr": (i32, [vp, i32, i32, vp, vp]),
        "pg_copy_arrivals": (i32, [vp, i32, vp]),
        "pg_set_timing": (i32, [vp, i32]),
        "pg_get_stats": (i32, [vp, P(_Stats)]),
        "pg_sync": (i32, [vp]),
        "pg_check_device": (i32, [vp]),
        "pg_philox4x32_10": (None, [vp, vp, vp]),
        "pg_poisson_table": (i32, [C.c_double, vp]),
        "pg_logf_host": (C.c_float, [C.c_float]),
        "pg_expf_host": (C.c_float, [C.c_float]),
        "pg_log_host": (C.c_double, [C.c_double]),
        "pg_exp_host": (C.c_double, [C.c_double]),
        "pg_version": (C.c_char_p, []),
        "pg_timer_start": (i32, [vp]),
        "pg_timer_stop": (i32, [vp, P(C.c_double)]),
        "pg_checkpoint": (i32, [vp]),
        "pg_restore": (i32, [vp]),
        "pg_er_generate_noalloc": (i32, [u64, i64, i64, i64, C.c_double, vp, vp, i64, P(i64), vp]),
        "pg_set_tuning": (i32, [vp, P(_Tuning)]),
        "pg_get_tuning": (i32, [vp, P(_Tuning)]),
        "pg_autotune": (i32, [vp, i32, P(_Tuning), P(C.c_double)]),
        "pg_copy_anchors": (i32, [vp, i32, vp]),
        "pg_trace_load": (i32, [vp, P(_TraceDesc)]),
        "pg_loglik_fwd": (i32, [vp, i32, vp, vp]),
        "pg_loglik_bwd": (i32, [vp, i32, vp, vp, vp]),
        "pg_rc_configure": (i32, [vp, i32, P(_RcParams), vp, i64, vp, i32]),
        "pg_rc_set_nodes": (i32, [vp, i32, i64, i64, vp, vp, vp]),
        "pg_rc_copy_agents": (i32, [vp, i32, vp]),
        "pg_rc_bag_table": (i32, [vp, i64, vp]),
        "pg_rc_fitness_table": (i32, [vp]),
        "pg_format_edges": (i32, [vp, i32, vp, i64, vp, i64, P(i64)]),
        "pg_set_wait_limit": (i32, [vp, i64]),
        "pg_format_attributes": (i32, [vp, i32, P(_AttrRows), vp, i64, P(i64)]),
        "pg_format_g_host": (i32, [C.c_double, i32, C.c_char_p]),
        "pg_run_er_epochs": (i32, [vp, i32, i64, C.c_double, P(i64)]),
        "pg_lik_set_exact_exp2": (i32, [vp, i32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def philox(counter, key) -> np.ndarray:
    """Philox4x32-10 block of the library (host build of the shared header)."""
    lib = load_library()
    c = np.ascontiguousarray(counter, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    lib.pg_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def rc_bag_table(bag) -> np.ndarray:
    b = np.ascontiguousarray(bag, np.int32)
    t = np.zeros(MAX_OUT_DEGREE + 1, np.uint64)
    if load_library().pg_rc_bag_table(_ptr(b), len(b), _ptr(t)) != PG_OK:
        raise PGError(PG_ERR_ARG, "empty bag")
    return t


def rc_fitness_table() -> np.ndarray:
    t = np.zeros(1000, np.uint64)
    load_library().pg_rc_fitness_table(_ptr(t))
    return t


def poisson_table(lam: float) -> np.ndarray:
    lib = load_library()
    t = np.zeros(MAX_OUT_DEGREE + 1, np.uint64)
    if lib.pg_poisson_table(float(lam), _ptr(t)) != PG_OK:
        raise PGError(PG_ERR_ARG, "bad lambda")
    return t


class GrowthEngine:
    """One device context holding R replicas (R == 1: the drop-in growth step)."""

    def __init__(self, seed: int = 42, replicas: int = 1, device: int = 0,
                 record_trace: bool = False, weight_model: int = PG_WEIGHTS_BASELINE,
                 sampler: int = PG_SAMPLER_THINNING, replica_base: int = 0):
        self._lib = load_library()
        self._ctx = C.c_void_p()
        cfg = _Config(device, replicas, seed, weight_model, 1 if record_trace else 0, sampler,
                      replica_base)
        st = self._lib.pg_create(C.byref(self._ctx), C.byref(cfg))
        if st != PG_OK:
            msg = self._lib.pg_last_error(self._ctx).decode() if self._ctx else "pg_create failed"
            self.close()
            raise PGError(st, msg)
        self.replicas = replicas
        self.record_trace = record_trace

    # ------------------------------------------------------------------ lifecycle
    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.pg_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        if st != PG_OK:
            raise PGError(st, self._lib.pg_last_error(self._ctx).decode())

    # ------------------------------------------------------------------ input
    def load_graph(self, pub_epoch, fitness, src, dst, params: PAParams | None = None,
                   planned_epochs: int = 1) -> None:
        self.load_replicas([ReplicaInput(pub_epoch, fitness, src, dst, params or PAParams(),
                                         planned_epochs)])

    def load_replicas(self, reps: list[ReplicaInput]) -> None:
        keep = []
        descs = (_ReplicaDesc * len(reps))()
        for d, r in zip(descs, reps):
            pub = np.ascontiguousarray(r.pub_epoch, np.int32)
            fit = np.ascontiguousarray(r.fitness, np.float32)
            s = np.ascontiguousarray(r.src, np.int32)
            t = np.ascontiguousarray(r.dst, np.int32)
            keep += [pub, fit, s, t]
            d.num_nodes = len(pub)
            d.pub_epoch = pub.ctypes.data
            d.fitness = fit.ctypes.data
            d.num_edges = len(s)
            d.src = s.ctypes.data if len(s) else None
            d.dst = t.ctypes.data if len(t) else None
            d.node_capacity = r.node_capacity
            d.edge_capacity = r.edge_capacity
            d.planned_epochs = r.planned_epochs
            d.params = r.params._c()
        self._check(self._lib.pg_load_replicas(self._ctx, descs, len(reps)))

    def set_params(self, params: PAParams, replica: int = 0) -> None:
        p = params._c()
        self._check(self._lib.pg_set_params(self._ctx, replica, C.byref(p)))

    # ---------------------------------------------------------------- refcompat functor
    def rc_configure(self, rc: "RCParams", bag, recency, replica: int = 0) -> None:
        """ParAGraph's own model for `replica` (context created with PG_WEIGHTS_REFCOMPAT):
        parameters, out-degree bag and recency probabilities recency[age]."""
        prm = _RcParams(rc.pa_weight, rc.rec_weight, rc.fit_weight, rc.alpha, rc.fully_random,
                        rc.same_year, rc.growth_rate, int(rc.gamma), int(rc.decay))
        b = np.ascontiguousarray(bag, np.int32)
        r = np.ascontiguousarray(recency, np.float64)
        self._check(self._lib.pg_rc_configure(self._ctx, replica, C.byref(prm), _ptr(b), len(b),
                                              _ptr(r) if len(r) else None, len(r)))

    def rc_set_nodes(self, first: int, lag, peak, dur, replica: int = 0) -> None:
        """Fitness windows (lag, peak value, duration) of papers [first, first + len(lag))."""
        lag = np.ascontiguousarray(lag, np.int32)
        peak = np.ascontiguousarray(peak, np.int32)
        dur = np.ascontiguousarray(dur, np.int32)
        self._check(self._lib.pg_rc_set_nodes(self._ctx, replica, first, len(lag), _ptr(lag),
                                              _ptr(peak), _ptr(dur)))

    def rc_agents(self, replica: int = 0) -> np.ndarray:
        """Last refcompat epoch, per new paper: pa, rec, fit weights, alpha, generator, out-degree."""
        k = self.stats()["new_nodes"] if self.replicas == 1 else None
        if k is None:
            raise PGError(PG_ERR_ARG, "rc_agents of a multi-replica context: use the C ABI")
        out = np.zeros((k, 6), np.float64)
        self._check(self._lib.pg_rc_copy_agents(self._ctx, replica, _ptr(out)))
        return out

    def set_epoch(self, epoch: int) -> None:
        self._check(self._lib.pg_set_epoch(self._ctx, epoch))

    # ------------------------------------------------------------------ growth
    def grow_epoch(self) -> tuple[int, int]:
        nn, ne = C.c_int64(), C.c_int64()
        self._check(self._lib.pg_grow_epoch(self._ctx, C.byref(nn), C.byref(ne)))
        return nn.value, ne.value

    def run_epochs(self, epochs: int, use_graph: bool = True) -> int:
        ne = C.c_int64()
        self._check(self._lib.pg_run_epochs(self._ctx, epochs, 1 if use_graph else 0, C.byref(ne)))
        return ne.value

    def run_epochs_out(self, epochs: int, out: tuple[np.ndarray, np.ndarray],
                       use_graph: bool = True) -> tuple[int, np.ndarray]:
        """run_epochs that also writes every new citation (source, target) into the caller's
        int32 buffers `out`, epoch by epoch and replica by replica; page-locked buffers are written
        from the device while the run goes on.  Returns (new citations, counts[epoch, replica])."""
        s, d = out
        if (s.dtype != np.int32 or d.dtype != np.int32 or not s.flags.c_contiguous
                or not d.flags.c_contiguous or len(s) != len(d)):
            raise PGError(PG_ERR_ARG, "out buffers must be contiguous int32 arrays of one length")
        counts = np.zeros((epochs, self.replicas), np.int64)
        ne = C.c_int64()
        self._check(self._lib.pg_run_epochs_out(self._ctx, epochs, 1 if use_graph else 0, _ptr(s), _ptr(d),
                                                len(s), _ptr(counts), C.byref(ne)))
        return ne.value, counts

    def er_epoch(self, delta: int, p: float) -> int:
        ne = C.c_int64()
        self._check(self._lib.pg_er_epoch(self._ctx, delta, p, C.byref(ne)))
        return ne.value

    def run_er_epochs(self, epochs: int, delta: int, p: float) -> int:
        """`epochs` ER epochs of `delta` new nodes without host synchronisation between them."""
        ne = C.c_int64()
        self._check(self._lib.pg_run_er_epochs(self._ctx, int(epochs), int(delta), float(p), C.byref(ne)))
        return ne.value

    def reserve(self, n_cap: int, m_cap: int) -> None:
        """Grow a single-replica context to n_cap nodes and m_cap citations ahead of its epochs."""
        self._check(self._lib.pg_reserve(self._ctx, int(n_cap), int(m_cap)))

    # ------------------------------------------------------------------ output
    def counts(self, replica: int = 0) -> tuple[int, int]:
        n, m = C.c_int64(), C.c_int64()
        self._check(self._lib.pg_get_counts(self._ctx, replica, C.byref(n), C.byref(m)))
        return n.value, m.value

    def epoch_edges(self, replica: int = 0) -> tuple[int, int]:
        f, c = C.c_int64(), C.c_int64()
        self._check(self._lib.pg_epoch_edges(self._ctx, replica, C.byref(f), C.byref(c)))
        return f.value, c.value

    def edges(self, first: int, count: int, replica: int = 0,
              out: tuple[np.ndarray, np.ndarray] | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Edges [first, first + count) in forward-CSR order; `out` may hold caller-owned int32
        buffers of at least `count` entries (e.g. page-locked memory for a faster copy)."""
        if out is None:
            s = np.empty(count, np.int32)
            d = np.empty(count, np.int32)
        else:
            s, d = out
            if (s.dtype != np.int32 or d.dtype != np.int32 or len(s) < count or len(d) < count
                    or not s.flags.c_contiguous or not d.flags.c_contiguous):
                raise PGError(PG_ERR_ARG, "out buffers must be contiguous int32 of >= count entries")
        self._check(self._lib.pg_copy_edges(self._ctx, replica, first, count, _ptr(s), _ptr(d)))
        return s[:count], d[:count]

    def format_edges(self, ids, replica: int = 0) -> bytes:
        """The edge list as "source,target\\n" text with node v printed as ids[v], formatted on the
        device (the rows of the reference's WriteGraph)."""
        ids = np.ascontiguousarray(ids, np.int64)
        size = C.c_int64()
        self._check(self._lib.pg_format_edges(self._ctx, replica, _ptr(ids), len(ids), None, 0,
                                              C.byref(size)))
        buf = C.create_string_buffer(max(size.value, 1))
        self._check(self._lib.pg_format_edges(self._ctx, replica, _ptr(ids), len(ids), buf,
                                              size.value, C.byref(size)))
        return buf.raw[:size.value]

    def format_attributes(self, ids, draws, ints, generators, num_seed: int, peak_integer: bool,
                          replica: int = 0) -> bytes:
        """The attribute-file rows (Graph::WriteAttributes) formatted on the device: ids[n],
        draws[n, 4] (pa, rec, fit weight, alpha), ints[n, 4] (lag, duration, assigned out-degree,
        planted line), generators[n, 4] (printed ids, -1 unused); nodes below num_seed are seeds."""
        ids = np.ascontiguousarray(ids, np.int64)
        draws = np.ascontiguousarray(draws, np.float64)
        ints = np.ascontiguousarray(ints, np.int32)
        gens = np.ascontiguousarray(generators, np.int64)
        rows = _AttrRows(len(ids), int(num_seed), ids.ctypes.data, draws.ctypes.data, ints.ctypes.data,
                         gens.ctypes.data, 1 if peak_integer else 0, 0)
        size = C.c_int64()
        self._check(self._lib.pg_format_attributes(self._ctx, replica, C.byref(rows), None, 0, C.byref(size)))
        buf = C.create_string_buffer(max(size.value, 1))
        self._check(self._lib.pg_format_attributes(self._ctx, replica, C.byref(rows), buf, size.value,
                                                   C.byref(size)))
        return buf.raw[:size.value]

    def last_epoch_edges(self, replica: int = 0) -> tuple[np.ndarray, np.ndarray]:
        f, c = self.epoch_edges(replica)
        return self.edges(f, c, replica)

    def degrees(self, replica: int = 0) -> tuple[np.ndarray, np.ndarray]:
        n, _ = self.counts(replica)
        i = np.empty(n, np.int32)
        o = np.empty(n, np.int32)
        self._check(self._lib.pg_copy_degrees(self._ctx, replica, _ptr(i), _ptr(o)))
        return i, o

    def nodes(self, replica: int = 0) -> tuple[np.ndarray, np.ndarray]:
        n, _ = self.counts(replica)
        p = np.empty(n, np.int32)
        f = np.empty(n, np.float32)
        self._check(self._lib.pg_copy_nodes(self._ctx, replica, _ptr(p), _ptr(f)))
        return p, f

    def csr(self, which: int = 0, replica: int = 0) -> tuple[np.ndarray, np.ndarray]:
        n, m = self.counts(replica)
        off = np.empty(n + 1, np.int64)
        col = np.empty(max(m, 1), np.int32)
        self._check(self._lib.pg_copy_csr(self._ctx, replica, which, _ptr(off), _ptr(col)))
        return off, col[:m]

    def arrivals(self, replica: int = 0) -> np.ndarray:
        _, c = self.epoch_edges(replica)
        a = np.empty(max(c, 1), np.int32)
        self._check(self._lib.pg_copy_arrivals(self._ctx, replica, _ptr(a)))
        return a[:c]

    def anchors(self, count: int | None = None, replica: int = 0) -> np.ndarray:
        """Anchors of the last PA epoch's agents, [count, 4] (needs record_trace); count defaults
        to the epoch's new nodes of a single-replica context."""
        d = int(self.stats()["new_nodes"]) if count is None else int(count)
        a = np.empty((max(d, 1), 4), np.int32)
        self._check(self._lib.pg_copy_anchors(self._ctx, replica, _ptr(a)))
        return a[:d]

    def set_timing(self, enable: bool) -> None:
        self._check(self._lib.pg_set_timing(self._ctx, 1 if enable else 0))

    def stats(self) -> dict:
        s = _Stats()
        self._check(self._lib.pg_get_stats(self._ctx, C.byref(s)))
        return {name: getattr(s, name) for name, _ in _Stats._fields_}

    def sync(self) -> None:
        self._check(self._lib.pg_sync(self._ctx))

    def check_device(self) -> None:
        self._check(self._lib.pg_check_device(self._ctx))

    def timer_start(self) -> None:
        self._check(self._lib.pg_timer_start(self._ctx))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._check(self._lib.pg_timer_stop(self._ctx, C.byref(ms)))
        return ms.value

    def checkpoint(self) -> None:
        """Save the graph state in device memory (checkpoint/resume is bit-exact)."""
        self._check(self._lib.pg_checkpoint(self._ctx))

    def restore(self) -> None:
        self._check(self._lib.pg_restore(self._ctx))

    def set_tuning(self, agent_ctas_per_sm: int = 0, small_hash: int = 0,
                   copy_ctas_per_sm: int = 0, lik_chunk_agents: int = 0, epoch_kernel: int = 0,
                   er_slot_sigmas: int = 0) -> None:
        """Launch shape of the agent and moved-row copy kernels, the likelihood's ball chunking,
        one persistent kernel per epoch, and the ER walks' slot reservation (results never depend
        on them)."""
        t = _Tuning(agent_ctas_per_sm, small_hash, copy_ctas_per_sm, lik_chunk_agents, epoch_kernel,
                    er_slot_sigmas)
        self._check(self._lib.pg_set_tuning(self._ctx, C.byref(t)))

    def set_wait_limit(self, polls: int) -> None:
        """Failure-path hook: polls of the first bounded wait on each staged copy of the agent
        kernel (0: give up at once, < 0: the default).  A wait that gives up fails the epoch with
        PG_ERR_TIMEOUT."""
        self._check(self._lib.pg_set_wait_limit(self._ctx, int(polls)))

    def tuning(self) -> dict:
        t = _Tuning()
        self._check(self._lib.pg_get_tuning(self._ctx, C.byref(t)))
        return {k: getattr(t, k) for k, _ in _Tuning._fields_}

    def autotune(self, epochs: int) -> tuple[dict, float]:
        """Time the candidate tunings on the next `epochs` epochs, keep the fastest; the graph is
        left as it was.  Returns (tuning, milliseconds of the best candidate)."""
        t = _Tuning()
        ms = C.c_double()
        self._check(self._lib.pg_autotune(self._ctx, int(epochs), C.byref(t), C.byref(ms)))
        return {k: getattr(t, k) for k, _ in _Tuning._fields_}, ms.value

    # ---------------------------------------------------------------- trace log-likelihood
    def load_trace(self, t: TraceInput) -> None:
        """Copy a growth trace to the device for loglik / loglik_grad."""
        self._trace = t  # keeps the arrays alive while the descriptor points at them
        d = _TraceDesc(t.num_nodes, _ptr(t.pub), _ptr(t.fitness), len(t.seed_src), _ptr(t.seed_src),
                       _ptr(t.seed_dst), t.num_epochs, t.num_anchors, _ptr(t.epoch_nodes),
                       _ptr(t.epoch_t), _ptr(t.anchors), _ptr(t.cite_off), _ptr(t.cites))
        self._check(self._lib.pg_trace_load(self._ctx, C.byref(d)))

    def set_lik_exact_exp2(self, exact: bool) -> None:
        """Arithmetic of the next likelihood passes: True carries the weight exponent without
        rounding of its own, takes 2^x from an fp32 exp2 accurate to ~2 ulp and sums every ball
        weight and product on its own (the gradient stays within 1e-6 of the FP64 value even where
        it nearly vanishes); False (default) uses the special-function unit's exp2 of a once-rounded
        exponent and pairwise ball sums, about three times as fast."""
        self._check(self._lib.pg_lik_set_exact_exp2(self._ctx, 1 if exact else 0))

    def loglik(self, theta) -> np.ndarray:
        """log L at each row (alpha, tau, gamma, beta) of theta (forward pass)."""
        th = np.ascontiguousarray(np.atleast_2d(theta), np.float64)
        out = np.empty(th.shape[0])
        self._check(self._lib.pg_loglik_fwd(self._ctx, th.shape[0], _ptr(th), _ptr(out)))
        return out

    def loglik_grad(self, theta, dloglik=None) -> np.ndarray:
        """Adjoint pass at the points of the last loglik call: [B, 4] gradient (times dloglik)."""
        th = np.ascontiguousarray(np.atleast_2d(theta), np.float64)
        g = np.empty((th.shape[0], 4))
        dl = None if dloglik is None else np.ascontiguousarray(dloglik, np.float64)
        self._check(self._lib.pg_loglik_bwd(self._ctx, th.shape[0], _ptr(th), _ptr(dl), _ptr(g)))
        return g
