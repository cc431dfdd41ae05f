"""Benchmark of the per-epoch graph-growth step (citation edges per second on one GB300).

Default workload -- PA at scale: a 1,000,000-node seed with Pareto(2.5) in-degrees (about 15.4M
citations), grown 30 epochs at 3 % per epoch (about 2.43M nodes and 44M new citations), Poisson(30)
out-degree, alpha=1, tau=5, gamma=1, beta=4, 2-hop neighbourhoods of 3 anchors.  One step regrows all
30 epochs from the device-resident seed (restore + one CUDA-graph replay).  Inputs are synthetic
(seeded numpy), the working set (CSR arrays, 0.5-0.9 GB) is larger than L2 (129 MB).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value   = new citations of the K timed steps / their device time (CUDA events on the engine's
          stream, inputs resident in HBM), max over ranks, summed over ranks.
e2e     = the same metric through the C ABI from page-locked host buffers: load the seed (raw edge
          arrays H2D, CSR built on the device), grow 30 epochs, copy every new citation back (D2H),
          wall clock.
roofline: the agent kernel (dominant), algorithmic bytes / its summed CUDA-event time.
cpu_baseline: the CPU oracle (OpenMP, all host threads) on a bounded sample of the same workload.
--impl reference times that CPU path alone (the reference itself cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "pa_scale_1M_seed_30_epochs_3pct"
EPOCHS = 30


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return world, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def workload_config(g) -> dict:
    """The workload as both arms name it (the reference arm times a bounded sample of it, stated in
    its cpu_baseline.sample)."""
    return {"workload": WORKLOAD, "seed_nodes": g.n, "seed_citations": g.m,
            "epochs_per_step": EPOCHS, "growth": 0.03, "mean_out_degree": 30,
            "alpha": 1.0, "tau": 5.0, "gamma": 1.0, "beta": 4.0, "anchors": 3,
            "l2": "inputs larger than L2 (CSR 0.5-0.9 GB)", "parallelism": "replicas only"}


def seed_graph(seed: int):
    from paragraph_gb300 import workloads as W

    return W.pareto_seed(1_000_000, 2.5, 16.0, seed=seed), W.scale_pa_params()


def traffic_per_agent_byte() -> float | None:
    """DRAM bytes per algorithmic byte of the agent kernel, from the committed ncu summary."""
    p = ROOT / "profiles" / "agents_traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return float(d["dram_bytes"]) / float(d["bytes_alg"])
    except Exception:
        return None


# ------------------------------------------------------------------ CPU legs (oracle)
def cpu_sample(g, prm, seed: int, max_epochs: int = 3, budget_s: float = 12.0,
               sampler: int = 1, threads: int = 0) -> dict:
    """Time the OpenMP oracle (all host threads) on the first epochs of the workload.

    sampler 1 (default) is the reference's algorithm -- enumerate each agent's 2-hop neighbourhood
    and key every candidate (src/abm.cu:461-565,577-682); sampler 0 is this project's thinning
    sampler run on the CPU."""
    import oracle as O

    og = O.OracleGraph(seed, 0)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.set_params(**prm.__dict__)
    og.set_sampler(sampler)
    threads = threads or os.cpu_count() or 1
    edges, secs, epochs = 0, 0.0, 0
    while epochs < max_epochs and (epochs == 0 or secs < budget_s):
        m0 = og.m
        t0 = time.perf_counter()
        og.pa_epoch(threads)
        secs += time.perf_counter() - t0
        edges += og.m - m0
        epochs += 1
    og.close()
    algo = "neighbourhood enumeration (the reference's algorithm)" if sampler else "thinning sampler"
    return {"value": edges / secs, "unit": "citations/s", "cores": threads, "kind": "port",
            "sample": f"first {epochs} epoch(s) of the workload from the seed ({edges} citations, "
                      f"{secs:.1f} s), CPU oracle with OpenMP, {algo}"}


def run_reference(args) -> None:
    world, rank, _, dist = dist_setup()
    if rank != 0:
        barrier(dist)
        return
    import oracle as O

    g, prm = seed_graph(args.seed)
    threads = os.cpu_count() or 1
    # each step = epoch 0 of the workload from the seed (a bounded sample; the oracle reloads the
    # seed between steps outside the timed region)
    def one_step():
        og2 = O.OracleGraph(args.seed, 0)
        og2.load(g.pub, g.fitness, g.src, g.dst)
        og2.set_params(**prm.__dict__)
        og2.set_sampler(1)  # the reference's algorithm: enumerate the 2-hop neighbourhood
        t0 = time.perf_counter()
        og2.pa_epoch(threads)
        dt = time.perf_counter() - t0
        e = og2.epoch_edges()[1]
        og2.close()
        return e, dt

    for _ in range(args.warmup):
        one_step()
    edges, secs = 0, 0.0
    for _ in range(args.steps):
        e, dt = one_step()
        edges += e
        secs += dt
    v = edges / secs
    line = {"metric": "citation edges/sec (PA growth step)", "value": v, "unit": "citations/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/u64/f32", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(g),
            "cpu_baseline": {"value": v, "unit": "citations/s", "cores": threads, "kind": "port",
                             "sample": "epoch 0 of the workload per step (the 30-epoch step is "
                                       "out of reach: the enumerated 2-hop balls grow to millions "
                                       "of nodes per agent), the reference's algorithm (2-hop "
                                       "enumeration, ES top-k) in the CPU oracle on all host "
                                       "threads; the reference itself cannot be built "
                                       "(cuCollections is absent)"},
            "e2e": {"value": v, "unit": "citations/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)
    barrier(dist)


# ------------------------------------------------------------------ GPU leg
def run_ours(args) -> None:
    world, rank, local, dist = dist_setup()
    from paragraph_gb300 import GrowthEngine

    seed = args.seed + rank
    g, prm = seed_graph(seed)
    eng = GrowthEngine(seed=seed, device=local)
    eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=EPOCHS)
    eng.checkpoint()
    if args.small_hash is not None:
        eng.set_tuning(small_hash=args.small_hash)
    if args.autotune:
        eng.autotune(EPOCHS)  # untimed; the graph is left as it was
    tuned = eng.tuning()

    def step():
        eng.restore()
        return eng.run_epochs(EPOCHS, use_graph=True)

    for _ in range(args.warmup):
        step()
    agents_ms = agents_bytes = 0.0
    edges = 0
    launches = 0
    barrier(dist)
    eng.sync()
    with ClockSampler(local) as clocks:
        t_wall = time.perf_counter()
        eng.timer_start()
        for _ in range(args.steps):
            edges += step()
            st = eng.stats()
            agents_ms += st["run_ms_agents"]
            agents_bytes += st["run_bytes_alg_agents"]
            launches += st["run_kernel_launches"]
        ms = eng.timer_stop()
        wall = time.perf_counter() - t_wall
    barrier(dist)
    ms_max = reduce_max(dist, ms)
    edges_all = reduce_sum(dist, float(edges))
    value = edges_all / (ms_max / 1000.0)

    # end to end through the C ABI from host buffers
    e2e = None
    if not args.no_e2e:
        import torch

        # page-locked host buffers, filled before the timed region: the seed's raw arrays in,
        # every new citation (source, target) out
        def pinned(a):
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

        hp, hf, hs, hd = pinned(g.pub), pinned(g.fitness), pinned(g.src), pinned(g.dst)
        cap = int(edges // max(1, args.steps)) + 1
        out = (torch.empty(cap, dtype=torch.int32).pin_memory().numpy(),
               torch.empty(cap, dtype=torch.int32).pin_memory().numpy())
        e2e_edges, e2e_secs = 0, 0.0
        h2d = d2h = 0
        for i in range(max(1, args.e2e_steps)):
            with GrowthEngine(seed=seed, device=local) as e2:
                e2.set_tuning(**tuned)
                t0 = time.perf_counter()
                e2.load_graph(hp, hf, hs, hd, prm, planned_epochs=EPOCHS)
                n0, m0 = e2.counts()
                # every epoch's citations are written into the page-locked buffers while the
                # following epochs run
                ne, _ = e2.run_epochs_out(EPOCHS, out, use_graph=False)
                n1, m1 = e2.counts()
                dt = time.perf_counter() - t0
            e2e_edges += ne
            e2e_secs += dt
            h2d = 4 * g.n * 2 + 4 * g.m * 2  # publication epochs, fitness, raw sources and targets
            d2h = 8 * (m1 - m0)  # every new citation: source and target
        e2e = {"value": e2e_edges / e2e_secs, "unit": "citations/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "inputs": "page-locked host buffers; seed CSR built on the device"}

    if rank != 0:
        eng.close()
        if not args.no_extra:
            extra_lines(args, world, rank, local, dist)
        return
    peak, peak_kind = peaks()
    achieved = agents_bytes / (agents_ms / 1000.0) / 1e9 if agents_ms > 0 else 0.0
    ratio = traffic_per_agent_byte()
    per_launch_alg = agents_bytes / max(1, args.steps * EPOCHS * 2)
    line = {
        "metric": "citation edges/sec (PA growth step)",
        "value": value, "unit": "citations/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32/u64/f32", "data": "synthetic",
        "config": {**workload_config(g), "tuning": tuned},
        "roofline": {"bound": "hbm", "kernel": "k_agents", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": per_launch_alg * ratio if ratio else None},
        "e2e": e2e,
        "gpu_launches": launches,
        "wall_s": wall,
        "clocks": clocks.summary(),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(g, prm, seed, sampler=1)
        line["cpu_thinning"] = cpu_sample(g, prm, seed, sampler=0, max_epochs=2, budget_s=5.0)
        line["cpu_baseline_1thread"] = cpu_sample(g, prm, seed, sampler=1, max_epochs=1, threads=1)
    eng.close()
    if not args.no_extra:
        line["ensemble"], line["loglik"] = extra_lines(args, world, rank, local, dist)
    print(json.dumps(line), flush=True)


def extra_lines(args, world, rank, local, dist) -> tuple[dict | None, dict | None]:
    """The batched-ensemble and calibration measurements in short form for the default line (5
    timed steps each, their own CUDA-event timing and serial loops; see --ensemble and --loglik for
    the full lines)."""
    import copy

    a = copy.copy(args)
    a.steps, a.warmup = min(args.steps, 5), 3
    ens = ensemble_measure(a, world, rank, local, dist, with_cpu=False)
    lik = loglik_measure(a, world, rank, local, dist, with_cpu=not args.no_cpu)
    if ens is None or lik is None:
        return None, None
    e = {"value": ens["value"], "unit": ens["unit"], "workload": ENS_WORKLOAD,
         "serial_speedup": ens["serial"]["speedup_device"],
         "serial_speedup_wall": ens["serial"]["speedup_wall"],
         "citations_per_s": ens["citations_per_s"], "e2e": ens["e2e"],
         "gpu_launches_per_step": ens["gpu_launches"] / a.steps, "steps": a.steps,
         "tuning": ens["config"]["tuning"], "device_ms_per_step": ens["config"]["device_ms_per_step"]}
    cb = lik.get("cpu_baseline") or {}
    l = {"value": lik["value"], "unit": lik["unit"], "workload": LIK_WORKLOAD,
         "serial_speedup": lik["serial"]["speedup"], "e2e": lik["e2e"],
         "grad_rel_err_vs_fp64": cb.get("grad_rel_err_vs_fp64"),
         "loglik_rel_err_vs_fp64": cb.get("loglik_rel_err_vs_fp64"),
         "roofline_frac": lik["roofline"]["frac"], "steps": a.steps}
    return e, l


ENS_REPLICAS, ENS_EPOCHS = 256, 10
ENS_WORKLOAD = "ensemble_256_replicas_5k_200k_10_epochs_3pct"


def run_ensemble(args) -> None:
    line = ensemble_measure(args, *dist_setup(), with_cpu=not args.no_cpu)
    if line is not None:
        print(json.dumps(line), flush=True)


def ensemble_measure(args, world, rank, local, dist, with_cpu: bool = True) -> dict | None:
    """Batched ensemble: 256 replicas (seed sizes log-uniform in [5k, 200k], per-replica alpha,
    tau, gamma, beta, Poisson(20), 3 % growth) grown 10 epochs in ONE context -- one launch of each
    epoch kernel over all replicas, the 10 epochs captured as one CUDA graph, launch shape picked by
    the engine's autotuner.  The same replicas grown serially, one single-replica context each
    (the plain per-replica method), give the serial time.  An eval is one replica grown 10 epochs.
    Under torchrun the replicas are split across ranks (no exchange).  Returns rank 0's line."""
    from paragraph_gb300 import GrowthEngine
    from paragraph_gb300 import workloads as W

    reps_all = W.ensemble_inputs(replicas=ENS_REPLICAS, lo=5_000, hi=200_000, epochs=ENS_EPOCHS,
                                 seed=args.seed)
    idx = list(range(rank, ENS_REPLICAS, world))
    reps = [reps_all[i] for i in idx]
    eng = GrowthEngine(seed=args.seed, replicas=len(reps), device=local)
    eng.load_replicas(reps)
    tuned, tune_ms = eng.autotune(ENS_EPOCHS)
    eng.checkpoint()
    m_seed = [eng.counts(r)[1] for r in range(len(reps))]

    def step():
        eng.restore()
        return eng.run_epochs(ENS_EPOCHS, use_graph=True)

    for _ in range(args.warmup):
        step()
    new_edges = [eng.counts(r)[1] - m_seed[r] for r in range(len(reps))]
    barrier(dist)
    edges, dev_ms, wall = 0, 0.0, 0.0
    launches = 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            eng.restore()
            t0 = time.perf_counter()
            edges += eng.run_epochs(ENS_EPOCHS, use_graph=True)
            wall += time.perf_counter() - t0
            st = eng.stats()
            dev_ms += st["ms_total"]
            launches += st["run_kernel_launches"]
    barrier(dist)
    dev_ms_max = reduce_max(dist, dev_ms)
    wall_max = reduce_max(dist, wall)
    evals = reduce_sum(dist, float(len(reps) * args.steps))
    edges_all = reduce_sum(dist, float(edges))
    # the other way of running an epoch (one persistent kernel, or the stage-kernel sequence),
    # timed the same way for comparison
    other = dict(tuned)
    other["epoch_kernel"] = 1 - int(tuned.get("epoch_kernel", 0))
    eng.set_tuning(**other)
    step()  # captures its graph
    other_ms = 0.0
    for _ in range(args.steps):
        eng.restore()
        eng.run_epochs(ENS_EPOCHS, use_graph=True)
        other_ms += eng.stats()["ms_total"]
    other_ms = reduce_max(dist, other_ms) / args.steps
    eng.set_tuning(**tuned)
    eng.close()
    per_step = {"tuned": dev_ms_max / args.steps,
                ("epoch_kernel" if other["epoch_kernel"] else "launch_sequence"): other_ms}

    # serial: the plain per-replica method, one context and one 10-epoch graph run per replica
    ser_dev_ms, ser_wall = 0.0, 0.0
    ser_steps = max(1, min(args.steps, 2))
    engines = []
    for i, ri in zip(idx, reps):
        e1 = GrowthEngine(seed=args.seed, device=local, replica_base=i)
        e1.load_replicas([ri])
        e1.checkpoint()
        e1.run_epochs(ENS_EPOCHS, use_graph=True)  # warm: capture the graph
        engines.append(e1)
    barrier(dist)
    for _ in range(ser_steps):
        for e1 in engines:
            e1.restore()
            t0 = time.perf_counter()
            e1.run_epochs(ENS_EPOCHS, use_graph=True)
            ser_wall += time.perf_counter() - t0
            ser_dev_ms += e1.stats()["ms_total"]
    for e1 in engines:
        e1.close()
    barrier(dist)
    ser_wall = reduce_max(dist, ser_wall) / ser_steps
    ser_dev_ms = reduce_max(dist, ser_dev_ms) / ser_steps

    # end to end: host inputs -> load -> 10 epochs -> every new citation back on the host
    e2e = None
    if not args.no_e2e:
        import dataclasses

        import torch

        # page-locked host buffers, filled before the timed region (as in the PA line): the
        # replicas' raw inputs in, every new citation (source, target) out
        def pinned(a):
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

        preps = [dataclasses.replace(r, pub_epoch=pinned(r.pub_epoch), fitness=pinned(r.fitness),
                                     src=pinned(r.src), dst=pinned(r.dst)) for r in reps]
        tot = int(sum(new_edges)) + 1
        out_s = torch.empty(tot, dtype=torch.int32).pin_memory().numpy()
        out_d = torch.empty(tot, dtype=torch.int32).pin_memory().numpy()
        h2d = d2h = 0
        # timed as the PA line: from the load call to every citation on the host (the context's
        # creation and release are outside)
        with GrowthEngine(seed=args.seed, replicas=len(reps), device=local) as e2:
            e2.set_tuning(**tuned)
            t0 = time.perf_counter()
            e2.load_replicas(preps)
            m0 = [e2.counts(r) for r in range(len(reps))]
            # every epoch's citations, replica by replica, written into the page-locked buffers
            # while the following epochs run (a single run: launched directly, as in the PA line --
            # capturing and instantiating a graph costs more than it saves once)
            ne, _ = e2.run_epochs_out(ENS_EPOCHS, (out_s, out_d), use_graph=False)
            t1 = time.perf_counter()
            for r in range(len(reps)):
                n0_, mm0 = m0[r]
                n1, m1 = e2.counts(r)
                h2d += 4 * n0_ * 2 + 4 * len(reps[r].src) * 2  # publication epochs, fitness, raw edges
                d2h += 8 * (m1 - mm0)  # sources and targets
        dt = reduce_max(dist, t1 - t0)
        e2e = {"value": reduce_sum(dist, float(len(reps))) / dt, "unit": "evals/s",
               "h2d_bytes_per_step": int(reduce_sum(dist, float(h2d))),
               "d2h_bytes_per_step": int(reduce_sum(dist, float(d2h))),
               "citations_per_s": reduce_sum(dist, float(ne)) / dt}
    if rank != 0:
        return None
    value = evals / (dev_ms_max / 1000.0)
    line = {
        "metric": "ensemble evals/sec (replica grown 10 epochs)",
        "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32/u64/f32", "data": "synthetic",
        "config": {"workload": ENS_WORKLOAD, "replicas": ENS_REPLICAS, "epochs": ENS_EPOCHS,
                   "mean_out_degree": 20, "growth": 0.03, "tuning": tuned,
                   "autotune_best_ms": tune_ms, "device_ms_per_step": per_step,
                   "parallelism": "replicas only",
                   "l2": "inputs larger than L2 (all replicas' CSRs, several GB)"},
        "citations_per_s": edges_all / (dev_ms_max / 1000.0),
        "wall_evals_per_s": evals / wall_max,
        "serial": {"device_ms_per_step": ser_dev_ms, "wall_ms_per_step": 1000.0 * ser_wall,
                   "evals_per_s_device": len(idx) * world / (ser_dev_ms / 1000.0),
                   "speedup_device": (ser_dev_ms / 1000.0) / (dev_ms_max / 1000.0 / args.steps),
                   "speedup_wall": ser_wall / (wall_max / args.steps)},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if with_cpu:
        line["cpu_baseline"] = ensemble_cpu_sample(reps_all, args.seed)
    return line


def ensemble_cpu_sample(reps, seed: int, budget_s: float = 12.0) -> dict:
    """The CPU oracle (OpenMP, neighbourhood enumeration) growing replicas of the ensemble for
    all 10 epochs, in order, until the time budget is spent."""
    import oracle as O

    threads = os.cpu_count() or 1
    secs, done = 0.0, 0
    for r, ri in enumerate(reps):
        og = O.OracleGraph(seed, r)
        og.load(ri.pub_epoch, ri.fitness, ri.src, ri.dst)
        og.set_params(**ri.params.__dict__)
        og.set_sampler(1)
        t0 = time.perf_counter()
        for _ in range(ENS_EPOCHS):
            og.pa_epoch(threads)
        secs += time.perf_counter() - t0
        og.close()
        done += 1
        if secs > budget_s:
            break
    return {"value": done / secs, "unit": "evals/s", "cores": threads, "kind": "port",
            "sample": f"first {done} replicas of the ensemble, 10 epochs each ({secs:.1f} s), CPU "
                      f"oracle with OpenMP, neighbourhood enumeration"}


LIK_EPOCHS, LIK_POINTS = 10, 64
LIK_WORKLOAD = "calibration_200k_seed_10_epochs_64_points"


def lik_bytes(st: dict, trace, points: int) -> int:
    """Algorithmic bytes of one forward + adjoint pass over `points` parameter points: per pass the
    per-epoch feature sweep (16 B per node and epoch), one 16-B feature gather per ball element,
    4 B per adjacency entry read to build the balls, 20 B per citation (id + feature), and per
    agent and point the normaliser (written by the forward, read by the adjoint) and the outputs."""
    sweep = 16 * int(sum(int(x) for x in trace.epoch_nodes[:-1]))
    per_pass = sweep + 16 * st["lik_ball_elems"] + 4 * st["lik_adj_entries"] + 20 * st["lik_citations"]
    return 2 * per_pass + 8 * trace.agents * points * (2 + 1 + 4)


def run_loglik(args) -> None:
    line = loglik_measure(args, *dist_setup(), with_cpu=not args.no_cpu)
    if line is not None:
        print(json.dumps(line), flush=True)


def loglik_measure(args, world, rank, local, dist, with_cpu: bool = True) -> dict | None:
    """Differentiable calibration: a PA trace grown on the GPU from a 200,000-node seed over 10
    epochs at theta* = (1, 5, 1, 4) (Poisson(20), 3 % growth, 3 anchors); one step evaluates the
    log-likelihood (forward) and its gradient (adjoint) at 64 parameter points drawn from
    alpha~U[0.5,1.5], tau~U[2,10], gamma~U[0.5,2], beta~U[1,8] in one batch.  The serial method
    calls the same pair once per point.  Under torchrun the points are split across ranks.  Returns
    rank 0's line."""
    from paragraph_gb300 import GrowthEngine
    from paragraph_gb300 import workloads as W

    g = W.plain_pa_seed(args.lik_seed_nodes, 10, seed=args.seed)
    trace = W.grow_trace(g, W.calibration_params(), LIK_EPOCHS, seed=args.seed, device=local)
    pts_all = W.theta_batch(LIK_POINTS, seed=args.seed)
    pts = np.ascontiguousarray(pts_all[rank::world])
    eng = GrowthEngine(seed=args.seed, device=local)
    eng.load_trace(trace)

    def step():
        ll = eng.loglik(pts)
        gr = eng.loglik_grad(pts)
        return ll, gr

    for _ in range(args.warmup):
        step()
    barrier(dist)
    ms_f = ms_b = 0.0
    with ClockSampler(local) as clocks:
        eng.timer_start()
        for _ in range(args.steps):
            ll, gr = step()
            st = eng.stats()
            ms_f += st["lik_ms_fwd"]
            ms_b += st["lik_ms_bwd"]
        ms = eng.timer_stop()
    barrier(dist)
    ms_max = reduce_max(dist, ms)
    evals = reduce_sum(dist, float(len(pts) * args.steps))
    st = eng.stats()
    # serial: the same forward/adjoint pair once per point
    eng.timer_start()
    for p in pts:
        eng.loglik(p[None])
        eng.loglik_grad(p[None])
    ser_ms = reduce_max(dist, eng.timer_stop())
    # the exact arithmetic (fp32 exp2 to ~2 ulp, ball weights and products summed one by one): the
    # same batch and the same serial loop
    eng.set_lik_exact_exp2(True)
    for _ in range(max(1, args.warmup)):
        step()
    eng.timer_start()
    for _ in range(args.steps):
        step()
    ms_x = reduce_max(dist, eng.timer_stop())
    eng.timer_start()
    for p in pts:
        eng.loglik(p[None])
        eng.loglik_grad(p[None])
    ser_x = reduce_max(dist, eng.timer_stop())
    eng.set_lik_exact_exp2(False)
    # end to end: host trace -> device, forward + adjoint, results on the host (wall clock)
    e2e = None
    if not args.no_e2e:
        # from the trace load to the gradients on the host (the context's creation and release
        # are outside, as in the PA line)
        with GrowthEngine(seed=args.seed, device=local) as e2:
            t0 = time.perf_counter()
            e2.load_trace(trace)
            e2.loglik(pts)
            e2.loglik_grad(pts)
            dt = reduce_max(dist, time.perf_counter() - t0)
        h2d = (trace.pub.nbytes + trace.fitness.nbytes + trace.seed_src.nbytes * 2 +
               trace.anchors.nbytes + trace.cite_off.nbytes + trace.cites.nbytes + pts.nbytes * 2)
        e2e = {"value": reduce_sum(dist, float(len(pts))) / dt, "unit": "gradient evals/s",
               "h2d_bytes_per_step": int(reduce_sum(dist, float(h2d))),
               "d2h_bytes_per_step": int(reduce_sum(dist, float(8 * 5 * len(pts))))}
    if rank != 0:
        eng.close()
        return None
    peak, peak_kind = peaks()
    nbytes = lik_bytes(st, trace, len(pts))
    achieved = nbytes / ((ms_f + ms_b) / args.steps / 1000.0) / 1e9
    line = {
        "metric": "gradient evals/sec (log-likelihood + adjoint per parameter point)",
        "value": evals / (ms_max / 1000.0), "unit": "gradient evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 weights / f64 normalisers", "data": "synthetic",
        "config": {"workload": LIK_WORKLOAD, "seed_nodes": g.n, "trace_nodes": trace.num_nodes,
                   "agents": trace.agents, "citations": int(trace.cite_off[-1]),
                   "epochs": LIK_EPOCHS, "points": LIK_POINTS, "theta_star": [1.0, 5.0, 1.0, 4.0],
                   "parallelism": "replicas only (points split across ranks)",
                   "l2": "per-epoch feature sweep and ball gathers over the trace (43 MB of features); "
                         "every step re-reads them"},
        "ball_elements": st["lik_ball_elems"], "adjacency_entries": st["lik_adj_entries"],
        "weight_evals_per_s": 2 * st["lik_ball_elems"] * len(pts) * args.steps / ((ms_f + ms_b) / 1000.0),
        "ms_forward": ms_f / args.steps, "ms_adjoint": ms_b / args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_lik_global + k_lik_agents (forward + adjoint)",
                     "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "note": "at 64 points the passes are bound by the per-point exp of every ball "
                             "element, not by HBM"},
        "serial": {"ms_per_step": ser_ms, "speedup": ser_ms / (ms_max / args.steps)},
        "exact_arithmetic": {"value": evals / (ms_x / 1000.0), "unit": "gradient evals/s",
                             "ms_per_step": ms_x / args.steps, "serial_ms_per_step": ser_x,
                             "speedup": ser_x / (ms_x / args.steps),
                             "note": "pg_lik_set_exact_exp2(1): gradient within 1e-6 of the FP64 "
                                     "oracle at the generating point as well"},
        "e2e": e2e,
        "gpu_launches": 8 * args.steps,
        "clocks": clocks.summary(),
    }
    if with_cpu:
        line["cpu_baseline"] = loglik_cpu_sample(trace, pts_all, ll, gr)
    eng.close()
    return line


def loglik_cpu_sample(trace, pts, ll_gpu, gr_gpu, budget_points: int = 2) -> dict:
    """The FP64 CPU oracle (OpenMP, all host threads) on the first points of the batch, and the
    GPU's relative errors against it at those points."""
    import oracle as O

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    llo, gro = O.loglik(trace, pts[:budget_points], grad=True, threads=threads)
    secs = time.perf_counter() - t0
    rel_ll = float(np.max(np.abs(ll_gpu[:budget_points] - llo) / np.abs(llo)))
    rel_g = float(np.max(np.linalg.norm(gr_gpu[:budget_points] - gro, axis=1) /
                         np.linalg.norm(gro, axis=1)))
    return {"value": budget_points / secs, "unit": "gradient evals/s", "cores": threads,
            "kind": "port",
            "sample": f"{budget_points} points of the batch, FP64 oracle log-likelihood + gradient "
                      f"({secs:.1f} s)",
            "loglik_rel_err_vs_fp64": rel_ll, "grad_rel_err_vs_fp64": rel_g}


def run_small_configs(args) -> None:
    """The two small configurations as separate lines (not the headline): plain PA growth (10k
    seed, 3 epochs of 5,000, Poisson(15), 3 anchors) and ER G(n,p) growth (100k seed without edges,
    10 epochs of 10,000 at p in {1e-5, 1e-4, 1e-3}).  Each step regrows all epochs from the
    device-resident seed; the CPU oracle times the same work on all host threads."""
    import oracle as O
    from paragraph_gb300 import GrowthEngine, PAParams
    from paragraph_gb300 import workloads as W

    peak, peak_kind = peaks()
    threads = os.cpu_count() or 1
    # plain PA
    g = W.plain_pa_seed(10_000, 10, seed=args.seed)
    prm = W.plain_pa_params()
    with GrowthEngine(seed=args.seed) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=3)
        eng.checkpoint()
        for _ in range(args.warmup):
            eng.restore()
            eng.run_epochs(3, use_graph=True)
        eng.sync()
        edges = 0
        eng.timer_start()
        for _ in range(args.steps):
            eng.restore()
            edges += eng.run_epochs(3, use_graph=True)
        ms = eng.timer_stop()
        st = eng.stats()
    og = O.OracleGraph(args.seed, 0)
    og.load(g.pub, g.fitness, g.src, g.dst)
    og.set_params(**prm.__dict__)
    og.set_sampler(1)
    t0 = time.perf_counter()
    cpu_edges = 0
    for _ in range(3):
        m0 = og.m
        og.pa_epoch(threads)
        cpu_edges += og.m - m0
    cpu_s = time.perf_counter() - t0
    og.close()
    gbs = st["run_bytes_alg"] / (ms / args.steps / 1000.0) / 1e9 if ms > 0 else 0.0
    print(json.dumps({
        "metric": "citation edges/sec (plain PA growth)", "value": edges / (ms / 1000.0),
        "unit": "citations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "dtype": "int32/u64/f32",
        "data": "synthetic", "config": {"workload": "plain_pa_10k_seed_3x5000", "seed_nodes": 10_000,
                                        "epochs": 3, "agents_per_epoch": 5000, "mean_out_degree": 15},
        "epoch_bytes_roofline": {"achieved": gbs, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                                 "frac": gbs / peak if peak else None,
                                 "note": "whole-epoch algorithmic bytes / epoch time; launch-bound at this size"},
        "cpu_baseline": {"value": cpu_edges / cpu_s, "unit": "citations/s", "cores": threads, "kind": "port",
                         "sample": "the 3 epochs, CPU oracle, neighbourhood enumeration"}}), flush=True)
    # ER
    g = W.er_seed(100_000)
    for p in (1e-5, 1e-4, 1e-3):
        with GrowthEngine(seed=args.seed) as eng:
            def er_step(timed: bool):
                # reload the seed (untimed), then the 10 epochs between device events
                eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(fixed_new_nodes=10_000),
                               planned_epochs=1)
                # room for the 10 epochs' expected edges (1.45e10 p in all) with an 8-sigma margin
                n0, m0 = eng.counts()
                mu = [10_000 * (n0 + 10_000 * t) * p for t in range(10)]
                eng.reserve(n0 + 100_000, m0 + sum(int(np.ceil(x + 8 * x ** 0.5 + 1024)) + 1 for x in mu))
                eng.sync()
                eng.timer_start()
                e = eng.run_er_epochs(10, 10_000, p)  # the 10 epochs without host synchronisation
                return e, eng.timer_stop()

            for _ in range(args.warmup):
                er_step(False)
            edges, ms = 0, 0.0
            for _ in range(args.steps):
                e, t = er_step(True)
                edges += e
                ms += t
        og = O.OracleGraph(args.seed, 0)
        og.load(g.pub, g.fitness, g.src, g.dst)
        t0 = time.perf_counter()
        m0 = og.m
        for _ in range(10):
            og.er_epoch(10_000, p, threads)
        cpu_s = time.perf_counter() - t0
        cpu_edges = og.m - m0
        og.close()
        print(json.dumps({
            "metric": "citation edges/sec (ER G(n,p) growth)", "value": edges / (ms / 1000.0),
            "unit": "citations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "dtype": "int32/f32 skips (f64 near integers)",
            "data": "synthetic", "config": {"workload": "er_100k_seed_10x10000", "p": p},
            "timing": "10 epochs enqueued without host synchronisation (pg_run_er_epochs), device events around the step",
            "cpu_baseline": {"value": cpu_edges / cpu_s, "unit": "citations/s", "cores": threads,
                             "kind": "port", "sample": "the 10 epochs, CPU oracle"}}), flush=True)


def run_refcompat(args) -> None:
    """The reference's own per-paper model (refcompat weights: preferential, recency and fitness
    scores, 1-hop/2-hop split, same-year and uniform citations) on a 200k-paper seed, 10 epochs at
    3 % growth with 10 % same-year citations, regrown from a device checkpoint each step; the CPU
    oracle of the same model (all host threads) on the same 10 epochs beside it."""
    import oracle as O
    from paragraph_gb300 import PG_WEIGHTS_REFCOMPAT, GrowthEngine, PAParams, RCParams
    from paragraph_gb300 import workloads as W

    threads = os.cpu_count() or 1
    g = W.rc_seed(200_000, 10, seed=args.seed)
    bag, rec = W.rc_tables(seed=args.seed)
    rc = RCParams(growth_rate=0.03, same_year=0.1)
    epochs = 10
    with GrowthEngine(seed=args.seed, weight_model=PG_WEIGHTS_REFCOMPAT) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, PAParams(growth_rate=0.03), planned_epochs=epochs)
        eng.rc_configure(rc, bag, rec)
        # the bag, not the PA plan, bounds the out-degrees: room for every epoch before the
        # checkpoint (an arena regrown mid-run drops it)
        n0, m0 = eng.counts()
        n1 = n0
        for _ in range(epochs):
            n1 += int(np.ceil(n1 * 0.03))
        eng.reserve(n1, m0 + (n1 - n0) * int(min(max(bag), 256)))
        eng.checkpoint()

        def step():
            eng.restore()
            eng.sync()
            eng.timer_start()
            ne = eng.run_epochs(epochs, use_graph=True)
            return ne, eng.timer_stop()

        for _ in range(args.warmup):
            step()
        edges, ms = 0, 0.0
        for _ in range(args.steps):
            e, t = step()
            edges += e
            ms += t
        launches = eng.stats()["run_kernel_launches"]
    cpu = None
    if not args.no_cpu:
        og = O.OracleGraph(args.seed, 0)
        og.load(g.pub, g.fitness, g.src, g.dst)
        og.rc_configure(rc, bag, rec)
        t0 = time.perf_counter()
        m0 = og.m
        for _ in range(epochs):
            og.rc_epoch(threads)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": (og.m - m0) / cpu_s, "unit": "citations/s", "cores": threads, "kind": "port",
               "sample": "the 10 epochs, CPU oracle of the refcompat model (all threads)"}
        og.close()
    print(json.dumps({
        "metric": "citation edges/sec (refcompat growth step)", "value": edges / (ms / 1000.0),
        "unit": "citations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32/u128 scores/f64", "data": "synthetic",
        "config": {"workload": "refcompat_200k_seed_10_epochs_3pct", "same_year": 0.1,
                   "parallelism": "replicas only"},
        "gpu_launches": launches, "cpu_baseline": cpu}), flush=True)


def epoch_report(args) -> None:
    """One JSON line per epoch of the workload: stage times (CUDA events) and byte-model counters.
    Stops early when an epoch exceeds --epoch-cap-s (the enumeration sampler slows down as hubs
    grow)."""
    from paragraph_gb300 import GrowthEngine

    g, prm = seed_graph(args.seed)
    with GrowthEngine(seed=args.seed, sampler=args.sampler) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=EPOCHS)
        for e in range(args.report_epochs):
            t0 = time.perf_counter()
            nn, ne = eng.grow_epoch()
            wall = time.perf_counter() - t0
            s = eng.stats()
            keep = ("new_edges", "rows_expanded", "elems_streamed", "draws", "bwd_moved",
                    "bytes_alg", "bytes_alg_agents", "ms_total", "ms_weights", "ms_setup",
                    "ms_agents", "ms_csr")
            rec = {"epoch": e, "sampler": args.sampler, "nodes": eng.counts()[0], "new_nodes": nn}
            rec.update({k: (round(s[k], 4) if isinstance(s[k], float) else s[k]) for k in keep})
            print(json.dumps(rec), flush=True)
            if wall > args.epoch_cap_s:
                break


def profile_case(args) -> None:
    """Small bounded case for ncu: load the workload's seed and run two PA epochs; with
    --profile-stages also one ER epoch (100k seed, 10,000 new nodes, p = 1e-3) and one refcompat
    epoch (200k seed), so every stage kernel launches at least once."""
    from paragraph_gb300 import PG_WEIGHTS_REFCOMPAT, GrowthEngine, PAParams, RCParams
    from paragraph_gb300 import workloads as W

    g, prm = seed_graph(args.seed)
    with GrowthEngine(seed=args.seed, sampler=args.sampler) as eng:
        eng.load_graph(g.pub, g.fitness, g.src, g.dst, prm, planned_epochs=2)
        for e in range(2):
            eng.grow_epoch()
            s = eng.stats()
            print(json.dumps({"epoch": e, "bytes_alg_agents": s["bytes_alg_agents"],
                              "bytes_alg": s["bytes_alg"], "ms_agents": s["ms_agents"],
                              "ms_csr": s["ms_csr"], "ms_weights": s["ms_weights"],
                              "new_edges": s["new_edges"], "bwd_moved": s["bwd_moved"],
                              "nodes": s["nodes_weighted"]}), flush=True)
    if not args.profile_stages:
        return
    ge = W.er_seed(100_000)
    with GrowthEngine(seed=args.seed) as eng:
        eng.load_graph(ge.pub, ge.fitness, ge.src, ge.dst, PAParams(fixed_new_nodes=10_000), planned_epochs=1)
        ne = eng.er_epoch(10_000, 1e-3)
        s = eng.stats()
        print(json.dumps({"er_edges": ne, "ms_er": s["ms_er"], "bytes_alg": s["bytes_alg"]}), flush=True)
    gr = W.rc_seed(200_000, 10, seed=args.seed)
    bag, rec = W.rc_tables(seed=args.seed)
    with GrowthEngine(seed=args.seed, weight_model=PG_WEIGHTS_REFCOMPAT) as eng:
        eng.load_graph(gr.pub, gr.fitness, gr.src, gr.dst, PAParams(growth_rate=0.03), planned_epochs=1)
        eng.rc_configure(RCParams(growth_rate=0.03, same_year=0.1), bag, rec)
        nn, ne = eng.grow_epoch()
        s = eng.stats()
        print(json.dumps({"rc_new_nodes": nn, "rc_edges": ne, "ms_agents": s["ms_agents"],
                          "ms_weights": s["ms_weights"], "elems": s["elems_streamed"]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-extra", action="store_true",
                    help="default line without the nested ensemble and calibration measurements")
    ap.add_argument("--sampler", type=int, default=0, help="0 thinning, 1 neighbourhood enumeration")
    ap.add_argument("--small-hash", type=int, default=None, help="shape of the k <= 64 agent kernel (0, 1)")
    ap.add_argument("--autotune", action="store_true", help="run the engine's autotuner before the warm-up")
    ap.add_argument("--epoch-report", action="store_true", help="per-epoch stage report instead")
    ap.add_argument("--report-epochs", type=int, default=EPOCHS)
    ap.add_argument("--epoch-cap-s", type=float, default=10.0)
    ap.add_argument("--profile-case", action="store_true", help="two epochs for ncu, then exit")
    ap.add_argument("--profile-stages", action="store_true",
                    help="with --profile-case: also one ER and one refcompat epoch")
    ap.add_argument("--ensemble", action="store_true",
                    help="batched ensemble (256 replicas x 10 epochs) against the serial loop")
    ap.add_argument("--loglik", action="store_true",
                    help="log-likelihood + adjoint at 64 points against the per-point loop")
    ap.add_argument("--lik-seed-nodes", type=int, default=200_000,
                    help="seed size of the calibration trace (smaller cases for profiling)")
    ap.add_argument("--small-configs", action="store_true",
                    help="plain PA (10k seed) and ER G(n,p) lines with their CPU baselines")
    ap.add_argument("--refcompat", action="store_true",
                    help="the reference's own per-paper model (refcompat) with its CPU baseline")
    args = ap.parse_args()
    if args.refcompat:
        if args.warmup < 3:
            args.warmup = 3
        return run_refcompat(args)
    if args.small_configs:
        if args.warmup < 3:
            args.warmup = 3
        return run_small_configs(args)
    if args.ensemble or args.loglik:
        if args.warmup < 3:
            args.warmup = 3
        return run_ensemble(args) if args.ensemble else run_loglik(args)
    if args.epoch_report:
        return epoch_report(args)
    if args.profile_case:
        return profile_case(args)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
