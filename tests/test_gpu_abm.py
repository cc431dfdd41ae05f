"""The `abm` driver end to end on the GPU: reference-format input files in, reference-format edge
list and attribute file out, checked against the CPU oracle grown from the same inputs.

The `abm` program draws the seed papers' fitness itself and writes it to the attribute file
(fit_peak_value), so the oracle is seeded from that column; ids are mapped as the reference maps
them (sequence ids in ascending original id, new papers max id + 1, + 2, ...)."""
import subprocess

import numpy as np
import pytest

import oracle as O
from paragraph_gb300 import RCParams
from paragraph_gb300 import workloads as W
from paragraph_gb300.build import DRIVER

pytestmark = pytest.mark.gpu


def _inputs(tmp, g, delim=","):
    ids = 1000 + 3 * np.arange(g.n)           # original ids, ascending with the sequence id
    years = 2000 + g.pub.astype(np.int64)      # calendar years; the run starts at max + 1
    with open(tmp / "nodes.csv", "w") as f:
        f.write(f"#node{delim}year\n")
        for i, y in zip(ids, years):
            f.write(f"{i}{delim}{y}\n")
    with open(tmp / "edges.csv", "w") as f:
        f.write(f"#source{delim}target\n")
        for s, d in zip(g.src, g.dst):
            f.write(f"{ids[s]}{delim}{ids[d]}\n")
        f.write(f"{ids[5]}{delim}{ids[2]}\n")  # a duplicate collapses
        f.write(f"{ids[5]}{delim}999999\n")    # an unknown endpoint is dropped
    return ids, years


def _tables(tmp, bag, rec):
    with open(tmp / "bag.csv", "w") as f:
        f.write("#index,out_degree\n")
        for i, v in enumerate(bag):
            f.write(f"{i},{v}\n")
    with open(tmp / "rec.csv", "w") as f:
        f.write("#year_diff,probability\n")
        for a, p in enumerate(rec):
            f.write(f"{a},{float(p)!r}\n")


def _run(tmp, *extra):
    cmd = [str(DRIVER), "--edgelist", str(tmp / "edges.csv"), "--nodelist", str(tmp / "nodes.csv"),
           "--output-file", str(tmp / "out.csv"), "--auxiliary-information-file", str(tmp / "aux.csv"),
           "--log-file", str(tmp / "log.txt"), *map(str, extra)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def _edges(tmp, ids_all):
    lines = (tmp / "out.csv").read_text().splitlines()
    assert lines[0] == "#source,target"
    e = np.array([l.split(",") for l in lines[1:]], dtype=np.int64).reshape(-1, 2)
    seq = {int(x): i for i, x in enumerate(ids_all)}
    return np.array([seq[s] for s in e[:, 0]]), np.array([seq[d] for d in e[:, 1]])


def _aux(tmp):
    lines = (tmp / "aux.csv").read_text().splitlines()
    assert lines[0].split(",")[0] == "node_id" and len(lines[0].split(",")) == 15
    return [l.split(",") for l in lines[1:]]


def _compare(og, tmp, ids):
    n = og.n
    ids_all = np.concatenate([ids, ids[-1] + 1 + np.arange(n - len(ids))])
    s, d = _edges(tmp, ids_all)
    off, col = og.csr(0)
    np.testing.assert_array_equal(s, np.repeat(np.arange(n), np.diff(off)))
    np.testing.assert_array_equal(d, col)
    aux = _aux(tmp)
    assert len(aux) == n
    indeg, outdeg = og.degrees()
    np.testing.assert_array_equal([int(r[10]) for r in aux], indeg)
    np.testing.assert_array_equal([int(r[11]) for r in aux], outdeg)
    assert all(r[1] == "seed" for r in aux[:len(ids)]) and all(r[1] == "agent" for r in aux[len(ids):])


def test_abm_refcompat_matches_oracle(gpu, tmp_path):
    g = W.rc_seed(1500, 8, seed=2)
    ids, years = _inputs(tmp_path, g)
    bag, rec = W.rc_tables(seed=3, bag_mean=12.0)
    _tables(tmp_path, bag, rec)
    (tmp_path / "planted.csv").write_text("#year,lag,peak,duration,count\n2,1,900,2,20\n2,0,500,5,10\n")
    _run(tmp_path, "--out-degree-bag", tmp_path / "bag.csv", "--recency-probabilities", tmp_path / "rec.csv",
         "--planted-nodes", tmp_path / "planted.csv", "--growth-rate", 0.05, "--num-cycles", 3,
         "--same-year-proportion", 0.1, "--alpha", 0.5, "--seed", 7, "--output-nodelist",
         tmp_path / "grown_nodes.csv")
    aux = _aux(tmp_path)
    fit = np.array([float(r[7]) for r in aux[:g.n]], np.float32)
    assert np.all(fit >= 1) and np.all(fit <= 1000) and np.all(fit == np.round(fit))
    og = O.OracleGraph(7, 0)
    og.load(years.astype(np.int32), fit, g.src, g.dst)
    og.set_epoch(int(years.max()) + 1)
    og.rc_configure(RCParams(alpha=0.5, same_year=0.1, growth_rate=0.05), bag, rec)
    for cycle in (1, 2, 3):
        n = og.n
        og.rc_epoch()
        if cycle == 2:
            og.rc_set_nodes(og.n - (og.n - n), [1] * 20, [900] * 20, [2] * 20)
            og.rc_set_nodes(og.n - (og.n - n) + 20, [0] * 10, [500] * 10, [5] * 10)
    _compare(og, tmp_path, ids)
    aux = _aux(tmp_path)
    grown = (tmp_path / "grown_nodes.csv").read_text().splitlines()
    assert len(grown) == og.n + 1
    planted_rows = [r for r in aux if r[13] != "-1"]
    assert len(planted_rows) == 30 and {r[7] for r in planted_rows} == {"900", "500"}


def test_abm_baseline_and_tab_separated_inputs(gpu, tmp_path):
    g = W.plain_pa_seed(1200, 6, seed=4)
    ids, years = _inputs(tmp_path, g, delim="\t")
    _run(tmp_path, "--weight-model", "baseline", "--growth-rate", 0.1, "--num-cycles", 2,
         "--same-year-proportion", 0, "--pa-alpha", 1.0, "--tau", 5, "--gamma", 1, "--beta", 4,
         "--num-anchors", 3, "--mean-out-degree", 10, "--seed", 11)
    fit = np.array([float(r[7]) for r in _aux(tmp_path)[:g.n]], np.float32)
    og = O.OracleGraph(11, 0)
    og.load(years.astype(np.int32), fit, g.src, g.dst)
    og.set_params(alpha=1.0, tau=5.0, gamma=1.0, beta=4.0, mean_out_degree=10.0, growth_rate=0.1,
                  fixed_new_nodes=0, num_anchors=3)
    og.set_epoch(int(years.max()) + 1)
    og.pa_epoch()
    og.pa_epoch()
    _compare(og, tmp_path, ids)


def test_abm_er(gpu, tmp_path):
    g = W.plain_pa_seed(3000, 4, seed=5)
    ids, years = _inputs(tmp_path, g)
    _run(tmp_path, "--model", "er-gnp", "--er-probability", 0.002, "--growth-rate", 0.2,
         "--num-cycles", 2, "--seed", 3)
    fit = np.array([float(r[7]) for r in _aux(tmp_path)[:g.n]], np.float32)
    og = O.OracleGraph(3, 0)
    og.load(years.astype(np.int32), fit, g.src, g.dst)
    og.set_epoch(int(years.max()) + 1)
    for _ in range(2):
        og.er_epoch(int(np.ceil(og.n * 0.2)), 0.002)
    _compare(og, tmp_path, ids)
