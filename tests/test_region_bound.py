"""The backward region's size bound, checked on the span policy itself.

A cited node's span holds its forward row copy (prefix P = out-degree rounded up to 4) in front of
its backward entries; a span is brow_cap(L + P) = (2 (L + P) + 3) & ~3 entries, and a row moves to a
new span when its length outgrows the room (the span minus P).  The engine sizes each replica's
region at 8 m + 18 n + 4 entries (m edges, n nodes) and never grows it, so every run must stay
under that: per row the spans together take less than 4 (L + P) + 6 entries.  This restates the
policy of pg_engine.cuh (brow_cap, fwd_prefix, brow_span) and replays growth histories against it,
adversarial ones included (one entry at a time, rows that get every citation)."""
import numpy as np


def brow_cap(x):
    return (2 * x + 3) & ~3


def fwd_prefix(o):
    return (o + 3) & ~3


def spans_of_row(o, increments):
    """Entries the row's spans take over a history of per-epoch increments (first citation: a
    span is taken; no span while uncited)."""
    P = fwd_prefix(o)
    length, room, total = 0, 0, 0
    for inc in increments:
        if inc == 0:
            continue
        new = length + inc
        if new > room:
            span = brow_cap(new + P)
            total += span
            room = span - P
            assert room >= new and room % 4 == 0 and span % 4 == 0
        length = new
    return length, P, total


def test_per_row_bound_on_adversarial_histories():
    rng = np.random.default_rng(3)
    for o in (0, 1, 3, 4, 5, 30, 256, 1000):
        for hist in ([1] * 5000, [1, 1, 2, 4, 8, 16, 32, 64, 128, 256, 512], [7] * 700,
                     list(rng.integers(0, 40, 300)), [10_000], [3, 0, 0, 1, 2, 9999]):
            L, P, total = spans_of_row(o, hist)
            if L:
                assert total < 4 * (L + P) + 6 + 1, (o, hist[:5], L, P, total)


def test_region_bound_on_random_graph_growth():
    """Random graphs grown epoch by epoch (preferential targets, so a few rows get most entries):
    the spans of all rows stay under 8 m + 18 n."""
    rng = np.random.default_rng(7)
    for trial in range(6):
        n0, epochs = int(rng.integers(50, 2000)), int(rng.integers(1, 12))
        outdeg = list(rng.integers(0, 60, n0))
        hist = [[] for _ in range(n0)]
        n = n0
        for _ in range(epochs):
            delta = max(1, n // 20)
            ks = rng.integers(0, 60, delta)
            w = np.arange(1, n + 1, dtype=np.float64) ** -1.5  # heavy-tailed target choice
            w /= w.sum()
            inc = np.zeros(n, np.int64)
            for k in ks:
                for t in rng.choice(n, size=min(int(k), n), replace=False, p=w):
                    inc[t] += 1
            for v in range(n):
                hist[v].append(int(inc[v]))
            outdeg += list(ks)
            hist += [[] for _ in range(delta)]
            n += delta
        m = int(sum(outdeg))
        used = 0
        for v in range(n):
            L, P, total = spans_of_row(int(outdeg[v]), hist[v])
            used += total
        assert used <= 8 * m + 18 * n + 4, (trial, used, m, n)
