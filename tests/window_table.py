"""The window-rank test table of the reference (src/tests/bench_query_window_rank.c:136-170): one
bench_rng stream seeded 0x9E3779B97F4A7C15 drawn key by key, row by row; key 0 has 7 values, key 2 has 50,
keys 1 and 3 are wide with fractions (draw % 4e12 / 7) in the "wide" set and 50 values in the "narrow" one;
and its cases (label, keys, partition keys, DESC mask, narrow)."""
import numpy as np

from tests.bench_rng import draws

SEED = 0x9E3779B97F4A7C15

CASES = [
    ("order wide", 1, 0, 0, 0),
    ("order wide desc", 1, 0, 1, 0),
    ("partition 7, order wide", 2, 1, 0, 0),
    ("partition 7, order wide desc", 2, 1, 2, 0),
    ("partition 7, order 50, wide", 3, 1, 4, 0),
    ("partitions 7 and wide, order 50", 3, 2, 0, 0),
    ("four keys", 4, 2, 10, 0),
    ("narrow partition and order", 2, 1, 0, 1),
    ("narrow four keys with ties", 4, 2, 5, 1),
]


def tables(n):
    """(wide, narrow): four f64 key arrays each."""
    r = draws(SEED, 4 * n).reshape(4, n)
    wide, narrow = [], []
    for k in range(4):
        small = (r[k] % np.uint64(7 if k == 0 else 50)).astype(np.float64)
        narrow.append(small)
        wide.append(small if k in (0, 2) else (r[k] % np.uint64(4000000000000)).astype(np.float64) / 7.0)
    return wide, narrow


def verify(keys, desc, partitions, rows, row_number, rank, dense):
    """win_verify (bench_query_window_rank.c:40-104): every row once, keys in order, and the three ranks
    recomputed from that order. Returns the first bad position + 1, or 0."""
    n = len(keys[0])
    seen = np.zeros(n, dtype=bool)
    part_start = peer_start = dense_now = 0
    for i in range(n):
        row = int(rows[i])
        if row >= n or seen[row]:
            return i + 1
        seen[row] = True
        new_part = new_peer = i == 0
        if i > 0:
            prev = int(rows[i - 1])
            for k in range(len(keys)):
                a, b = keys[k][prev], keys[k][row]
                if a == b:
                    continue
                if (a < b) if desc[k] else (a > b):
                    return i + 1
                new_part = k < partitions
                new_peer = True
                break
        if new_part:
            part_start = peer_start = i
            dense_now = 1
        elif new_peer:
            peer_start = i
            dense_now += 1
        if row_number[i] != i - part_start + 1 or rank[i] != peer_start - part_start + 1 or dense[i] != dense_now:
            return i + 1
    return 0
