"""Synthetic tables of the benchmark configurations, generated on the device from splitmix64.

Draw k of the stream seeded s is splitmix64's k-th output (src/tests/bench_common.h:30-37); a
table's columns are drawn in row order, one draw per drawn column per row, in the listed order.

  fact (10M or 1B rows), seed 0:  id = row number (a sequence, never drawn),
                                  region = draw % 50, amount = draw % 10000, flag = draw % 100
  dim50 (50 rows), seed 1:        k = 0..49, name_id = draw % 10, val = draw (32 bits)
  dim1M (1M rows), seed 2:        k = 0..999999, seg = draw % 20
"""
from __future__ import annotations

from dataclasses import dataclass

FACT_SEED, DIM50_SEED, DIM1M_SEED = 0, 1, 2

# (name, draw index within the row, range) of the drawn fact columns
FACT_DRAWN = [("region", 0, 50), ("amount", 1, 10000), ("flag", 2, 100)]
DIM50_DRAWN = [("name_id", 0, 10), ("val", 1, 0)]
DIM1M_DRAWN = [("seg", 0, 20)]


@dataclass
class FactTable:
    rows: int
    id: object
    region: object
    amount: object
    flag: object


def fact_table(rows, seed=FACT_SEED):
    from .ops import Column
    cols = {name: Column.splitmix(rows, seed, len(FACT_DRAWN), idx, rng) for name, idx, rng in FACT_DRAWN}
    return FactTable(rows, Column.sequence(rows, 0), cols["region"], cols["amount"], cols["flag"])


def fact_numpy(rows, seed=FACT_SEED, gen=None):
    """The same table on the host, for the oracle (`gen` is oracle.splitmix_u32)."""
    out = {"id": None}
    for name, idx, rng in FACT_DRAWN:
        out[name] = gen(rows, seed, len(FACT_DRAWN), idx, rng)
    return out


def dim_tables():
    """dim50 (k, name_id, val) and dim1M (k, seg) as host arrays, drawn on the device like the fact table."""
    import numpy as np
    from .ops import Column
    n50, n1m = 50, 1_000_000
    d50 = {name: Column.splitmix(n50, DIM50_SEED, len(DIM50_DRAWN), idx, rng).buffer.read(np.uint32) for name, idx, rng in DIM50_DRAWN}
    d1m = {name: Column.splitmix(n1m, DIM1M_SEED, len(DIM1M_DRAWN), idx, rng).buffer.read(np.uint32) for name, idx, rng in DIM1M_DRAWN}
    d50["k"] = np.arange(n50, dtype=np.uint32)
    d1m["k"] = np.arange(n1m, dtype=np.uint32)
    return d50, d1m
