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
    """dim50 (k, name_id, val) and dim1M (k, seg), drawn on the device like the fact table: host arrays under
    the column names, and the device columns (kept resident, as the fact table is) under "<name>_col"."""
    import numpy as np
    from .ops import Column
    n50, n1m = 50, 1_000_000
    d50, d1m = {}, {}
    for table, rows, seed, drawn in ((d50, n50, DIM50_SEED, DIM50_DRAWN), (d1m, n1m, DIM1M_SEED, DIM1M_DRAWN)):
        for name, idx, rng in drawn:
            col = Column.splitmix(rows, seed, len(drawn), idx, rng)
            table[name + "_col"] = col
            table[name] = col.buffer.read(np.uint32)
        table["k_col"] = Column.affine(rows, 1, 0, 0)
        table["k"] = np.arange(rows, dtype=np.uint32)
    return d50, d1m


# ---------------------------------------------------------------------------------------------
# The 10M-row, 30-column event table and its users table (the wide-table configuration), drawn on the
# host from the same splitmix64 streams. Per row, in order: u0..u9 (draw % 2^20), i0..i4 (draw % 2^41 -
# 2^40), m0..m7 (lognormal mu 3 sigma 1 by Box-Muller from two draws, each mapped to (0, 1]), user_id
# (% 1M), region (% 50), status (% 5), s0..s3 (Zipf s = 1.1 over 200 dictionary values, inverse CDF of
# one draw mapped to [0, 1)), session (% 4M): 39 draws a row. users (1M rows, seed 3): user_id = row,
# segment = draw % 20. The dictionary's 200 values are 8-24 lowercase letters drawn from seed + 1000.

EVENT_SEED, USERS_SEED = 0, 3
EVENT_DRAWS = 39
EVENT_U32 = [f"u{i}" for i in range(10)]
EVENT_I64 = [f"i{i}" for i in range(5)]
EVENT_F64 = [f"m{i}" for i in range(8)]
EVENT_DICT = [f"s{i}" for i in range(4)]
DICT_VALUES, ZIPF_S = 200, 1.1

_GOLDEN, _M1, _M2 = 0x9E3779B97F4A7C15, 0xBF58476D1CE4E5B9, 0x94D049BB133111EB


def splitmix_draws(seed, k):
    """splitmix64's draws k (a uint64 array, 0-based) of the stream seeded `seed` (bench_common.h:30-37)."""
    import numpy as np
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (k.astype(np.uint64) + np.uint64(1)) * np.uint64(_GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(_M1)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(_M2)
        return z ^ (z >> np.uint64(31))


def _unit(d, closed_top):
    """the top 53 bits of a draw as a double: in (0, 1] or [0, 1)"""
    import numpy as np
    top = (d >> np.uint64(11)).astype(np.float64)
    return (top + 1.0) * 2.0 ** -53 if closed_top else top * 2.0 ** -53


def event_dictionary(seed=EVENT_SEED):
    """The 200 dictionary strings of the event table's string columns."""
    import numpy as np
    out, k = [], 0
    for _ in range(DICT_VALUES):
        length = 8 + int(splitmix_draws(seed + 1000, np.array([k]))[0] % np.uint64(17))
        k += 1
        letters = splitmix_draws(seed + 1000, np.arange(k, k + length)) % np.uint64(26)
        k += length
        out.append("".join(chr(97 + int(c)) for c in letters))
    return out


def event_numpy(rows, seed=EVENT_SEED):
    """The event table as host arrays (dictionary columns as codes) plus the dictionary."""
    import numpy as np
    base = np.arange(rows, dtype=np.uint64) * np.uint64(EVENT_DRAWS)
    draw = lambda j: splitmix_draws(seed, base + np.uint64(j))
    t = {}
    for i, name in enumerate(EVENT_U32):
        t[name] = (draw(i) % np.uint64(1 << 20)).astype(np.uint32)
    for i, name in enumerate(EVENT_I64):
        t[name] = (draw(10 + i) % np.uint64(1 << 41)).astype(np.int64) - (1 << 40)
    for i, name in enumerate(EVENT_F64):
        u1, u2 = _unit(draw(15 + 2 * i), True), _unit(draw(16 + 2 * i), True)
        t[name] = np.exp(3.0 + np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2))
    t["user_id"] = (draw(31) % np.uint64(1_000_000)).astype(np.uint32)
    t["region"] = (draw(32) % np.uint64(50)).astype(np.uint32)
    t["status"] = (draw(33) % np.uint64(5)).astype(np.uint32)
    weights = 1.0 / np.arange(1, DICT_VALUES + 1, dtype=np.float64) ** ZIPF_S
    cdf = np.cumsum(weights) / weights.sum()
    for i, name in enumerate(EVENT_DICT):
        t[name] = np.minimum(np.searchsorted(cdf, _unit(draw(34 + i), False), side="right"), DICT_VALUES - 1).astype(np.uint32)
    t["session"] = (draw(38) % np.uint64(4_000_000)).astype(np.uint32)
    users = {"user_id": np.arange(1_000_000, dtype=np.uint32),
             "segment": (splitmix_draws(USERS_SEED, np.arange(1_000_000, dtype=np.uint64)) % np.uint64(20)).astype(np.uint32)}
    return t, users, event_dictionary(seed)


def event_table(rows, seed=EVENT_SEED):
    """The event table resident on the device: a dict of columns (dictionary strings as coded string
    columns over the shared dictionary), the users table as host arrays (and its two columns resident under
    "<name>_col"), and the host arrays."""
    from .ops import Column, StringColumn
    h, users, words = event_numpy(rows, seed)
    # the users table is resident too (the join's dim-side pass reads it on the device)
    users["user_id_col"] = Column.from_numpy(users["user_id"])
    users["segment_col"] = Column.from_numpy(users["segment"])
    cols = {}
    for name, arr in h.items():
        if name in EVENT_DICT:
            cols[name] = StringColumn.from_codes(arr, words)
        else:
            cols[name] = Column.from_numpy(arr)
    return cols, users, h, words
