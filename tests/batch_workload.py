"""The batched configuration's workload: a table of 4 u32 and 4 f64 columns (u32 uniform [0, 2^16),
f64 uniform [0, 1)), WHERE shapes drawn like the reference's per-query kernel benchmark
(pc_random_shape, src/tests/bench_perquery_compile.c:238-258, restated in tests/where_shapes.py) and
queries that each take one shape with fresh literals, followed by COUNT(*) and SUM of an f64 column.
"""
import numpy as np

from tests.where_shapes import random_shape

U32 = ["u0", "u1", "u2", "u3"]
F64 = ["d0", "d1", "d2", "d3"]


def table(rows, seed):
    rng = np.random.default_rng(seed)
    cols = {n: rng.integers(0, 1 << 16, rows).astype(np.uint32) for n in U32}
    cols.update({n: rng.random(rows) for n in F64})
    return cols


def literal(col, rng):
    if col.startswith("u"):
        return int(rng.integers(0, 1 << 16))
    return round(float(rng.random()), 6)


def shapes(count, seed):
    """`count` shape generators: each call with an rng returns the shape's condition with new literals."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        state = rng.integers(0, 2**63)

        def make(qrng, state=state):
            srng = np.random.default_rng(int(state))     # the same columns, ops and joiners every time
            return random_shape(srng, U32 + F64, lambda col, r: literal(col, qrng))
        out.append(make)
    return out


def queries(count, shape_count, seed):
    """(condition, summed column) of `count` queries over `shape_count` shapes."""
    gens = shapes(shape_count, seed)
    rng = np.random.default_rng(seed + 1)
    return [(gens[q % shape_count](rng), F64[q % 4]) for q in range(count)]
