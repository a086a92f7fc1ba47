"""WHERE shapes for the per-query-kernel tests, and the oracle's view of a compiled program.

random_shape restates the shape generator of the reference's per-query kernel benchmark
(pc_random_shape, src/tests/bench_perquery_compile.c:238-258): 1 to 8 comparisons over the
columns, each a lower or upper bound, inclusive or not, joined by OR one time in four, with one
parenthesised pair when there are 4 or more. SQL precedence (AND before OR) turns the chain into
the s-expression the operator layer compiles.
"""
import numpy as np

import oracle


def random_shape(rng, columns, literal):
    n = 1 + int(rng.integers(0, 8))
    leaves, joiner = [], []
    for _ in range(n):
        col = columns[int(rng.integers(0, len(columns)))]
        upper = bool(rng.integers(0, 2))
        inclusive = bool(rng.integers(0, 2))
        op = ("<=" if inclusive else "<") if upper else (">=" if inclusive else ">")
        leaves.append(f"({op} {col} {literal(col, rng)!r})")
        joiner.append(int(rng.integers(0, 4)) == 0)
    group = None
    if n >= 4:
        start = int(rng.integers(0, n - 2))
        group = start
        joiner[start] = not joiner[start + 1]
    # tokens: leaf, op, leaf, ...; a group wraps leaves start and start + 1
    items = []
    i = 0
    while i < n:
        if group is not None and i == group:
            j = "or" if joiner[i] else "and"
            items.append(f"({j} {leaves[i]} {leaves[i + 1]})")
            items.append("or" if joiner[i + 1] else "and")
            i += 2
        else:
            items.append(leaves[i])
            items.append("or" if joiner[i] else "and")
            i += 1
    items = items[:-1]
    # AND binds before OR
    or_terms, cur = [], [items[0]]
    for k in range(1, len(items), 2):
        if items[k] == "and":
            cur.append(items[k + 1])
        else:
            or_terms.append(cur)
            cur = [items[k + 1]]
    or_terms.append(cur)

    def chain(op, xs):
        out = xs[0]
        for x in xs[1:]:
            out = f"({op} {out} {x})"
        return out

    return chain("or", [chain("and", t) for t in or_terms])


def _slots(program, arrays):
    """the oracle's slot arrays and types for a compiled ops.Program, arrays: name -> numpy column (a
    string column as (bytes uint8, offsets uint64))"""
    slots = [None] * 10
    types = [0] * 10
    p = program.prog
    for b in range(p.binding_count):
        name = program.names[p.binding_column[b]]
        slot = p.binding_slot[b]
        types[slot] = p.binding_type[b]
        a = arrays[name]
        if p.binding_dict[b]:
            slots[slot] = program.columns[p.binding_column[b]].codes
        elif isinstance(a, tuple):
            slots[slot], slots[slot + 1] = a
        else:
            slots[slot] = a
    return slots, types


def oracle_mask(program, arrays):
    """The oracle's match mask for a compiled ops.Program over host arrays."""
    slots, types = _slots(program, arrays)
    p = program.prog
    rows = program.columns[0].rows
    return oracle.eval_program(program.words, list(p.consts[: 2 * p.const_count]), bytes(p.str_pool[: p.str_pool_size]), slots, types, rows)


def oracle_batch(programs, sum_names, arrays, rows):
    """The oracle's COUNT(*) and compensated SUM(sum column) of each compiled program over host arrays, all
    programs in one pass over the table (numeric programs only)."""
    batch = []
    for prog, s in zip(programs, sum_names):
        slots, types = _slots(prog, arrays)
        batch.append((prog.words, list(prog.prog.consts[: 2 * prog.prog.const_count]), slots, types, arrays[s] if s else None))
    return oracle.batch_count_sum(batch, rows)


def string_arrays(values):
    raw = [v.encode() for v in values]
    offs = np.zeros(len(raw) + 1, dtype=np.uint64)
    for i, v in enumerate(raw):
        offs[i + 1] = offs[i] + len(v)
    blob = np.frombuffer(b"".join(raw) + b"\0" * 16, dtype=np.uint8).copy()
    return blob, offs
