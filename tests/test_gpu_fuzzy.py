"""Fuzzy search on the GPU: SIMILARITY (trigram) and EDIT_DISTANCE comparisons on the interpreter
(scan_filter), the matching rows and their scores equal to the oracle's, alone and with other
predicates; a count-only scan of a scored program too."""
import numpy as np
import pytest

import oracle
from tests.where_shapes import string_arrays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(gpu):
    from computeql_gb300 import ops
    rng = np.random.default_rng(12)
    alphabet = np.array(list("abcdefghij"))
    n = 200_003
    lens = rng.integers(0, 14, n)
    values = ["".join(alphabet[rng.integers(0, 10, l)]) for l in lens]
    values[17] = "abcabcabc"
    values[18] = "x" * 300
    amount = rng.integers(0, 1000, n).astype(np.uint32)
    cols = {"s": ops.StringColumn(values), "amount": ops.Column.from_numpy(amount)}
    arrays = {"s": string_arrays(values), "amount": amount}
    return ops, cols, arrays


def _oracle(program, arrays):
    p = program.prog
    slots = [None] * 10
    types = [0] * 10
    for b in range(p.binding_count):
        name = program.names[p.binding_column[b]]
        slot = p.binding_slot[b]
        types[slot] = p.binding_type[b]
        a = arrays[name]
        if isinstance(a, tuple):
            slots[slot], slots[slot + 1] = a
        else:
            slots[slot] = a
    return oracle.eval_program(program.words, list(p.consts[: 2 * p.const_count]), bytes(p.str_pool[: p.str_pool_size]), slots, types,
                               program.columns[0].rows, scores=True)


@pytest.mark.parametrize("where", [
    "(> (similarity s 'abcab') 0.2)",
    "(>= (similarity s 'ab') 0.5)",
    "(<= (edit_distance s 'abcde') 2)",
    "(< (edit_distance s 'jjjj') 3)",
    "(and (> (similarity s 'cdefg') 0.1) (< amount 500))",
    "(or (<= (edit_distance s 'abc') 1) (= amount 7))",
])
def test_rows_and_scores_equal_the_oracle(env, where):
    ops, cols, arrays = env
    prog = ops.Program(where, cols)
    count, rows, scores = ops.scan_scored(prog)
    mask, want = _oracle(prog, arrays)
    idx = np.nonzero(mask)[0]
    assert count == len(idx), where
    assert np.array_equal(rows, idx.astype(np.uint32)), where
    assert np.array_equal(scores, want[idx]), where
    c2, _, _ = ops.scan_filter(prog)
    assert c2 == count
