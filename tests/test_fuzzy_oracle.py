"""SIMILARITY / EDIT_DISTANCE: the WHERE builder's bytecode (qe_compile_condition's fuzzy branch,
src/query_exec/query_exec.c:307-349) and the oracle's restatement of the kernel functions
(scan_filter.comp:236-323) on worked examples (CPU only)."""
import numpy as np
import pytest

import oracle
from tests.where_shapes import string_arrays


@pytest.fixture(scope="module")
def ops():
    from computeql_gb300 import build, ops as o
    build.build()
    return o


def _scores(values, word):
    data, offs = string_arrays(values)
    # (<= (edit_distance s word) 1000) / (>= (similarity s word) 0): every row, its score
    out = {}
    for op, code in (("edit", 16), ("sim", 15)):
        pool = word.encode() + b"\0" * ((-len(word)) % 4)
        words = [code, 0, 0, len(word), 2, 0, 7 if code == 16 else 8, 13]
        consts = list(np.array([1000.0 if code == 16 else 0.0]).view(np.uint32))
        mask, sc = oracle.eval_program(words, consts, pool, [data, offs], [5, 0], len(values), scores=True)
        assert mask.all()
        out[op] = sc
    return out


def test_edit_distance_known_values():
    s = _scores(["kitten", "sitting", "", "kitten", "mitten"], "sitting")
    assert list(s["edit"]) == [3.0, 0.0, 7.0, 3.0, 3.0]


def test_trigram_similarity_known_values():
    s = _scores(["abcd", "abce", "xyz", "ab", "abcd"], "abcd")
    # grams abc bcd against abc bcd: 2 shared of 2; abc bce: 1 of 3; none: 0 of 3 (xyz has one gram); a row
    # shorter than a gram matches only itself exactly
    assert list(s["sim"]) == [1.0, float(np.float32(1 / 3)), 0.0, 0.0, 1.0]


def test_builder_emits_the_fuzzy_opcodes(ops):
    cols = {"s": ops.Column(ops.TYPE_STRING8, 2), "n": ops.Column(ops.TYPE_U32, 2, zone=(1.0, 2.0))}
    p = ops.Program("(and (> (similarity s 'needle') 0.4) (< n 5))", cols)
    w = p.words
    assert w[:4] == [15, 0, 0, 6] and p.prog.has_score_output == 1
    q = ops.Program("(<= (edit_distance s 'word') 2)", cols)
    assert q.words[0] == 16 and q.prog.has_score_output == 2
    long = ops.Program("(<= (edit_distance s '" + "x" * 100 + "') 2)", cols)
    assert long.words[3] == 64   # the needle cut to 64 bytes
    with pytest.raises(ops.OpError):
        ops.Program("(> (similarity n 'x') 0.5)", cols)
