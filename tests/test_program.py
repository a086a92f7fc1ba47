"""WHERE compilation and per-query kernel sources (CPU only: no device call).

The bytecode is checked word for word against what the reference's compiler emits for the same
condition (qe_compile_condition, src/query_exec/query_exec.c:204-548); every generated source is
compiled with NVRTC for sm_103a here, without a GPU.
"""
import numpy as np
import pytest

from computeql_gb300 import native, ops
from tests.where_shapes import random_shape

PUSH_TRUE, LOAD, CONST, EQ, NE, LT, GT, LE, GE, AND, OR, STR_EQ, CONTAINS, HALT, PUSH_FALSE = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14
STR_NE, STR_LT = 17, 18


@pytest.fixture(scope="module")
def lib():
    from computeql_gb300 import build
    build.build()
    return native.load_ops()


def cols():
    c = {
        "flag": ops.Column(ops.TYPE_U32, 100, zone=(0.0, 99.0)),
        "amount": ops.Column(ops.TYPE_U32, 100, zone=(0.0, 9999.0)),
        "x": ops.Column(ops.TYPE_F64, 100),
        "f": ops.Column(ops.TYPE_F32, 100),
        "i": ops.Column(ops.TYPE_I32, 100),
        "s": ops.Column(ops.TYPE_STRING8, 100),
    }
    return c


def test_comparison_bytecode(lib):
    p = ops.Program("(< flag 2)", cols())
    # LoadNumCol (U32 << 8 | slot 0), PushConst 0, CmpLt, Halt
    assert p.words == [LOAD, (1 << 8) | 0, CONST, 0, LT, HALT]
    assert p.consts == [2.0]


def test_and_or_tree_and_slot_order(lib):
    p = ops.Program("(and (>= amount 10) (or (= flag 3) (< x 2.5)))", cols())
    assert p.words == [LOAD, 256, CONST, 0, GE, LOAD, 257, CONST, 1, EQ, LOAD, (4 << 8) | 2, CONST, 2, LT, OR, AND, HALT]
    assert p.consts == [10.0, 3.0, 2.5]
    assert p.stack_depth() == 4


def test_in_list_is_an_or_chain_and_not_in_an_and_chain(lib):
    p = ops.Program("(in flag 1 2 3)", cols())
    assert p.words == [LOAD, 256, CONST, 0, EQ, LOAD, 256, CONST, 1, EQ, OR, LOAD, 256, CONST, 2, EQ, OR, HALT]
    q = ops.Program("(not_in i -1 5)", cols())
    assert q.words == [LOAD, (7 << 8), CONST, 0, NE, LOAD, (7 << 8), CONST, 1, NE, AND, HALT]


def test_in_list_limits(lib):
    assert ops.Program("(in flag)", cols()).words == [PUSH_FALSE, HALT]
    assert ops.Program("(not_in flag)", cols()).words == [PUSH_TRUE, HALT]
    long_list = "(in flag " + " ".join(str(k) for k in range(33)) + ")"
    with pytest.raises(ops.OpError, match="IN list too long"):
        ops.Program(long_list, cols())


def test_null_tests_and_constants(lib):
    assert ops.Program("(is_not_null x)", cols()).words == [PUSH_TRUE, HALT]
    p = ops.Program("(is_null x)", cols())
    assert p.words == [CONST, 0, HALT] and p.consts == [0.0]
    assert ops.Program("", cols()).words == [PUSH_TRUE, HALT]


def test_string_operations_use_two_slots(lib):
    p = ops.Program("(and (= s 'abc') (< flag 5))", cols())
    # the string column takes slots 0 (bytes) and 1 (offsets), flag slot 2
    assert p.words == [STR_EQ, 0, 0, 3, LOAD, (1 << 8) | 2, CONST, 0, LT, AND, HALT]
    assert bytes(p.prog.str_pool[:3]) == b"abc"
    q = ops.Program("(and (contains s 'bc') (!= s 'zz'))", cols())
    assert q.words[:4] == [CONTAINS, 0, 0, 2] and q.words[4:8] == [STR_NE, 0, 1, 2]


def test_dictionary_equality_uses_codes(lib):
    c = cols()
    sc = ops.StringColumn.__new__(ops.StringColumn)
    # a dictionary-coded column without device data: the compiler only needs the dictionary
    ops.Column.__init__(sc, ops.TYPE_STRING8, 4)
    vals = [b"red", b"green", b"blue"]
    offs = np.array([0, 3, 8, 12], dtype=np.uint32)
    import ctypes as C
    sc._dict_offsets = offs
    sc._dict_bytes = C.create_string_buffer(b"".join(vals), 12)
    sc.dict_struct = native.CqlDict(3, offs.ctypes.data, C.addressof(sc._dict_bytes))
    sc.offsets_buf = None
    c["color"] = sc
    p = ops.Program("(= color 'blue')", c)
    assert p.words == [LOAD, (1 << 8) | 0, CONST, 0, EQ, HALT] and p.consts == [2.0]
    assert ops.Program("(= color 'pink')", c).words == [PUSH_FALSE, HALT]
    assert ops.Program("(!= color 'pink')", c).words == [PUSH_TRUE, HALT]


def test_simple_leaves_only_for_numeric_and_trees(lib):
    import ctypes as C
    buf = (native.CqlLeaf * 8)()
    p = ops.Program("(and (< flag 2) (and (>= amount 5) (> x 0.5)))", cols())
    assert native.load_ops().cqlops_program_simple_leaves(C.byref(p.prog), buf, 8) == 3
    q = ops.Program("(or (< flag 2) (>= amount 5))", cols())
    assert native.load_ops().cqlops_program_simple_leaves(C.byref(q.prog), buf, 8) == 0


@pytest.mark.parametrize("seed", range(12))
def test_generated_sources_compile_for_sm103a(lib, seed):
    rng = np.random.default_rng(seed)
    names = ["flag", "amount", "x", "f", "i"]
    where = random_shape(rng, names, lambda c, r: round(float(r.random()) * 100, 3))
    p = ops.Program(where, cols())
    ok, log = ops.compile_check(p.source(ops.KERNEL_SCAN))
    assert ok, log


def test_fused_sources_compile(lib):
    import ctypes as C
    c = cols()
    p = ops.Program("(or (< flag 2) (> x 0.25))", c)
    s_amount = native.load_ops().cqlops_program_bind(C.byref(p.prog), p._cols, p.index("amount"))
    s_i = native.load_ops().cqlops_program_bind(C.byref(p.prog), p._cols, p.index("i"))
    f = native.CqlFusedAgg()
    f.column_count = 3
    f.slots[0], f.coltypes[0] = s_amount, ops.TYPE_U32
    f.slots[1], f.coltypes[1] = s_i, ops.TYPE_I32
    f.slots[2], f.coltypes[2] = 1, ops.TYPE_F64  # x, bound second by the filter
    ok, log = ops.compile_check(p.source(ops.KERNEL_FUSED_AGG, f))
    assert ok, log
    g = native.CqlFusedAgg()
    g.grouped, g.key_count, g.column_count = 1, 2, 1
    g.key_slots[0], g.key_types[0], g.key_ranges[0] = 0, ops.TYPE_U32, 100
    g.key_slots[1], g.key_types[1], g.key_ranges[1] = s_i, ops.TYPE_I32, 10
    g.group_count = 1000
    g.slots[0], g.coltypes[0] = s_amount, ops.TYPE_U32
    ok, log = ops.compile_check(p.source(ops.KERNEL_FUSED_GROUP, g))
    assert ok, log


def test_deep_or_chain_compiles(lib):
    # depth 12: deeper than the interpreter's 8-slot stack, fine for a generated kernel
    where = "(< flag 0)"
    for k in range(1, 12):
        where = f"(or (= flag {k}) {where})"
    p = ops.Program(where, cols())
    assert p.stack_depth() >= 3
    ok, log = ops.compile_check(p.source())
    assert ok, log
