"""Row materialization (cqlops_gather_rows / cqlops_gather_strings) against the oracle's gather.

The reference's selection_gather.comp (modes 0/1) writes dest[i] = source[row i]; the oracle restates that
with the column encodings decoded as the scans read them. Every column type, narrow and sequence
encodings, dictionary and raw strings, host and device selections (unsorted, repeated rows), more columns
than one launch takes, and the refusals.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops():
    from computeql_gb300 import build, native, ops as o
    build.build()
    native.init()
    return o


def _table(ops, n, seed):
    rng = np.random.default_rng(seed)
    data = {
        "u32": rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32),
        "i32": rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32),
        "f32": rng.standard_normal(n).astype(np.float32),
        "u64": rng.integers(0, 2**63, n, dtype=np.uint64),
        "i64": rng.integers(-2**62, 2**62, n, dtype=np.int64),
        "f64": rng.lognormal(3.0, 1.0, n),
        "narrow8": rng.integers(1000, 1200, n).astype(np.uint32),
        "narrow16": rng.integers(-30000, 30000, n).astype(np.int32),
    }
    cols = {k: ops.Column.from_numpy(v, narrow=k.startswith("narrow")) for k, v in data.items()}
    assert cols["narrow8"].width == 1 and cols["narrow16"].width == (2 if n >= 1000 else 1)
    flags = rng.integers(0, 2, n).astype(np.uint8)
    pad = np.concatenate([flags, np.zeros((-n) % 16, dtype=np.uint8)])
    cols["bool"] = ops.Column(6, n, ops.DeviceBuffer(pad.nbytes, pad), zone=None)
    data["bool"] = flags
    cols["seq"] = ops.Column.sequence(n, first=4_000_000_000)
    data["seq"] = None
    return data, cols


def _expect(data, cols, name, rows):
    """The oracle's gather over what the column stores (codes for narrow widths, nothing for a sequence),
    as the 32-bit words (encoded columns) or values the operator returns."""
    c = cols[name]
    if name == "seq":
        return oracle.gather_column(None, rows, 3, c.base)
    if c.width in (1, 2):
        codes = data[name].astype(np.int64) - np.int64(np.uint32(c.base).astype(np.int32))
        return oracle.gather_column(codes, rows, c.width, c.base)
    return oracle.gather_column(data[name], rows)


@pytest.mark.parametrize("n", [1, 1000, 3_000_001])
def test_every_type_host_rows(ops, n):
    data, cols = _table(ops, n, n)
    rng = np.random.default_rng(7)
    rows = rng.integers(0, n, max(1, n // 100)).astype(np.uint32)   # unsorted, with repeats
    names = list(cols)
    got = ops.gather_rows([cols[k] for k in names], rows=rows)
    for k, g in zip(names, got):
        want = _expect(data, cols, k, rows)
        if k in ("narrow8", "narrow16", "seq"):
            g = g.view(np.uint32)
        assert g.dtype == want.dtype, k
        np.testing.assert_array_equal(g, want, err_msg=k)


def test_device_selection_and_all_rows(ops):
    n = 200_000
    data, cols = _table(ops, n, 3)
    rows = np.nonzero(data["u32"] % 37 == 5)[0].astype(np.uint32)
    sel = ops.DeviceBuffer(rows.nbytes, rows)
    got = ops.gather_rows([cols["f64"], cols["narrow16"], cols["seq"]], selection=sel)
    np.testing.assert_array_equal(got[0], data["f64"][rows])
    np.testing.assert_array_equal(got[1].view(np.int32), data["narrow16"][rows])
    np.testing.assert_array_equal(got[2], (4_000_000_000 + rows.astype(np.int64)) & 0xFFFFFFFF)
    every = ops.gather_rows([cols["i64"], cols["bool"]], count=n)
    np.testing.assert_array_equal(every[0], data["i64"])
    np.testing.assert_array_equal(every[1], data["bool"])


def test_thirty_columns_one_percent(ops):
    """More columns than one launch gathers (13): three launches into one destination."""
    n = 500_000
    rng = np.random.default_rng(11)
    arrays = [rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32) if i % 2 == 0 else rng.random(n) for i in range(30)]
    cols = [ops.Column.from_numpy(a) for a in arrays]
    rows = np.sort(rng.choice(n, n // 100, replace=False)).astype(np.uint32)
    got = ops.gather_rows(cols, rows=rows)
    for a, g in zip(arrays, got):
        np.testing.assert_array_equal(g, oracle.gather_column(a, rows))


def test_dictionary_and_raw_strings(ops):
    rng = np.random.default_rng(5)
    words = ["", "a", "north", "south-east", "x" * 300, "éclair", "zz"]
    values = [words[i] for i in rng.integers(0, len(words), 50_000)]
    dcol = ops.StringColumn(values, dictionary=True)
    rcol = ops.StringColumn(values)
    rows = rng.integers(0, len(values), 4000).astype(np.uint32)
    codes = ops.gather_rows([dcol], rows=rows)[0]
    np.testing.assert_array_equal(codes, dcol.codes[rows])
    got = ops.gather_strings(rcol, rows=rows)
    assert got == oracle.gather_strings(rcol.values, rows)
    sel = ops.DeviceBuffer(rows.nbytes, rows)
    assert ops.gather_strings(rcol, selection=sel) == got
    assert ops.gather_strings(rcol, rows=np.zeros(0, dtype=np.uint32)) == []


def test_refusals(ops):
    n = 1000
    data, cols = _table(ops, n, 9)
    with pytest.raises(ops.OpError):
        ops.gather_rows([cols["u32"]], rows=np.array([0, n], dtype=np.uint32))
    rcol = ops.StringColumn(["a", "bb"])
    with pytest.raises(ops.OpError):
        ops.gather_rows([rcol], rows=np.array([0], dtype=np.uint32))
    assert [g.size for g in ops.gather_rows([cols["u32"]], rows=np.zeros(0, dtype=np.uint32))] == [0]
