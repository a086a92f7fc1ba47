"""The oracle's row gather (selection_gather.comp:64-78 with the encodings decoded): CPU only."""
import numpy as np

import oracle


def test_plain_columns_keep_their_values_in_selection_order():
    src = np.array([10.5, -1.0, 7.25, 3.0])
    rows = np.array([3, 0, 3, 2], dtype=np.uint32)
    np.testing.assert_array_equal(oracle.gather_column(src, rows), [3.0, 10.5, 3.0, 7.25])


def test_narrow_codes_decode_as_base_plus_code_in_32_bits():
    codes = np.array([0, 1, 200, 65535], dtype=np.int64)
    base = (-30000) & 0xFFFFFFFF
    got = oracle.gather_column(codes, np.array([0, 2, 3]), 2, base)
    assert got.dtype == np.uint32
    np.testing.assert_array_equal(got.view(np.int32), [-30000, -29800, 35535])


def test_sequence_is_base_plus_row_wrapping_at_32_bits():
    got = oracle.gather_column(None, np.array([0, 1, 294967296]), 3, 4_000_000_000)
    np.testing.assert_array_equal(got, [4_000_000_000, 4_000_000_001, 0])


def test_strings_in_selection_order():
    assert oracle.gather_strings([b"a", b"", b"ccc"], np.array([2, 1, 2])) == [b"ccc", b"", b"ccc"]
