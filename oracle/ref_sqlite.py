"""The reference's vendored SQLite (src/third_party/sqlite/sqlite3.c, SQLite 3.53.4), built from the
reference's own source tree into oracle/_ref/ and driven through ctypes: an independent SQL engine that the
reference's own benchmarks check their answers against (src/tests/bench_common.h:590-670, loading in
src/tests/scale/bench_query_xlarge.c:287-340). Test infrastructure only: the tests use it to pin the
oracle's restatement of the reference's operators to answers of a SQL engine over the same rows.

The recipe compiles the amalgamation where it lies (nothing is copied into this repository) and writes only
oracle/_ref/libsqlite3.so. Where the reference's tree is absent (the GPU machine), nothing is built and the
tests that need it are skipped.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("CQL_REFERENCE_ROOT", "/root/reference")
SOURCE = os.path.join(REF_ROOT, "src", "third_party", "sqlite", "sqlite3.c")
LIB = os.path.join(HERE, "_ref", "libsqlite3.so")

SQLITE_OK, SQLITE_ROW, SQLITE_DONE = 0, 100, 101
SQLITE_INTEGER, SQLITE_FLOAT, SQLITE_TEXT, SQLITE_NULL = 1, 2, 3, 5


def available():
    return os.path.exists(SOURCE) or os.path.exists(LIB)


def build():
    """Compiles the amalgamation into oracle/_ref/libsqlite3.so (about 12 s); None when the source is absent."""
    if not os.path.exists(SOURCE):
        return LIB if os.path.exists(LIB) else None
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SOURCE):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O1", "-fPIC", "-shared", "-DSQLITE_THREADSAFE=0", "-DSQLITE_OMIT_LOAD_EXTENSION", "-o", LIB, SOURCE, "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("sqlite build failed:\n" + r.stdout[-4000:])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        if not path:
            raise FileNotFoundError("the reference's SQLite source is not present")
        L = C.CDLL(path)
        P, i, i64, dbl, s = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_char_p
        L.sqlite3_open.argtypes = [s, C.POINTER(P)]
        L.sqlite3_close.argtypes = [P]
        L.sqlite3_exec.argtypes = [P, s, P, P, C.POINTER(C.c_char_p)]
        L.sqlite3_errmsg.argtypes = [P]
        L.sqlite3_errmsg.restype = s
        L.sqlite3_prepare_v2.argtypes = [P, s, i, C.POINTER(P), P]
        L.sqlite3_step.argtypes = [P]
        L.sqlite3_finalize.argtypes = [P]
        L.sqlite3_column_count.argtypes = [P]
        L.sqlite3_column_type.argtypes = [P, i]
        L.sqlite3_column_int64.argtypes = [P, i]
        L.sqlite3_column_int64.restype = i64
        L.sqlite3_column_double.argtypes = [P, i]
        L.sqlite3_column_double.restype = dbl
        L.sqlite3_column_text.argtypes = [P, i]
        L.sqlite3_column_text.restype = s
        L.sqlite3_libversion.restype = s
        _lib = L
    return _lib


class Database:
    """An in-memory database of the reference's SQLite."""

    def __init__(self):
        self.db = C.c_void_p()
        if lib().sqlite3_open(b":memory:", C.byref(self.db)) != SQLITE_OK:
            raise RuntimeError("sqlite3_open failed")

    def execute(self, sql):
        if lib().sqlite3_exec(self.db, sql.encode(), None, None, None) != SQLITE_OK:
            raise RuntimeError(lib().sqlite3_errmsg(self.db).decode() + " in: " + sql[:200])

    def load(self, table, columns, rows_per_insert=4000):
        """CREATE TABLE `table` with the numpy arrays of `columns` (name -> array, integers or doubles) and
        insert their rows in order (rowid = row number + 1)."""
        import numpy as np
        names = list(columns)
        kinds = ["REAL" if np.asarray(columns[n]).dtype.kind == "f" else "INTEGER" for n in names]
        self.execute(f"CREATE TABLE {table} (" + ", ".join(f"{n} {k}" for n, k in zip(names, kinds)) + ")")
        n = len(columns[names[0]])
        self.execute("BEGIN")
        cols = [np.asarray(columns[c]) for c in names]
        for first in range(0, n, rows_per_insert):
            parts = []
            for c, k in zip(cols, kinds):
                chunk = c[first: first + rows_per_insert]
                parts.append([repr(float(x)) for x in chunk] if k == "REAL" else [str(int(x)) for x in chunk])
            values = ",".join("(" + ",".join(p[r] for p in parts) + ")" for r in range(len(parts[0])))
            self.execute(f"INSERT INTO {table} VALUES {values}")
        self.execute("COMMIT")

    def query(self, sql):
        """The result rows as tuples of int, float, str or None."""
        L = lib()
        st = C.c_void_p()
        if L.sqlite3_prepare_v2(self.db, sql.encode(), -1, C.byref(st), None) != SQLITE_OK:
            raise RuntimeError(L.sqlite3_errmsg(self.db).decode() + " in: " + sql[:200])
        out = []
        try:
            ncol = L.sqlite3_column_count(st)
            while True:
                rc = L.sqlite3_step(st)
                if rc == SQLITE_DONE:
                    break
                if rc != SQLITE_ROW:
                    raise RuntimeError(L.sqlite3_errmsg(self.db).decode())
                row = []
                for c in range(ncol):
                    t = L.sqlite3_column_type(st, c)
                    row.append(L.sqlite3_column_int64(st, c) if t == SQLITE_INTEGER else L.sqlite3_column_double(st, c) if t == SQLITE_FLOAT
                               else None if t == SQLITE_NULL else L.sqlite3_column_text(st, c).decode())
                out.append(tuple(row))
        finally:
            L.sqlite3_finalize(st)
        return out

    def close(self):
        if self.db:
            lib().sqlite3_close(self.db)
            self.db = C.c_void_p()
