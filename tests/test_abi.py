"""The C-ABI libraries build and export every entry point their headers declare (CPU only: no
compute call is made)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"_[a-z0-9_]+)\s*\(", text)))


def exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], stdout=subprocess.PIPE, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


@pytest.fixture(scope="module")
def libs():
    from computeql_gb300 import build
    return build.build()


def test_cqlcuda_exports_every_declared_symbol(libs):
    names = declared("cqlcuda.h", "cqlcuda")
    assert len(names) > 50
    missing = [n for n in names if n not in exported(libs[0])]
    assert not missing, missing


def test_cqlops_exports_every_declared_symbol(libs):
    names = declared("cqlops.h", "cqlops")
    missing = [n for n in names if n not in exported(libs[1])]
    assert not missing, missing


def test_cqlserve_exports_every_declared_symbol(libs):
    names = declared("cqlserve.h", "cqlserve")
    assert len(names) >= 8
    missing = [n for n in names if n not in exported(libs[1])]
    assert not missing, missing


def test_python_bindings_cover_the_headers():
    from computeql_gb300 import native
    bound = {n for n, _, _ in native.CUDA_API} | {n for n, _, _ in native.OPS_API}
    want = set(declared("cqlcuda.h", "cqlcuda")) | set(declared("cqlops.h", "cqlops")) | set(declared("cqlserve.h", "cqlserve"))
    assert want <= bound, sorted(want - bound)


def test_serve_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the operator layer's and the server's structs have the C layout: every field's
    offset and the size."""
    import ctypes as C
    from computeql_gb300 import native
    checks = []
    for name, cls in (("CqlServeConfig", native.CqlServeConfig), ("CqlServeRequest", native.CqlServeRequest),
                      ("CqlServeStats", native.CqlServeStats), ("CqlServeJoin", native.CqlServeJoin),
                      ("CqlServeSort", native.CqlServeSort), ("CqlJoinAgg", native.CqlJoinAgg), ("CqlColumn", native.CqlColumn),
                      ("CqlHostColumn", native.CqlHostColumn), ("CqlLeaf", native.CqlLeaf)):
        checks.append((f"sizeof({name})", C.sizeof(cls)))
        for field, _ in cls._fields_:
            checks.append((f"offsetof({name}, {field})", getattr(cls, field).offset))
    prog = "#include <stddef.h>\n#include <stdio.h>\n#include \"cqlserve.h\"\nint main(void)\n{\n"
    prog += "".join(f'  printf("%zu\\n", (size_t){expr});\n' for expr, _ in checks) + "  return 0;\n}\n"
    src = tmp_path / "layout.c"
    src.write_text(prog)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True, check=True).stdout.split()]
    assert got == [v for _, v in checks], [(e, v, g) for (e, v), g in zip(checks, got) if v != g]


def test_libraries_load_without_a_gpu(libs):
    from computeql_gb300 import native
    native.load_ops()  # dlopen only; cqlcuda_init is not called here

