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


def test_python_bindings_cover_the_headers():
    from computeql_gb300 import native
    bound = {n for n, _, _ in native.CUDA_API} | {n for n, _, _ in native.OPS_API}
    want = set(declared("cqlcuda.h", "cqlcuda")) | set(declared("cqlops.h", "cqlops"))
    assert want <= bound, sorted(want - bound)


def test_libraries_load_without_a_gpu(libs):
    from computeql_gb300 import native
    native.load_ops()  # dlopen only; cqlcuda_init is not called here

