"""The reference-side adapter files compiled against the reference's own headers (CPU only).

computeql_gb300/adapter/gpu_cuda.c (the GPU_Backend vtable over libcqlcuda.so) and
computeql_gb300/adapter/query_kernel_cuda.c (every qk_* function of src/query_exec/query_kernel.h:198-240,
emitting CUDA C++) are meant for the reference's C99 unity build. tests/adapter/harness.c lays the
reference's headers out as src/main.c:9-17 does, includes both files, links libcqlops/libcqlcuda and
runs checks that need no GPU: the vtable's size and slots, and NVRTC compiles of the generated
sources. Skipped where the reference's sources are not present.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("CQL_REFERENCE_SRC", "/root/reference/src")

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "gpu", "gpu_backend.h")),
                                reason="the reference's sources are not present")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from computeql_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("adapter") / "harness")
    pkg = os.path.join(ROOT, "computeql_gb300")
    cmd = ["gcc", "-std=gnu11", "-O0", "-Wall", "-Wno-unused-function", "-Wno-unused-parameter", "-Wno-unused-variable",
           "-Wno-unused-but-set-variable", "-Wno-missing-braces", "-Werror=implicit-function-declaration",
           "-Werror=incompatible-pointer-types", "-Werror=int-conversion",
           "-I", os.path.join(ROOT, "tests", "adapter"), "-I", os.path.join(pkg, "adapter"), "-I", os.path.join(ROOT, "include"),
           "-I", REF_SRC, "-I", os.path.join(REF_SRC, "third_party", "vulkan"),
           os.path.join(ROOT, "tests", "adapter", "harness.c"), "-o", out, "-L", pkg, "-lcqlops", "-lcqlcuda", "-Wl,-rpath," + pkg]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    return out


def test_adapter_compiles_against_the_reference_headers_and_passes(harness):
    r = subprocess.run([harness], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    lines = r.stdout.splitlines()
    assert lines[-1] == "all ok", r.stdout
    assert not [l for l in lines if l.startswith("FAIL") or l.startswith("empty slot")]
    assert "ok every slot filled" in lines
    assert "ok the scan source compiles for sm_103a" in lines
