"""The C++ drop-in headers (include/openfpm_dcpse/Dcpse.hpp, DCPSE_op.hpp) on
the GPU: compiles tests/cpp/test_dcpse_api.cpp against the built library and
the oracle and runs it (reference test scenarios + bit-exact checks)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(out):
    from openfpm_numerics_gb300 import build as b
    import oracle

    lib = b.build()
    orc = oracle.build()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wno-unused-variable", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_dcpse_api.cpp"), "-L" + os.path.dirname(lib), "-ldcpse_gb300",
           "-L" + os.path.dirname(orc), "-lorc",
           "-Wl,-rpath," + os.path.dirname(lib) + ":" + os.path.dirname(orc), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_cpp_headers_compile(tmp_path):
    """CPU: the headers and the test program compile and link."""
    _compile(str(tmp_path / "t"))


@pytest.mark.gpu
def test_cpp_api_on_gpu(cuda, tmp_path):
    exe = str(tmp_path / "test_dcpse_api")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, cwd=str(tmp_path), timeout=600)
    print(r.stdout)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout[-3000:] + r.stderr[-2000:]
