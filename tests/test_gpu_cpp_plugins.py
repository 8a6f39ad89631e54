"""Builds tests/cpp/plugin_parity.cpp against the in-tree library and runs it:
the C++ plugin adapters (include/prodm_gb300_mdr.hpp) driven as the
reference's ComposedRefactor / ComposedReconstructor drive their plugins."""
import os
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_plugin_adapters_round_trip():
    from prodm_gb300 import build
    lib = build.build()
    cuda = "/usr/local/cuda"
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "plugin_parity")
        cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", cuda + "/include",
               os.path.join(ROOT, "tests", "cpp", "plugin_parity.cpp"), lib,
               "-L", cuda + "/lib64", "-L", cuda + "/lib", "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
               "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "PLUGIN PARITY OK" in r.stdout
