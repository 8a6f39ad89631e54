"""Builds the C++ plugin checks against the in-tree library and runs them:
* tests/cpp/plugin_parity.cpp: the C++ plugin adapters
  (include/prodm_gb300_mdr.hpp) driven as the reference's ComposedRefactor /
  ComposedReconstructor drive their plugins;
* tests/cpp/reference_dropin.cpp (where the reference's headers are present:
  the reference tree, or the copy the oracle recipe stages under oracle/_ref):
  the reference's own ComposedRefactor / ComposedReconstructor driving the
  adapters, with level files and metadata byte-identical to the reference's
  CPU components and reconstructions meeting every tolerance."""
import os
import subprocess
import tempfile

import pytest

import importlib

build_oracle = importlib.import_module("oracle.build_oracle")

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


def reference_include():
    inc = os.path.join(build_oracle.reference_tree(), "include")
    if os.path.isdir(os.path.join(inc, "MDR")):
        return inc
    return build_oracle.STAGED if os.path.isdir(os.path.join(build_oracle.STAGED, "MDR")) else None


@pytest.mark.skipif(reference_include() is None, reason="reference headers not present")
def test_reference_composed_classes_drive_gpu_adapters():
    from prodm_gb300 import build
    lib = build.build()
    cuda = "/usr/local/cuda"
    z = build_oracle.zstd_library() or build_oracle.ZSTD_STUB
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "reference_dropin")
        cmd = ["g++", "-std=c++17", "-O2", "-w", "-DPRODM_WITH_REFERENCE_CONCEPTS",
               "-I", os.path.join(ROOT, "include"), "-I", reference_include(),
               "-I", os.path.join(ROOT, "oracle", "ref_harness", "shim"), "-I", cuda + "/include",
               os.path.join(ROOT, "tests", "cpp", "reference_dropin.cpp"), z, lib,
               "-L", cuda + "/lib64", "-L", cuda + "/lib", "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
               "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600)
        print(r.stdout)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "REFERENCE DROP-IN OK" in r.stdout
