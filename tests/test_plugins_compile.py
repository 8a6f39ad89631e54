"""The C++ plugin adapters instantiate inside the reference's own
ComposedRefactor / ComposedReconstructor templates (compile-time drop-in
check; needs the reference headers, so it runs only where they exist)."""
import os
import shutil
import subprocess

import pytest

import importlib

build_oracle = importlib.import_module("oracle.build_oracle")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_INC = os.path.join(build_oracle.reference_tree(), "include")


@pytest.mark.skipif(not os.path.isdir(REF_INC), reason="reference headers not present")
def test_adapters_instantiate_in_reference_composed_classes():
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-DPRODM_WITH_REFERENCE_CONCEPTS",
           "-I", os.path.join(ROOT, "include"), "-I", REF_INC,
           "-I", os.path.join(ROOT, "oracle", "ref_harness", "shim"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "cpp", "reference_dropin.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
