"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/mdr_oracle.cpp into oracle/libmdr_oracle.so
  (works on x86_64 and aarch64 hosts; plain g++).
* ``build_ref()`` compiles the reference's own MDR headers, read in place from
  the reference tree, with the shims in oracle/ref_harness/shim into
  oracle/_ref/libprodm_ref.so. It only runs where the reference tree exists;
  elsewhere the prebuilt library (if any) is used as is.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libmdr_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libprodm_ref.so")
REFERENCE_TREE = "/root/reference"
ZSTD_LIB = "/lib/x86_64-linux-gnu/libzstd.so.1"


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "mdr_oracle.cpp"), os.path.join(HERE, "mdr_oracle.hpp")]
    if force or _stale(ORACLE_SO, srcs):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_SO, srcs[0]]
        subprocess.check_call(cmd)
    return ORACLE_SO


def build_ref(force=False):
    """Compile the reference harness if the reference tree is present."""
    inc = os.path.join(REFERENCE_TREE, "include")
    if not os.path.isdir(inc):
        return REF_SO if os.path.exists(REF_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_harness", "ref_harness.cpp")
    deps = [src, os.path.join(HERE, "mdr_oracle.hpp")]
    if force or _stale(REF_SO, deps):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
               "-I", os.path.join(HERE, "ref_harness", "shim"), "-I", inc,
               "-o", REF_SO, src]
        if os.path.exists(ZSTD_LIB):
            cmd.append(ZSTD_LIB)
        subprocess.check_call(cmd)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
