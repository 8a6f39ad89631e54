"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/mdr_oracle.cpp into oracle/libmdr_oracle.so
  (works on x86_64 and aarch64 hosts; plain g++).
* ``build_ref()`` compiles the reference's own MDR headers with the shims in
  oracle/ref_harness/shim into oracle/_ref/libprodm_ref.so. Where the
  reference tree is present (the directory named by PRODM_REFERENCE_TREE,
  default /root/reference), its headers are first staged, unmodified, into the
  git-ignored oracle/_ref/include; a host without the tree (the GPU host)
  builds from that staged copy, so the benchmark's CPU arm runs the compiled
  reference there too. Nothing under oracle/_ref is committed.
"""
import ctypes.util
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libmdr_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libprodm_ref.so")
STAGED = os.path.join(REF_DIR, "include")
ZSTD_STUB = os.path.join(HERE, "ref_harness", "zstd_absent.c")


def reference_tree():
    return os.environ.get("PRODM_REFERENCE_TREE", "/root/reference")


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


def stage_headers():
    """Copy the reference's include tree (MDR/ and qoi_utils.hpp) into
    oracle/_ref/include when the reference tree exists; returns the include
    directory to compile against, or None."""
    inc = os.path.join(reference_tree(), "include")
    if os.path.isdir(inc):
        stamp = os.path.join(STAGED, ".staged")
        newest = max(os.path.getmtime(os.path.join(d, f)) for d, _, fs in os.walk(inc) for f in fs)
        if not os.path.exists(stamp) or os.path.getmtime(stamp) < newest:
            if os.path.isdir(STAGED):
                shutil.rmtree(STAGED)
            shutil.copytree(os.path.join(inc, "MDR"), os.path.join(STAGED, "MDR"))
            shutil.copy2(os.path.join(inc, "qoi_utils.hpp"), os.path.join(STAGED, "qoi_utils.hpp"))
            open(stamp, "w").close()
        return STAGED
    return STAGED if os.path.isdir(os.path.join(STAGED, "MDR")) else None


def zstd_library():
    """Path of the system libzstd (x86_64 or aarch64), or None."""
    for p in ("/lib/x86_64-linux-gnu/libzstd.so.1", "/usr/lib/x86_64-linux-gnu/libzstd.so.1",
              "/lib/aarch64-linux-gnu/libzstd.so.1", "/usr/lib/aarch64-linux-gnu/libzstd.so.1",
              "/usr/lib64/libzstd.so.1"):
        if os.path.exists(p):
            return p
    name = ctypes.util.find_library("zstd")
    for d in ("/lib", "/usr/lib", "/lib64", "/usr/lib64"):
        if name and os.path.exists(os.path.join(d, name)):
            return os.path.join(d, name)
    return None


def build_ref(force=False):
    """Compile the reference harness from the reference tree (staged first)
    or from an earlier staged copy; None when neither exists."""
    inc = stage_headers()
    if inc is None:
        return REF_SO if os.path.exists(REF_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_harness", "ref_harness.cpp")
    deps = [src, os.path.join(HERE, "mdr_oracle.hpp")]
    if force or _stale(REF_SO, deps) or _stale(REF_SO, [os.path.join(inc, "MDR", "Refactor", "ComposedRefactor.hpp")]):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
               "-I", os.path.join(HERE, "ref_harness", "shim"), "-I", inc,
               "-o", REF_SO, src]
        z = zstd_library()
        cmd.append(z if z else ZSTD_STUB)
        subprocess.check_call(cmd)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
