"""TEST INFRASTRUCTURE ONLY: build recipes for the CPU oracle.

Two libraries:

* ``oracle/_build/liboracle.so`` - the C restatement in ``oracle/bf_oracle.c``.
  Built on any host (x86 here, aarch64 on the GPU machine).
* ``oracle/_ref/libvsref.so`` - the reference's own CPU code, compiled directly
  from its sources (src/brute_force.cpp, src/hnsw.cpp; headers under include/)
  together with ``oracle/ref_shim.cpp``. Built only where the reference tree is
  present; it uses the reference's own default flags (``-O3 -march=native``,
  CMakeLists.txt:43-51), so on x86 it runs the AVX2 branch of distance.h.
  The reference's cmake build is not used.

Usage: ``python oracle/build_ref.py [--ref /path/to/vecsearch]``. Without ``--ref`` the
reference tree is taken from the environment variable ``VSG_REFERENCE_SRC``, else from the
recipe's default location.
"""
import argparse
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DEFAULT = os.environ.get("VSG_REFERENCE_SRC", "/root/reference")


def reference_present(ref=REF_DEFAULT):
    """True where the reference's CPU sources can be compiled (or were compiled already)."""
    return os.path.exists(os.path.join(ref, "src")) or os.path.exists(os.path.join(HERE, "_ref", "libvsref.so"))


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    """Compile the C restatement; returns the .so path."""
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(HERE, "bf_oracle.c")
    out = os.path.join(out_dir, "liboracle.so")
    if force or _stale(out, [src]):
        flags = ["-O3", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall"]
        if platform.machine() in ("x86_64", "AMD64"):
            flags.append("-mfma")  # hardware fmaf; results are identical either way
        _run(["gcc", *flags, src, "-o", out + ".tmp", "-lm", "-lpthread"])
        os.replace(out + ".tmp", out)
    return out


def build_reference(ref=REF_DEFAULT, force=False):
    """Compile the reference's CPU sources with the shim; returns the .so path or None."""
    srcs = [os.path.join(ref, "src", "brute_force.cpp"), os.path.join(ref, "src", "hnsw.cpp")]
    if not all(os.path.exists(s) for s in srcs):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.cpp")
    out = os.path.join(out_dir, "libvsref.so")
    if force or _stale(out, srcs + [shim]):
        _run(["g++", "-O3", "-march=native", "-std=c++17", "-fPIC", "-shared",
              "-I", os.path.join(ref, "include"), *srcs, shim, "-o", out + ".tmp", "-lpthread"])
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=REF_DEFAULT)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build_oracle(a.force))
    print(build_reference(a.ref, a.force))
