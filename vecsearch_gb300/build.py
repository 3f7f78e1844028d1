"""Compile the CUDA extension in-tree: vecsearch_gb300/_lib/libvsg_gb300.so (sm_103a only).

Each translation unit under csrc/ is compiled in parallel with nvcc, then linked
into one shared library with the static CUDA runtime, so the library depends on
nothing but the driver. ``python -m vecsearch_gb300.build [--verbose]``.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libvsg_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    inc = os.path.join(os.path.dirname(HERE), "include")
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Builds (if stale) and returns the path of the shared library."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = nvcc_path()
    flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                    "--expt-relaxed-constexpr"]
    if verbose:
        flags += ["-Xptxas", "-v"]
    headers = _headers()
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *flags, "-c", src, "-o", obj])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        failed = [r for r in results if r.returncode != 0]
        for r in results:
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
        if failed:
            raise RuntimeError("nvcc failed:\n" + "\n".join(" ".join(r.args) for r in failed))
    lib = os.path.join(OUT_DIR, LIB_NAME)
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp"
        subprocess.run([nvcc, *ARCH, "-shared", "-cudart", "static", *objs, "-o", tmp, "-lpthread"], check=True)
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force="--force" in sys.argv))
