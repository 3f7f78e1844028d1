"""Compile the CUDA extension in-tree: vecsearch_gb300/_lib/libvsg_gb300.so (sm_103a only).

Each translation unit under csrc/ is compiled in parallel with nvcc, then linked
into one shared library with the static CUDA runtime, so the library depends on
nothing but the driver. Then the pybind11 front end (csrc/pybind_module.cpp, the
reference's GpuBruteForceIndex surface) is compiled with g++ against it, where
pybind11's headers are installed (the pybind11 package or PyTorch's copy).
``python -m vecsearch_gb300.build [--verbose]``.
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


def pybind_include():
    """pybind11's headers: the pybind11 package, else the copy PyTorch ships (found without
    importing torch); None if neither is installed."""
    import importlib.util
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        pass
    spec = importlib.util.find_spec("torch")
    for loc in (spec.submodule_search_locations or []) if spec else []:
        inc = os.path.join(loc, "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    return None


def pybind_module_path():
    import sysconfig
    return os.path.join(OUT_DIR, "_vecsearch_gb300" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def build_pybind(lib, verbose=False, force=False):
    """The pybind11 front end (csrc/pybind_module.cpp) linked against the library; returns its path,
    or None where pybind11's or Python's headers are missing."""
    import sysconfig
    pyinc = sysconfig.get_paths().get("include")
    pbinc = pybind_include()
    if not pbinc or not pyinc or not os.path.exists(os.path.join(pyinc, "Python.h")):
        return None
    src = os.path.join(CSRC, "pybind_module.cpp")
    out = pybind_module_path()
    if force or _stale(out, [src, lib] + _headers()):
        cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
               "-I", pyinc, "-I", pbinc, src, "-o", out + ".tmp", "-L", OUT_DIR, "-l:" + LIB_NAME,
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("g++ failed: " + " ".join(cmd))
        os.replace(out + ".tmp", out)
    return out


def build(verbose=False, force=False):
    """Builds (if stale) and returns the path of the shared library (and the pybind11 front end
    where its headers are present)."""
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
    build_pybind(lib, verbose, force)
    return lib


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force="--force" in sys.argv))
