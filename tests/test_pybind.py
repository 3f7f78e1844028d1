"""CPU: the pybind11 front end (_vecsearch_gb300) has the reference's GPU class surface.

The reference's module (python/bindings.cpp:151-197) exposes GpuBruteForceIndex(dim, metric="l2",
device=0) with add, search, dim and len, and cuda_available(), which is False without a GPU
(the contract its CI checks on machines without CUDA, .github/workflows/ci.yml:51-66). Argument
errors raise ValueError before any CUDA call; a missing GPU raises RuntimeError.
"""
import inspect

import pytest

import vecsearch_gb300 as vsg


@pytest.fixture(scope="module")
def mod():
    from vecsearch_gb300 import build
    build.build()
    m = vsg.pybind_module()
    if m is None:
        pytest.skip("pybind11 headers not installed here")
    return m


def test_class_surface(mod):
    cls = mod.GpuBruteForceIndex
    for name in ("add", "search", "__len__"):
        assert callable(getattr(cls, name))
    assert isinstance(inspect.getattr_static(cls, "dim"), property)
    doc = cls.search.__doc__  # argument names and defaults as bindings.cpp:160-186 declares them
    assert "queries:" in doc and "k:" in doc and "= 10" in doc and "method: str = 'auto'" in doc
    assert "filter: object = None" in doc
    init = cls.__init__.__doc__
    assert "dim:" in init and "metric: str = 'l2'" in init and "device:" in init and "= 0" in init


def test_cuda_available_matches_the_ctypes_front_end(mod):
    assert mod.cuda_available() == vsg.cuda_available()


def test_argument_errors_come_first(mod):
    with pytest.raises(ValueError):
        mod.GpuBruteForceIndex(0)
    with pytest.raises(ValueError, match="metric must be"):
        mod.GpuBruteForceIndex(8, "hamming")
    with pytest.raises(TypeError):
        mod.GpuBruteForceIndex(-1)


def test_no_gpu_raises_runtime_error(mod):
    if mod.cuda_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        mod.GpuBruteForceIndex(8)
