"""ctypes binding of the C ABI in include/vsg.h (libvsg_gb300.so, built in-tree).

There is no fallback: if the library is missing, importing the GPU classes raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libvsg_gb300.so")

OK, ERR_INVALID, ERR_LENGTH, ERR_CUDA, ERR_DEVICE_TIMEOUT, ERR_NOMEM, ERR_IO = range(7)
METRIC_L2, METRIC_IP = 0, 1
METHODS = {"auto": 0, "naive": 1, "skinny": 2, "tiled": 3, "bf16": 4, "tc_exact": 5, "fp8": 6}
NONE = 0xFFFFFFFF
MAX_K = 128

_lib = None

_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_U32 = ctypes.c_uint32
_INT = ctypes.c_int

# name -> (restype, argtypes); the exported symbols of include/vsg.h.
SIGNATURES = {
    "vsg_cuda_available": (_INT, []),
    "vsg_last_error": (ctypes.c_char_p, []),
    "vsg_create": (_INT, [_SZ, _U32, _INT, ctypes.POINTER(_P)]),
    "vsg_destroy": (None, [_P]),
    "vsg_add": (_INT, [_P, _P, _SZ]),
    "vsg_search": (_INT, [_P, _P, _SZ, _SZ, _P, _P, _U32]),
    "vsg_search_filtered": (_INT, [_P, _P, _SZ, _SZ, _P, _INT, _SZ, _P, _P, _U32]),
    "vsg_hnsw_exact_below": (_INT, [_P, _P, _SZ, _SZ, _P, _SZ, _SZ, _P, _P, ctypes.POINTER(_INT)]),
    "vsg_search_device": (_INT, [_P, _P, _SZ, _SZ, _SZ, _P, _INT, _SZ, _P, _P, _U32, _P]),
    "vsg_sync": (_INT, [_P]),
    "vsg_size": (_SZ, [_P]),
    "vsg_dim": (_SZ, [_P]),
    "vsg_metric": (_U32, [_P]),
    "vsg_device_rows": (_P, [_P, ctypes.POINTER(_SZ)]),
    "vsg_profile_enable": (_INT, [_P, _INT]),
    "vsg_profile_read": (_INT, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(_SZ)]),
    "vsg_set_tunable": (_INT, [_P, ctypes.c_char_p, ctypes.c_double]),
    "vsg_get_tunable": (_INT, [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]),
    "vsg_hnsw_file_info": (_INT, [ctypes.c_char_p, ctypes.POINTER(_SZ), ctypes.POINTER(_SZ), ctypes.POINTER(_U32)]),
    "vsg_add_hnsw_file": (_INT, [_P, ctypes.c_char_p, ctypes.POINTER(_SZ)]),
    "vsg_insert_candidates": (_INT, [_P, _SZ, _SZ, _U32, ctypes.c_int, _SZ, _SZ, _P, _P]),
    "vsg_tc_exact_stats": (_INT, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                  ctypes.POINTER(ctypes.c_uint64)]),
    "vsg_tiled_stats": (_INT, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "vsg_kernel_launches": (_INT, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "vsg_autotune": (_INT, [_P, ctypes.POINTER(_SZ), _SZ, _SZ, _U32]),
    "vsg_autotune_with_queries": (_INT, [_P, ctypes.c_void_p, _SZ, ctypes.POINTER(_SZ), _SZ, _SZ, _U32]),
    "vsg_autotune_table": (_INT, [_P, _U32, ctypes.POINTER(_SZ), ctypes.POINTER(_U32), ctypes.POINTER(_U32),
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_U32)]),
    "vsg_autotune_save": (_INT, [_P, ctypes.c_char_p]),
    "vsg_autotune_load": (_INT, [_P, ctypes.c_char_p]),
    "vsg_server_create": (_INT, [_P, _SZ, _SZ, _SZ, ctypes.POINTER(_P)]),
    "vsg_server_submit": (_INT, [_P, _P, _SZ, _SZ, _P, _P, _P, ctypes.POINTER(ctypes.c_uint64)]),
    "vsg_server_wait": (_INT, [_P, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "vsg_server_stats": (_INT, [_P] + [ctypes.POINTER(ctypes.c_uint64)] * 4),
    "vsg_server_uncertified": (_INT, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "vsg_server_destroy": (None, [_P]),
    "vsg_search_rows_noalloc": (_INT, [_P, _SZ, _SZ, _U32, _P, _SZ, _SZ, _P, _P, _P]),
}


class DeviceTimeoutError(RuntimeError):
    """A kernel's bounded wait ran out; the device context is still usable."""


def lib():
    """The loaded library; raises ImportError if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m vecsearch_gb300.build`")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(rc):
    """Raises the Python exception the reference's pybind11 layer would raise for a status code."""
    if rc == OK:
        return
    msg = lib().vsg_last_error().decode(errors="replace")
    if rc in (ERR_INVALID, ERR_LENGTH):
        raise ValueError(msg)
    if rc == ERR_NOMEM:
        raise MemoryError(msg)
    if rc == ERR_DEVICE_TIMEOUT:
        raise DeviceTimeoutError(msg)
    raise RuntimeError(msg)
