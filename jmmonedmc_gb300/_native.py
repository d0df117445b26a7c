"""Loader for libjmmgpu.so, the in-tree CUDA library behind include/jmm_gpu.h.

There is no fallback: if the library is missing or cannot be loaded the
import of any compute path raises, naming the build command.
"""
import ctypes as C
import os
import threading

from . import abi

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libjmmgpu.so")
_lock = threading.Lock()
_lib = None


class JmmError(RuntimeError):
    """A non-zero status from libjmmgpu.so, with the library's message."""

    def __init__(self, code, func, message):
        self.code = code
        name = abi.ERROR_NAMES.get(code, f"status {code}")
        super().__init__(f"{func}: {name}: {message}")


def lib_path():
    return _LIB_PATH


P = C.POINTER
u64, i32, u32, dbl, vp = C.c_uint64, C.c_int32, C.c_uint32, C.c_double, C.c_void_p

# name -> argtypes; every entry point returns int status unless listed in _RESTYPES
SIGNATURES = {
    "jmm_plain_create": [P(abi.Params), P(vp)],
    "jmm_plain_set_config": [vp, P(dbl), u64, dbl, u64],
    "jmm_plain_fad": [vp, u64, dbl],
    "jmm_plain_steps": [vp, u64, vp, vp],
    "jmm_plain_move": [vp, i32, u64, dbl, vp],
    "jmm_plain_update_thermo": [vp],
    "jmm_plain_reset_thermo": [vp],
    "jmm_plain_echeck": [vp, P(dbl), P(i32)],
    "jmm_plain_set_step_sizes": [vp, dbl, dbl],
    "jmm_plain_get_state": [vp, P(abi.State)],
    "jmm_plain_get_positions": [vp, P(dbl), u64],
    "jmm_plain_get_separations": [vp, P(dbl), u64],
    "jmm_plain_destroy": [vp],
    "jmm_last_error": [],
    "jmm_device_available": [],
    "jmm_measure_peaks": [P(dbl), P(dbl)],
}
_RESTYPES = {"jmm_last_error": C.c_char_p}


def register(signatures, restypes=None):
    """Add entry points declared by later modules (batch, gradients)."""
    SIGNATURES.update(signatures)
    if restypes:
        _RESTYPES.update(restypes)
    if _lib is not None:
        _bind(_lib)


def _bind(lib):
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = argtypes
        fn.restype = _RESTYPES.get(name, C.c_int)


def load():
    """The loaded library; raises if it was not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                raise ImportError(
                    f"{_LIB_PATH} is missing: build it with "
                    "`python -c \"import __graft_entry__ as g; g.build()\"` "
                    "(there is no CPU fallback)")
            lib = C.CDLL(_LIB_PATH)
            _bind(lib)
            _lib = lib
        return _lib


def call(name, *args):
    """Call an entry point and raise JmmError on a non-zero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != abi.JMM_OK:
        msg = lib.jmm_last_error()
        raise JmmError(rc, name, msg.decode() if msg else "")
    return rc


def device_available():
    return bool(load().jmm_device_available())
