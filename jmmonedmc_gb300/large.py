"""Python handle on the large-chain sweeps (jmm_large_* in include/jmm_gpu.h).

``LargeChains`` holds constant-L chains of up to 2^24 particles with hard
walls (FP64 positions in HBM, FP32 step arithmetic) and runs them either with
the alternating-domain sweep (``mode="domains"``: domains of ``domain_size``
particles from a random offset, two colours in random order, one warp per
domain) or with the sequential plain sweep (``mode="sequential"``: one warp
per chain, N steps in order).  The reference has no counterpart: its pair
arrays are O(N^2) per chain (src/jmmMCState.cpp:308-328,439-455).
"""
import ctypes as C

import numpy as np

from . import _native, abi

P = C.POINTER
_native.register({
    "jmm_large_create": [P(abi.BatchConfig), P(abi.ChainDesc), C.c_uint32, C.c_uint32,
                         P(C.c_void_p)],
    "jmm_large_run": [C.c_void_p, C.c_uint64, C.c_int32],
    "jmm_large_run_async": [C.c_void_p, C.c_uint64, C.c_int32, C.c_void_p],
    "jmm_large_results": [C.c_void_p, P(abi.LargeResult), C.c_uint32],
    "jmm_large_reset_stats": [C.c_void_p],
    "jmm_large_energies": [C.c_void_p, P(C.c_double), C.c_uint32],
    "jmm_large_get_positions": [C.c_void_p, C.c_uint32, P(C.c_double), C.c_uint64],
    "jmm_large_set_positions": [C.c_void_p, C.c_uint32, P(C.c_double), C.c_uint64],
    "jmm_large_destroy": [C.c_void_p],
    "jmm_large_run_host": [P(abi.BatchConfig), P(abi.ChainDesc), C.c_uint32, C.c_uint32,
                           C.c_int32, P(C.c_double), C.c_uint64, P(abi.LargeResult),
                           P(C.c_double)],
})

MODES = {"domains": abi.JMM_LARGE_DOMAINS, "sequential": abi.JMM_LARGE_SEQUENTIAL}


class LargeChains:
    def __init__(self, config, chains, domain_size=256):
        self.config = config
        self.chains = list(chains)
        self.domain_size = int(domain_size)
        arr = (abi.ChainDesc * len(self.chains))(*self.chains)
        self._h = C.c_void_p()
        _native.call("jmm_large_create", C.byref(config), arr, len(self.chains),
                     self.domain_size, C.byref(self._h))

    @property
    def n_chains(self):
        return len(self.chains)

    def close(self):
        if self._h:
            _native.load().jmm_large_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def run(self, n_sweeps, mode="domains"):
        _native.call("jmm_large_run", self._h, int(n_sweeps), MODES[mode])

    def run_async(self, n_sweeps, mode="domains", stream=None):
        """Enqueue on a CUDA stream handle (int or None = the handle's own)."""
        _native.call("jmm_large_run_async", self._h, int(n_sweeps), MODES[mode],
                     C.c_void_p(stream) if stream else None)

    def results(self):
        out = (abi.LargeResult * self.n_chains)()
        _native.call("jmm_large_results", self._h, out, self.n_chains)
        return np.frombuffer(out, dtype=np.dtype(abi.LARGE_RESULT_DTYPE)).copy()

    def reset_stats(self):
        _native.call("jmm_large_reset_stats", self._h)

    def energies(self):
        e = np.empty(self.n_chains, dtype=np.float64)
        _native.call("jmm_large_energies", self._h, e.ctypes.data_as(P(C.c_double)),
                     self.n_chains)
        return e

    def positions(self, k):
        n = int(self.chains[k].n)
        x = np.empty(n, dtype=np.float64)
        _native.call("jmm_large_get_positions", self._h, k, x.ctypes.data_as(P(C.c_double)), n)
        return x

    def set_positions(self, k, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        _native.call("jmm_large_set_positions", self._h, k, x.ctypes.data_as(P(C.c_double)),
                     x.size)


def run_host(config, chains, n_sweeps, domain_size=256, mode="domains", x_in=None, x_out=None):
    """jmm_large_run_host: positions (float64, chain after chain, or None for
    the configured lattice) in, results and final positions out.  x_out may
    be a caller-owned float64 array (pinned memory, for instance)."""
    chains = list(chains)
    arr = (abi.ChainDesc * len(chains))(*chains)
    n_tot = sum(int(c.n) for c in chains)
    if x_in is not None:
        x_in = np.ascontiguousarray(x_in, dtype=np.float64)
        if x_in.size != n_tot:
            raise ValueError(f"x_in holds {x_in.size} positions, the chains {n_tot}")
    if x_out is None:
        x_out = np.empty(n_tot, dtype=np.float64)
    elif not (isinstance(x_out, np.ndarray) and x_out.dtype == np.float64 and x_out.size == n_tot
              and x_out.flags.c_contiguous and x_out.flags.writeable):
        raise ValueError(f"x_out must be a writeable C-contiguous float64 array of {n_tot}")
    res = (abi.LargeResult * len(chains))()
    _native.call("jmm_large_run_host", C.byref(config), arr, len(chains), int(domain_size),
                 MODES[mode], x_in.ctypes.data_as(P(C.c_double)) if x_in is not None else None,
                 int(n_sweeps), res, x_out.ctypes.data_as(P(C.c_double)))
    return np.frombuffer(res, dtype=np.dtype(abi.LARGE_RESULT_DTYPE)).copy(), x_out
