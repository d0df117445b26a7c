"""The allocation-free full-energy entry point against the existing path.

jmm_plain_full_energy_noalloc serves callers that may not allocate device
memory (a stream being captured into a CUDA graph, a host that reserves all
memory at start-up, a per-step loop that cannot pay for an allocation).  It
must give the same nine FP64 totals, bit for bit, as the plain chain's own
full sum (set the positions, then fad(0, 0.5), which allocates its scratch
with the chain), on consecutive calls that share its fixed staging array.
This file sorts last so that a stop-at-first-failure run has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from jmmonedmc_gb300 import _native, abi
from jmmonedmc_gb300.plain import PlainChain

pytestmark = pytest.mark.gpu

MAX_N = 256


def _entry(lib):
    fn = lib.jmm_plain_full_energy_noalloc
    fn.argtypes = [C.POINTER(abi.Params), C.c_void_p, C.c_uint64, C.c_double, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    return fn


def _chain_positions(params, steps):
    ch = PlainChain(params)
    ch.fad()
    ch.steps(steps)
    return ch.positions(), ch.state().l


def _existing_totals(params, r, l):
    ch = PlainChain(params)
    ch.set_config(r, l)
    ch.fad(0, 0.5)
    return np.array(ch.state().tot)


def _noalloc_totals(lib, params, r, l):
    import torch
    r_dev = torch.tensor(np.asarray(r), dtype=torch.float64, device="cuda")
    out = torch.full((9,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = _entry(lib)(C.byref(params), r_dev.data_ptr(), r_dev.numel(), float(l), out.data_ptr(),
                     None)
    torch.cuda.synchronize()
    assert rc == abi.JMM_OK, lib.jmm_last_error().decode()
    return out.cpu().numpy()


def test_noalloc_full_energy_matches_existing_path(gpu):
    lib = _native.load()
    cases = [
        abi.make_params(n=200, ensemble=abi.JMM_NPT, p=1.0, t=1.0, cutoff=3.0, max_step=0.3,
                        max_dl=2.0, seed=3),
        abi.make_params(n=64, l=64 / 0.6, t=0.8, potential=abi.JMM_POT_LJ, nbn=3, max_step=0.3,
                        seed=9),
        abi.make_params(n=MAX_N, l=MAX_N / 0.7, t=1.2, cutoff=2.5, max_step=0.2, seed=5),
        # HARMONIC with a neighbour limit (the golden npt10_harmonic_nbn1 kind):
        # its virial divides by L; both paths leave phi[2..8] at 0
        abi.make_params(n=10, ensemble=abi.JMM_NPT, potential=abi.JMM_POT_HARMONIC, p=1.0,
                        t=1.0, cutoff=2.0, nbn=1, max_step=0.3, max_dl=0.5, seed=7),
    ]
    for params in cases:  # consecutive calls share the staging array
        r, l = _chain_positions(params, 3000)
        want = _existing_totals(params, r, l)
        got = _noalloc_totals(lib, params, r, l)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (got, want)


def test_noalloc_rejects_sizes_beyond_its_array(gpu):
    import torch
    lib = _native.load()
    params = abi.make_params(n=MAX_N + 1, l=400.0)
    r = torch.linspace(-190.0, 190.0, MAX_N + 1, dtype=torch.float64, device="cuda")
    out = torch.empty(9, dtype=torch.float64, device="cuda")
    rc = _entry(lib)(C.byref(params), r.data_ptr(), MAX_N + 1, 400.0, out.data_ptr(), None)
    assert rc == abi.JMM_ERR_INVALID
    assert b"exceeds" in lib.jmm_last_error()


def test_noalloc_refuses_host_memory_and_bad_box(gpu):
    """Pinned host buffers (which a kernel could read, so the check is what
    refuses them) and a box length that is not finite and positive are
    refused before any launch."""
    import torch
    lib = _native.load()
    params = abi.make_params(n=16, l=32.0)
    r_dev = torch.linspace(-15.0, 15.0, 16, dtype=torch.float64, device="cuda")
    out_dev = torch.empty(9, dtype=torch.float64, device="cuda")
    r_host = r_dev.cpu().pin_memory()
    out_host = torch.empty(9, dtype=torch.float64).pin_memory()
    for r, out in ((r_host, out_dev), (r_dev, out_host)):
        rc = _entry(lib)(C.byref(params), r.data_ptr(), 16, 32.0, out.data_ptr(), None)
        assert rc == abi.JMM_ERR_INVALID
        assert b"device memory" in lib.jmm_last_error()
    for l in (float("nan"), 0.0, -1.0, float("inf")):
        rc = _entry(lib)(C.byref(params), r_dev.data_ptr(), 16, l, out_dev.data_ptr(), None)
        assert rc == abi.JMM_ERR_INVALID
