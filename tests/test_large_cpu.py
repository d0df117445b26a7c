"""Argument checks of the large-chain entry points (jmm_large_*): every bad
combination is refused with JMM_ERR_INVALID before any device work, so these
run without a GPU."""
import pytest

from jmmonedmc_gb300 import _native, abi
from jmmonedmc_gb300.large import LargeChains


def _expect_invalid(cfg, chains, b):
    with pytest.raises(_native.JmmError) as ei:
        LargeChains(cfg, chains, domain_size=b)
    assert ei.value.code == abi.JMM_ERR_INVALID


def _chain(n=4096, **kw):
    return abi.make_chain(n, rho=0.7, t=1.2, cutoff=2.5, max_step=0.4, **kw)


def test_domain_size_bounds(native):
    cfg = abi.make_batch_config(seed=1)
    _expect_invalid(cfg, [_chain()], 16)       # below 2 x 16 halo particles
    _expect_invalid(cfg, [_chain()], 16384)    # above 8192
    _expect_invalid(cfg, [_chain(n=100)], 128)  # N below the domain size


def test_unsupported_chains(native):
    cfg = abi.make_batch_config(seed=1)
    _expect_invalid(cfg, [_chain(ensemble=abi.JMM_NPT)], 256)
    _expect_invalid(cfg, [_chain(potential=abi.JMM_POT_HARMONIC)], 256)
    _expect_invalid(abi.make_batch_config(seed=1, boundary=abi.JMM_BOUNDARY_PERIODIC),
                    [_chain()], 256)
    _expect_invalid(abi.make_batch_config(seed=1, precision=abi.JMM_PREC_EXACT), [_chain()], 256)


@pytest.mark.parametrize("field, value", [
    ("cutoff", float("inf")), ("l0", float("inf")), ("t", float("inf")),
    ("eps", float("nan")), ("sigma", float("inf")), ("max_step", float("inf")),
])
def test_chain_parameters_must_be_finite(native, field, value):
    c = _chain()
    setattr(c, field, value)
    _expect_invalid(abi.make_batch_config(seed=1), [_chain(), c], 256)


def test_run_host_checks_host_buffers():
    """Host buffers of the wrong size or type are refused before any native call."""
    import numpy as np
    from jmmonedmc_gb300.large import run_host
    cfg = abi.make_batch_config(seed=1)
    chains = [_chain(), _chain()]
    with pytest.raises(ValueError, match="x_in"):
        run_host(cfg, chains, 1, domain_size=256, x_in=np.zeros(100))
    for bad in (np.zeros(8191), np.zeros(8192, dtype=np.float32), np.zeros(16384)[::2]):
        with pytest.raises(ValueError, match="x_out"):
            run_host(cfg, chains, 1, domain_size=256, x_out=bad)
