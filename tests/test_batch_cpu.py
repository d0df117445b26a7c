"""Argument and position checks of the batched entry points that come before
any device work (jmm_batch_create_at, launch-shape choice), so these run
without a GPU: every bad input is refused with JMM_ERR_INVALID."""
import numpy as np
import pytest

from jmmonedmc_gb300 import _native, abi
from jmmonedmc_gb300.batch import ChainBatch


def _expect_invalid(cfg, chains, x=None):
    with pytest.raises(_native.JmmError) as ei:
        ChainBatch(cfg, chains, x=x)
    assert ei.value.code == abi.JMM_ERR_INVALID


def _lattice(c):
    step = c.l0 / c.n
    return (-0.5 * c.l0 + step * (np.arange(c.n) + 0.5)).astype(np.float32)


def test_create_at_refuses_bad_positions(native):
    cfg = abi.make_batch_config(seed=1)
    chains = [abi.make_chain(16, rho=0.5), abi.make_chain(24, rho=0.5)]
    good = np.concatenate([_lattice(c) for c in chains])
    bad = good.copy()
    bad[20], bad[21] = bad[21], bad[20]  # chain 1 not increasing
    _expect_invalid(cfg, chains, bad)
    bad = good.copy()
    bad[0] = -0.6 * chains[0].l0  # beyond the left wall
    _expect_invalid(cfg, chains, bad)
    bad = good.copy()
    bad[5] = np.nan
    _expect_invalid(cfg, chains, bad)
    with pytest.raises(ValueError):  # not every chain's positions
        ChainBatch(cfg, chains, x=good[:-1])


def test_create_at_periodic_span(native):
    cfg = abi.make_batch_config(seed=1, boundary=abi.JMM_BOUNDARY_PERIODIC)
    c = abi.make_chain(40, rho=0.5, cutoff=2.5)
    x = np.linspace(-0.5 * c.l0, 0.5 * c.l0, c.n).astype(np.float32)  # spans exactly L
    _expect_invalid(cfg, [c], x)


def test_unsupported_window(native):
    c = [abi.make_chain(64, rho=0.5)]
    # a window of 8 exists only for 2x16, 4x8 and 8x4
    _expect_invalid(abi.make_batch_config(seed=1, lanes_per_chain=4, steps_per_round=4, window=8), c)
    _expect_invalid(abi.make_batch_config(seed=1, lanes_per_chain=4, steps_per_round=8, window=6), c)


@pytest.mark.parametrize("field, value", [
    ("cutoff", float("inf")), ("l0", float("inf")), ("t", float("inf")),
    ("sigma", float("nan")), ("eps", float("nan")), ("eps", float("inf")),
    ("p", float("nan")), ("vol_step", float("nan")), ("vol_step", -0.01),
    ("max_step", float("inf")), ("cutoff", 0.0), ("t", -1.0),
])
def test_chain_parameters_must_be_finite(native, field, value):
    """Non-finite chain parameters (an infinite cut-off would make every
    neighbour a partner) and a negative volume step are refused on the host."""
    c = abi.make_chain(64, rho=0.5, ensemble=abi.JMM_NPT)
    setattr(c, field, value)
    _expect_invalid(abi.make_batch_config(seed=1), [abi.make_chain(32, rho=0.5), c])


def test_take_histograms_needs_configuration():
    b = ChainBatch.__new__(ChainBatch)  # no device handle: the check comes first
    b._h, b._hist, b.chains = None, None, []
    with pytest.raises(RuntimeError, match="histograms"):
        b.take_histograms()


def test_run_host_checks_positions_size():
    from jmmonedmc_gb300.batch import run_host
    chains = [abi.make_chain(16, rho=0.5), abi.make_chain(24, rho=0.5)]
    with pytest.raises(ValueError, match="x_in"):
        run_host(abi.make_batch_config(seed=1), chains, 1, x_in=np.zeros(39, dtype=np.float32))
