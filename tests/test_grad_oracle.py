"""The FP64 gradient oracle against central finite differences (CPU)."""
import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from tests import oracle_lib


def _config(rng, n, pot, cutoff, rho, periodic):
    l = n / rho
    x = ((np.arange(n) + 0.5) / n - 0.5) * l + rng.uniform(-0.08, 0.08, n) * (1 / rho)
    return abi.make_chain(n, potential=pot, cutoff=cutoff, l0=l), np.sort(x), l


def _pairs_near_cutoff(x, l, rc, h, periodic):
    d = np.abs(x[None, :] - x[:, None])
    if periodic:
        d = np.minimum(d, l - d)
    return np.any(np.abs(d[np.triu_indices(len(x), 1)] - rc) < 3 * rc * h)


@pytest.mark.parametrize("pot,cutoff", [(abi.JMM_POT_LJCUT, 3.0), (abi.JMM_POT_SOFTSPHERE, 2.5),
                                        (abi.JMM_POT_GAUSS, 4.0)])
@pytest.mark.parametrize("periodic", [False, True])
def test_fp64_gradient_matches_central_differences(pot, cutoff, periodic):
    rng = np.random.default_rng(7)
    checked = 0
    for trial in range(20):
        c, x, l = _config(rng, 96, pot, cutoff, 0.7, periodic)
        h = 1e-4
        if _pairs_near_cutoff(x, l, cutoff, h, periodic):
            continue
        g = oracle_lib.energy_grad64(c, x, l, periodic)

        def energy(eps=c.eps, sigma=c.sigma, scale=1.0):
            cc = abi.make_chain(c.n, potential=pot, cutoff=cutoff, eps=eps, sigma=sigma, l0=l)
            return oracle_lib.energy64(cc, x * scale, l * scale, periodic)

        fd_eps = (energy(eps=1 + h) - energy(eps=1 - h)) / (2 * h)
        fd_sig = (energy(sigma=1 + h) - energy(sigma=1 - h)) / (2 * h)
        fd_l = (energy(scale=1 + h) - energy(scale=1 - h)) / (2 * h * l)
        assert abs(g[0] - energy()) <= 1e-12 * max(1, abs(g[0]))
        for got, want in ((g[1], fd_eps), (g[2], fd_sig), (g[3], fd_l)):
            assert abs(got - want) <= 1e-6 * max(1.0, abs(want)), (got, want)
        checked += 1
    assert checked >= 5


def test_launch_checks_shapes_and_device():
    """Wrong sizes and host tensors are refused before any launch."""
    import torch
    from jmmonedmc_gb300.grad import Layout, chain_energy, energy_and_gradients
    lay = Layout([4, 6])
    ones = torch.ones(2, dtype=torch.float64)
    with pytest.raises(ValueError, match="positions"):
        energy_and_gradients(torch.zeros(9), ones, ones, ones, lay)
    with pytest.raises(ValueError, match="eps"):
        energy_and_gradients(torch.zeros(10), ones, torch.ones(3), ones, lay)
    with pytest.raises(ValueError, match="CUDA"):
        energy_and_gradients(torch.zeros(10), ones, ones, ones, lay)
    with pytest.raises(ValueError, match="CUDA"):
        chain_energy(torch.zeros(10, requires_grad=True), ones, ones, ones, lay)
