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


def test_fluctuation_gradients_formula():
    """d<A>/dtheta = <dA/dtheta> - beta (<A dU/dtheta> - <A><dU/dtheta>) from
    the accumulated sums, against the same formula on the samples directly."""
    from jmmonedmc_gb300.grad import fluctuation_gradients
    rng = np.random.default_rng(3)
    n_chains, m = 5, 400
    t = rng.uniform(0.5, 2.0, n_chains)
    stats = np.zeros(n_chains, dtype=np.dtype(abi.GRAD_STATS_DTYPE))
    want = {}
    for c in range(n_chains):
        u = rng.normal(-100, 5, m)
        g = np.stack([u / 1.3 + rng.normal(0, 1, m), rng.normal(40, 3, m),
                      rng.normal(-2, 1, m)], axis=1)
        l = rng.normal(50, 2, m)
        rho = 32 / l
        s = stats[c]
        s["samples"] = m
        s["sum_u"], s["sum_u2"], s["sum_rho"] = u.sum(), (u * u).sum(), rho.sum()
        s["sum_rho2"], s["sum_l"] = (rho * rho).sum(), l.sum()
        s["sum_g"], s["sum_u_g"] = g.sum(0), (u[:, None] * g).sum(0)
        s["sum_rho_g"], s["sum_l_g"] = (rho[:, None] * g).sum(0), (l[:, None] * g).sum(0)
        stats[c] = s
        b = 1 / t[c]
        for k, th in enumerate(("eps", "sigma")):
            cov = lambda a: (a * g[:, k]).mean() - a.mean() * g[:, k].mean()
            want.setdefault(f"dU_d{th}", []).append(g[:, k].mean() - b * cov(u))
            want.setdefault(f"drho_d{th}", []).append(-b * cov(rho))
            want.setdefault(f"dL_d{th}", []).append(-b * cov(l))
    got = fluctuation_gradients(stats, t)
    assert set(got) == set(want)
    for key, vals in want.items():
        np.testing.assert_allclose(got[key], vals, rtol=1e-9, atol=1e-9)
