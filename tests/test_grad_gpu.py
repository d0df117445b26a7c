"""The backward kernel (jmm_energy_grad / jmm_batch_energy_grad) and its
torch layer, on configurations of the differentiation workload (N = 512
Lennard-Jones particles at rho = 0.7, T = 1, cut-off 3):

* U and dU/d(eps, sigma, L) of the GPU's configurations against the FP64
  oracle gradient (1e-5 relative; U to 1e-6) and against central finite
  differences of FP64 energies with step 1e-4 (1e-4 relative);
* torch.autograd through chain_energy: parameter gradients and positions'
  gradients (forces) against the same references;
* the fluctuation-formula gradients of a sampled run, d<U>/deps (NVT) and
  d<rho>/dsigma (NPT), against finite differences of the ensemble averages
  of runs at eps (sigma) +- delta with the same random numbers.
"""
import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.batch import ChainBatch, averages
from tests import oracle_lib

pytestmark = pytest.mark.gpu


def _near_cutoff(x, rc, h):
    d = np.abs(x[None, :] - x[:, None])[np.triu_indices(len(x), 1)]
    return np.any(np.abs(d - rc) < 3 * rc * h)


def _equilibrated(n_chains, n, ensemble, sweeps, seed=3):
    chains = [abi.make_chain(n, ensemble=ensemble, rho=0.7, t=1.0, p=1.0, cutoff=3.0,
                             max_step=0.3, vol_step=0.02) for _ in range(n_chains)]
    b = ChainBatch(abi.make_batch_config(seed=seed, resum_sweeps=10), chains)
    b.run(sweeps)
    return b, chains


def test_kernel_gradient_matches_fp64_and_finite_differences(gpu):
    b, chains = _equilibrated(48, 512, abi.JMM_NLT, 40)
    g = b.energy_grad()
    res = b.results()
    h = 1e-4
    fd_checked = 0
    for k, c in enumerate(chains):
        x = b.positions(k).astype(np.float64)
        l = res["l"][k]
        ref = oracle_lib.energy_grad64(c, x, l)
        assert abs(g[k, 0] - ref[0]) <= 1e-6 * abs(ref[0])
        for q in (1, 2, 3):
            assert abs(g[k, q] - ref[q]) <= 1e-5 * max(1.0, abs(ref[q])), (k, q, g[k, q], ref[q])
        if _near_cutoff(x, c.cutoff, h):
            continue

        def energy(eps=1.0, sigma=1.0, scale=1.0):
            cc = abi.make_chain(c.n, cutoff=c.cutoff, eps=eps, sigma=sigma, l0=l)
            return oracle_lib.energy64(cc, x * scale, l * scale)

        fd = [(energy(eps=1 + h) - energy(eps=1 - h)) / (2 * h),
              (energy(sigma=1 + h) - energy(sigma=1 - h)) / (2 * h),
              (energy(scale=1 + h) - energy(scale=1 - h)) / (2 * h * l)]
        for q in (1, 2, 3):
            assert abs(g[k, q] - fd[q - 1]) <= 1e-4 * max(1.0, abs(fd[q - 1])), (k, q)
        fd_checked += 1
    assert fd_checked >= 10


def test_torch_autograd_through_chain_energy(gpu):
    import torch
    from jmmonedmc_gb300.grad import Layout, chain_energy, energy_and_gradients
    b, chains = _equilibrated(8, 512, abi.JMM_NLT, 20, seed=8)
    res = b.results()
    xs = [b.positions(k) for k in range(len(chains))]
    layout = Layout([c.n for c in chains], cutoff=3.0)
    dev = torch.device("cuda")
    x = torch.tensor(np.concatenate(xs), dtype=torch.float32, device=dev, requires_grad=True)
    l = torch.tensor(res["l"], dtype=torch.float64, device=dev, requires_grad=True)
    eps = torch.ones(len(chains), dtype=torch.float64, device=dev, requires_grad=True)
    sigma = torch.ones(len(chains), dtype=torch.float64, device=dev, requires_grad=True)
    u = chain_energy(x, l, eps, sigma, layout)
    w = torch.arange(1, len(chains) + 1, dtype=torch.float64, device=dev)
    (u * w).sum().backward()
    out, forces = energy_and_gradients(x.detach(), l, eps, sigma, layout, forces=True)
    wn = w.cpu().numpy()
    np.testing.assert_allclose(eps.grad.cpu().numpy(), wn * out[:, 1].cpu().numpy(), rtol=1e-12)
    np.testing.assert_allclose(sigma.grad.cpu().numpy(), wn * out[:, 2].cpu().numpy(), rtol=1e-12)
    np.testing.assert_allclose(l.grad.cpu().numpy(), wn * out[:, 3].cpu().numpy(), rtol=1e-12)
    # positions: -forces against central differences of FP64 energies
    gx = x.grad.cpu().numpy()
    h = 1e-5
    for k, c in ((0, chains[0]), (5, chains[5])):
        off = sum(cc.n for cc in chains[:k])
        xk = xs[k].astype(np.float64)
        for i in (0, 17, 256, 511):
            xp, xm = xk.copy(), xk.copy()
            xp[i] += h
            xm[i] -= h
            cc = abi.make_chain(c.n, cutoff=3.0, l0=res["l"][k])
            fd = (oracle_lib.energy64(cc, xp, res["l"][k]) - oracle_lib.energy64(cc, xm, res["l"][k])) / (2 * h)
            assert abs(gx[off + i] / (k + 1) - fd) <= 1e-3 * max(1.0, abs(fd)), (k, i, gx[off + i], fd)


def _sampled_average(ensemble, key, eps=1.0, sigma=1.0, n_chains=512, n=64, sweeps=4000,
                     seed=11):
    chains = [abi.make_chain(n, ensemble=ensemble, rho=0.7, t=1.0, p=1.0, cutoff=3.0, eps=eps,
                             sigma=sigma, max_step=0.3, vol_step=0.05) for _ in range(n_chains)]
    b = ChainBatch(abi.make_batch_config(seed=seed, resum_sweeps=10), chains)
    b.run(500)  # equilibration
    b.reset_stats()
    b.run_sampled(sweeps, 10)
    return b, b.grad_stats()


def test_fluctuation_gradient_of_energy_nvt(gpu):
    from jmmonedmc_gb300.grad import fluctuation_gradients
    b, st = _sampled_average(abi.JMM_NLT, "u")
    fg = fluctuation_gradients(st, np.ones(len(st)))
    est = fg["dU_deps"]
    delta = 0.05
    up = _sampled_average(abi.JMM_NLT, "u", eps=1 + delta)[1]
    dn = _sampled_average(abi.JMM_NLT, "u", eps=1 - delta)[1]
    fd = (up["sum_u"] / up["samples"] - dn["sum_u"] / dn["samples"]) / (2 * delta)
    diff = est.mean() - fd.mean()
    sem = np.sqrt(est.var(ddof=1) / len(est) + fd.var(ddof=1) / len(fd))
    print(f"d<U>/deps: fluctuation {est.mean():.4f}, finite difference {fd.mean():.4f}, "
          f"standard error {sem:.4f}")
    assert abs(diff) < 4 * sem + 0.02 * abs(fd.mean()), (est.mean(), fd.mean(), sem)


def test_fluctuation_gradient_of_density_npt(gpu):
    from jmmonedmc_gb300.grad import fluctuation_gradients
    b, st = _sampled_average(abi.JMM_NPT, "rho")
    fg = fluctuation_gradients(st, np.ones(len(st)))
    est = fg["drho_dsigma"]
    delta = 0.02
    up = _sampled_average(abi.JMM_NPT, "rho", sigma=1 + delta)[1]
    dn = _sampled_average(abi.JMM_NPT, "rho", sigma=1 - delta)[1]
    fd = (up["sum_rho"] / up["samples"] - dn["sum_rho"] / dn["samples"]) / (2 * delta)
    diff = est.mean() - fd.mean()
    sem = np.sqrt(est.var(ddof=1) / len(est) + fd.var(ddof=1) / len(fd))
    print(f"d<rho>/dsigma: fluctuation {est.mean():.5f}, finite difference {fd.mean():.5f}, "
          f"standard error {sem:.5f}")
    assert abs(diff) < 4 * sem + 0.02 * abs(fd.mean()), (est.mean(), fd.mean(), sem)
