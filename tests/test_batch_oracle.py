"""The batched form's oracle on its own (CPU): portable math, FP32 vs FP64
energies, and analytic limits that pin the chain's sampling (ideal-gas NPT
box length and order statistics), since the reference has no batched form
to compare with."""
import math

import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from tests import oracle_lib


def test_portable_logf_expf_against_libm():
    lib = oracle_lib.load()
    for u in np.linspace(1e-7, 1 - 1e-7, 4001, dtype=np.float32):
        ref = math.log(float(u))
        assert abs(lib.jmmo_portable_logf(float(u)) - ref) <= 4e-7 * max(1.0, abs(ref))
    for x in np.linspace(-80, 80, 4001, dtype=np.float32):
        ref = math.exp(float(x))
        assert abs(lib.jmmo_portable_expf(float(x)) - ref) <= 4e-7 * ref


def test_fp32_energies_agree_with_fp64():
    rng = np.random.default_rng(0)
    chains = [abi.make_chain(int(n), potential=p, cutoff=c, rho=float(r))
              for n, p, c, r in zip(rng.integers(32, 400, 12),
                                    [abi.JMM_POT_LJCUT, abi.JMM_POT_SOFTSPHERE, abi.JMM_POT_GAUSS] * 4,
                                    [3.0, 2.5, 4.0] * 4, rng.uniform(0.3, 0.9, 12))]
    cfg = abi.make_batch_config(seed=1, precision=abi.JMM_PREC_EXACT, init=abi.JMM_INIT_JITTER,
                                jitter=0.1)
    b = oracle_lib.OracleBatch(cfg, chains)
    b.run(20)
    e32 = b.energies()
    for k, c in enumerate(chains):
        e64 = oracle_lib.energy64(c, b.positions(k), b.results()["l"][k])
        assert abs(e32[k] - e64) <= 1e-6 * max(1.0, abs(e64))


@pytest.mark.parametrize("vol_move", [abi.JMM_VOLMOVE_LNL, abi.JMM_VOLMOVE_LINEAR])
def test_ideal_gas_npt_box_length(vol_move):
    """<L> = (N+1) T / P for N ideal particles in 1D at pressure P."""
    n, t, p = 6, 1.0, 1.0
    step = 0.3 if vol_move == abi.JMM_VOLMOVE_LNL else 3.0
    chains = [abi.make_chain(n, potential=abi.JMM_POT_GAUSS, eps=0.0, cutoff=0.5,
                             ensemble=abi.JMM_NPT, t=t, p=p, l0=7.0, max_step=1.5,
                             vol_step=step) for _ in range(64)]
    cfg = abi.make_batch_config(seed=21, vol_move=vol_move, vol_schedule=abi.JMM_VOLSCHED_RANDOM)
    b = oracle_lib.OracleBatch(cfg, chains, fp64=True)
    b.run(200)
    b.lib.jmmo_batch_run  # keep the handle alive
    res0 = b.results()
    b.run(3000)
    res = b.results()
    sum_l = res["sum_l"] - res0["sum_l"]
    samples = (res["samples"] - res0["samples"]).astype(float)
    per_chain = sum_l / samples
    mean, sem = per_chain.mean(), per_chain.std(ddof=1) / math.sqrt(len(per_chain))
    assert abs(mean - (n + 1) * t / p) < 4 * sem + 0.02, (mean, sem)


def test_ideal_gas_order_statistics():
    """Ideal particles between walls sample the ordered region uniformly:
    E[x_(k)] = L (k/(N+1) - 1/2)."""
    n, l = 5, 10.0
    chains = [abi.make_chain(n, potential=abi.JMM_POT_GAUSS, eps=0.0, cutoff=0.5, l0=l,
                             max_step=2.0) for _ in range(400)]
    b = oracle_lib.OracleBatch(abi.make_batch_config(seed=5), chains, fp64=True)
    b.run(300)
    x = np.array([b.positions(k) for k in range(len(chains))])
    want = l * (np.arange(1, n + 1) / (n + 1) - 0.5)
    sd = l * np.sqrt(np.arange(1, n + 1) * (n + 1 - np.arange(1, n + 1)) /
                     ((n + 1) ** 2 * (n + 2)))
    assert np.all(np.abs(x.mean(axis=0) - want) < 4 * sd / math.sqrt(len(chains)))
