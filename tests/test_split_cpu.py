"""Split chains (jmm_batch_config.split_n) on the CPU: the oracle's replay of
the alternating-domain sweep samples the same ensemble as the whole chain,
keeps its energy bookkeeping, and the batch refuses a bad split size.

The split sweep (per sweep: domains of B particles from a random offset, one
colour of domains at a time, frozen neighbours between active domains) is a
product of independent Metropolis chains per phase, each on the conditional
distribution of its domain given the rest; these tests check that claim
statistically against the plain sequential sweep of the same chains."""
import math

import numpy as np
import pytest

from jmmonedmc_gb300 import _native, abi
from jmmonedmc_gb300.batch import ChainBatch
from tests import oracle_lib

REPLICAS, EQUIL, PROD = 32, 300, 1500


def _run(split_n, pot, n, rho, t, cutoff, seed):
    chains = [abi.make_chain(n, potential=pot, ensemble=abi.JMM_NLT, cutoff=cutoff, t=t,
                             rho=rho, max_step=0.3) for _ in range(REPLICAS)]
    cfg = abi.make_batch_config(seed=seed, precision=abi.JMM_PREC_EXACT, resum_sweeps=50,
                                split_n=split_n)
    b = oracle_lib.OracleBatch(cfg, chains)
    b.run(EQUIL)
    r0 = b.results()
    b.run(PROD)
    r1 = b.results()
    s = (r1["samples"] - r0["samples"]).astype(np.float64)
    u = (r1["sum_e"] - r0["sum_e"]) / s / n
    e2 = (r1["sum_e2"] - r0["sum_e2"]) / s
    x = [b.positions(k) for k in range(REPLICAS)]
    b.close()
    return chains, r1, u, e2, x


@pytest.mark.parametrize("pot, rho, t, cutoff", [
    (abi.JMM_POT_LJCUT, 0.7, 1.0, 3.0),
    (abi.JMM_POT_GAUSS, 0.9, 0.5, 4.0),
])
def test_split_sweep_samples_the_whole_chains_ensemble(pot, rho, t, cutoff):
    """<U>/N and Var(U)/N of 32 replicas of N = 256 chains, split into
    domains of 32 (split_n = 64) against the same chains run whole: within 3
    combined standard errors (replica spread; the split run samples once per
    sweep, the whole run every step)."""
    n = 256
    _, rs, us, e2s, _ = _run(64, pot, n, rho, t, cutoff, 11)
    _, rw, uw, e2w, _ = _run(0, pot, n, rho, t, cutoff, 12)
    assert np.all(rs["samples"] == EQUIL + PROD) and np.all(rw["samples"] == (EQUIL + PROD) * n)
    for a, b, what in ((us, uw, "<U>/N"),
                       (e2s / n - us * us * n, e2w / n - uw * uw * n, "Var(U)/N")):
        se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
        z = (a.mean() - b.mean()) / se
        print(f"{what}: split {a.mean():.5f}, whole {b.mean():.5f}, z = {z:+.2f}")
        assert abs(z) < 3.0


def test_split_replay_keeps_its_energy_and_order():
    """After a split run every chain is ordered inside its walls and its
    running energy agrees with the fresh FP64 sum of its positions (the
    domains' FP32 changes add up to the energy's change)."""
    n = 700
    chains, res, _, _, xs = _run(128, abi.JMM_POT_LJCUT, n, 0.8, 0.8, 3.0, 5)
    assert not np.any(res["error"])
    for c, x, e, l in zip(chains, xs, res["e"], res["l"]):
        assert np.all(np.diff(x) > 0) and abs(x[0]) <= l / 2 and abs(x[-1]) <= l / 2
        fresh = oracle_lib.energy64(c, x, l)
        assert abs(e - fresh) <= 1e-5 * abs(fresh), (e, fresh)
    assert np.all(res["steps"] == (EQUIL + PROD) * n)


def test_split_size_must_be_zero_or_at_least_64(native):
    for bad in (1, 32, 63):
        with pytest.raises(_native.JmmError) as ei:
            ChainBatch(abi.make_batch_config(seed=1, split_n=bad), [abi.make_chain(128)])
        assert ei.value.code == abi.JMM_ERR_INVALID
