"""Split chains (jmm_batch_config.split_n) on the GPU.

* EXACT precision: every field of every chain's record and every position
  equals the oracle's replay of the alternating-domain sweep bit for bit
  (domains of one phase share no pair, so the oracle's one-after-another
  replay is the GPU's result), for a batch mixing split and whole chains of
  the three potentials, over several launches, with the default and a wide
  window.
* FAST precision: the uneven workload with its long chains split runs at
  full size without error, ordered, with energies equal to the FP64 oracle's
  sums of the GPU's positions; a checkpointed batch continues bit for bit.
"""
import argparse

import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.batch import ChainBatch
from tests import oracle_lib

pytestmark = pytest.mark.gpu

FIELDS = [f for f, _ in abi.CHAIN_RESULT_DTYPE]


def _mixed(rng, n_chains):
    pots = ((abi.JMM_POT_LJCUT, 3.0), (abi.JMM_POT_SOFTSPHERE, 2.5), (abi.JMM_POT_GAUSS, 4.0))
    chains = []
    for k in range(n_chains):
        pot, cut = pots[k % 3]
        chains.append(abi.make_chain(int(rng.integers(40, 900)), potential=pot,
                                     ensemble=abi.JMM_NLT, cutoff=cut,
                                     t=float(rng.uniform(0.5, 2.0)),
                                     rho=float(rng.uniform(0.3, 0.9)), max_step=0.3))
    # an NPT chain above split_n runs whole
    chains.append(abi.make_chain(600, ensemble=abi.JMM_NPT, t=1.0, p=1.0, rho=0.6,
                                 max_step=0.3, vol_step=0.01))
    return chains


@pytest.mark.parametrize("window", [0, 8], ids=["window_default", "window8"])
def test_split_exact_equals_oracle(gpu, window):
    rng = np.random.default_rng(31 + window)
    chains = _mixed(rng, 24)
    cfg = abi.make_batch_config(seed=17, precision=abi.JMM_PREC_EXACT, resum_sweeps=3,
                                lanes_per_chain=4, steps_per_round=8, window=window,
                                split_n=128)
    g, o = ChainBatch(cfg, chains), oracle_lib.OracleBatch(cfg, chains)
    n_split = sum(1 for c in chains if c.n >= 128 and c.ensemble == abi.JMM_NLT)
    assert n_split >= 10
    for sweeps in (5, 1, 7):
        g.run(sweeps)
        o.run(sweeps)
        rg, ro = g.results(), o.results()
        for f in FIELDS:
            a, b = rg[f], ro[f]
            bad = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0] if a.dtype.kind == "f" \
                else np.nonzero(a != b)[0]
            assert bad.size == 0, f"{f} differs for chains {bad[:6]}: {a[bad[:3]]} vs {b[bad[:3]]}"
        for k in range(len(chains)):
            assert np.array_equal(g.positions(k).astype(np.float64), o.positions(k)), k
    assert not np.any(rg["error"])
    # split chains sample once per sweep, whole chains every step
    for c, s in zip(chains, rg["samples"]):
        split = c.n >= 128 and c.ensemble == abi.JMM_NLT
        assert s == 13 * (1 if split else (c.n + (c.ensemble == abi.JMM_NPT)))
    g.close()
    o.close()


def _uneven(split_n):
    import bench
    args = argparse.Namespace(chains=1024, seed=1, workload="uneven", n=256)
    cfg, chains = bench.uneven_workload(args, 1)
    cfg.split_n = split_n
    return cfg, chains


def test_uneven_batch_split_at_full_size(gpu):
    cfg, chains = _uneven(384)
    b = ChainBatch(cfg, chains)
    b.run(20)
    res = b.results()
    assert np.all(res["error"] == 0)
    assert np.all(res["steps"] == 20 * np.array([c.n for c in chains]))
    fresh = b.energies()
    for k in range(0, 1024, 61):
        x = b.positions(k).astype(np.float64)
        assert np.all(np.diff(x) > 0)
        e64 = oracle_lib.energy64(chains[k], x, res["l"][k])
        assert abs(fresh[k] - e64) <= 1e-6 * max(1.0, abs(e64)), (k, fresh[k], e64)
        # the running energy (domains' FP32 changes) against the fresh sum
        assert abs(res["e"][k] - fresh[k]) <= 1e-4 * max(1.0, abs(fresh[k])), k
    b.close()


def test_split_checkpoint_continues_bit_for_bit(gpu, tmp_path):
    cfg, chains = _uneven(384)
    chains = chains[:64]
    a = ChainBatch(cfg, chains)
    a.run(5)
    path = tmp_path / "split.npz"
    a.checkpoint(str(path))
    a.run(5)
    b = ChainBatch.restore(str(path))
    b.run(5)
    ra, rb = a.results(), b.results()
    for f in FIELDS:
        assert ra[f].tobytes() == rb[f].tobytes(), f
    for k in range(len(chains)):
        assert np.array_equal(a.positions(k), b.positions(k))
