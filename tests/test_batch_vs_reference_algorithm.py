"""The batched form's chain against the reference's own algorithm, on CPU.

The batched FP64 restatement (oracle/batch_oracle.c) keeps particles in
order and finds partners in an index window; the plain restatement
(oracle/plain_oracle.c) is the reference's move loop bit for bit (pinned to
the reference build by tests/test_oracle_vs_reference.py).  For LJ particles
that never pass each other, with linear volume moves drawn with probability
1/(N+1) per step as the reference's Step does, both sample the same
ensemble, and so do ln L volume moves closing every sweep (each move keeps
detailed balance; the batched NPT workload uses them); so <E> and <L> of
independent replicas must agree within their
combined standard error (the replicas' spread carries each chain's
autocorrelation).  The GPU's batched kernels are pinned to the batched
restatement separately, so this links them to the reference's algorithm."""
import functools
import math

import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from tests import oracle_lib

N, T, P, CUT, MAX_STEP = 32, 1.0, 1.0, 3.0, 0.3
REPLICAS, EQUIL_SWEEPS, SWEEPS = 48, 300, 3000


@functools.lru_cache(maxsize=None)
def plain_replicas(ensemble, l0, max_dl):
    types = N + 1 if ensemble == abi.JMM_NPT else N
    e, l = [], []
    for r in range(REPLICAS):
        prm = abi.make_params(n=N, ensemble=ensemble, potential=abi.JMM_POT_LJCUT, p=P, l=l0,
                              t=T, cutoff=CUT, max_step=MAX_STEP, max_dl=max_dl,
                              seed=101 + r, eci=0)
        c = oracle_lib.OraclePlain(prm)
        c.fad()
        c.steps(EQUIL_SWEEPS * types)
        log = c.steps(SWEEPS * types, log=True)
        e.append(log["e"].mean())
        l.append(log["l"].mean())
        c.close()
    return np.array(e), np.array(l)


def batch_replicas(ensemble, l0, vol_step, vol_move, schedule, fp64):
    chains = [abi.make_chain(N, potential=abi.JMM_POT_LJCUT, ensemble=ensemble, cutoff=CUT,
                             t=T, p=P, l0=l0, max_step=MAX_STEP, vol_step=vol_step)
              for _ in range(REPLICAS)]
    cfg = abi.make_batch_config(seed=77, vol_move=vol_move, vol_schedule=schedule,
                                precision=abi.JMM_PREC_EXACT, resum_sweeps=10)
    b = oracle_lib.OracleBatch(cfg, chains, fp64=fp64)
    b.run(EQUIL_SWEEPS)
    r0 = b.results()
    b.run(SWEEPS)
    r1 = b.results()
    b.close()
    s = (r1["samples"] - r0["samples"]).astype(np.float64)
    return (r1["sum_e"] - r0["sum_e"]) / s, (r1["sum_l"] - r0["sum_l"]) / s


def agree(a, b):
    sem = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    return abs(a.mean() - b.mean()), sem


@pytest.mark.parametrize("fp64", [True, False], ids=["fp64", "fp32_exact_kernel"])
@pytest.mark.parametrize("ensemble, vol_move, schedule, vol_step", [
    (abi.JMM_NLT, abi.JMM_VOLMOVE_LINEAR, abi.JMM_VOLSCHED_RANDOM, 0.5),
    # the reference's own volume move: linear dL, drawn with P = 1/(N+1)
    (abi.JMM_NPT, abi.JMM_VOLMOVE_LINEAR, abi.JMM_VOLSCHED_RANDOM, 0.5),
    # the batched NPT workload's: ln L steps of 0.01, one closing every sweep
    (abi.JMM_NPT, abi.JMM_VOLMOVE_LNL, abi.JMM_VOLSCHED_SWEEP, 0.01),
])
def test_batched_chain_samples_the_reference_ensemble(ensemble, vol_move, schedule, vol_step,
                                                      fp64):
    """fp64: the batched FP64 restatement; fp32_exact_kernel: its FP32 mode,
    which the EXACT GPU kernel equals bit for bit."""
    l0 = N / 0.6 if ensemble == abi.JMM_NLT else float(N)
    pe, pl = plain_replicas(ensemble, l0, 0.5)
    be, bl = batch_replicas(ensemble, l0, vol_step, vol_move, schedule, fp64)
    d, sem = agree(pe, be)
    print(f"<E>: reference algorithm {pe.mean():.4f}, batched {be.mean():.4f}, "
          f"diff {d:.4f}, standard error {sem:.4f}")
    assert d < 4 * sem, (pe.mean(), be.mean(), sem)
    if ensemble == abi.JMM_NPT:
        d, sem = agree(pl, bl)
        print(f"<L>: reference algorithm {pl.mean():.4f}, batched {bl.mean():.4f}, "
              f"diff {d:.4f}, standard error {sem:.4f}")
        assert d < 4 * sem, (pl.mean(), bl.mean(), sem)
