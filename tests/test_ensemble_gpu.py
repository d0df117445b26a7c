"""Ensemble parity of the production batched chains (FAST precision) with the
FP64 CPU reference, on the batched NPT workload's own states.

The GPU runs the workload's chains (N = 256, LJ 12-6 truncated at 3, hard
walls, displacements up to 0.3, ln L steps of 0.01 closing every sweep, from
the lattice at density 0.6) in the benchmark's launch shape (4 lanes x 8
steps per round, window 4) on a grid of T x P in {0.5, 1, 2}^2, 128 replicas
per state, and compares with the fixture tests/golden/ensemble_states.json
(tests/golden/make_ensemble.py):

* the reference's move loop (FP64, all partners, linear dL volume moves
  drawn with probability 1/(N+1) per step; oracle/plain_oracle.c replays the
  reference build bit for bit), 24 replicas per state;
* the batched chain's FP64 restatement with the workload's own moves, 48
  replicas per state.

Observables: <U>/N, <rho> = <N/L> and Var(L) = <L^2> - <L>^2, each with its
standard error from independent replicas (Var L by the jackknife over
replicas; tests/ensemble_stats.py).  Pass rule, per CPU sampler: no |z| above
3 and the chi-square of all 27 z values above the 0.1 % tail.  The uneven
batch's soft-sphere and Gaussian-core classes are checked the same way (NVT,
<U>/N and Var(U)/N) against the FP64 restatement.
"""
import json
import os

import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.batch import ChainBatch
from tests import ensemble_stats as es

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                       "ensemble_states.json")
REPLICAS = 128
Z_MAX = 3.0
P_MIN = 1e-3


@pytest.fixture(scope="module")
def fixture():
    with open(FIXTURE) as f:
        return json.load(f)


def _tables(res, n_states, n):
    """Per state, the replica table of a batch laid out state after state."""
    s = res["samples"].astype(np.float64)
    out = []
    for k in range(n_states):
        sl = slice(k * REPLICAS, (k + 1) * REPLICAS)
        out.append({"n": n, "u": res["sum_e"][sl] / s[sl] / n, "e2": res["sum_e2"][sl] / s[sl],
                    "l": res["sum_l"][sl] / s[sl], "l2": res["sum_l2"][sl] / s[sl],
                    "rho": res["sum_rho"][sl] / s[sl]})
    return out


def _judge(rows, label):
    zs = [r[5] for r in rows]
    p = es.chi2_pvalue(zs)
    worst = max(abs(z) for z in zs)
    print(f"{label}: chi2 = {np.sum(np.square(zs)):.1f} over {len(zs)} (p = {p:.3f}), "
          f"max |z| = {worst:.2f}")
    assert worst <= Z_MAX, (label, worst)
    assert p >= P_MIN, (label, p)


def test_batched_npt_workload_matches_fp64_reference(gpu, fixture):
    proto = fixture["protocol"]["npt"]
    states = fixture["protocol"]["npt_states"]
    n = proto["n"]
    chains = [abi.make_chain(n, potential=abi.JMM_POT_LJCUT, ensemble=abi.JMM_NPT,
                             cutoff=proto["cutoff"], t=t, p=p, rho=proto["rho0"],
                             max_step=proto["max_step"], vol_step=proto["vol_step"])
              for t, p in states for _ in range(REPLICAS)]
    cfg = abi.make_batch_config(seed=2026, vol_move=abi.JMM_VOLMOVE_LNL,
                                vol_schedule=abi.JMM_VOLSCHED_SWEEP, precision=abi.JMM_PREC_FAST,
                                lanes_per_chain=4, steps_per_round=8, chains_per_block=4,
                                window=4)
    with ChainBatch(cfg, chains) as b:
        b.run(proto["equil"])
        b.reset_stats()
        b.run(proto["prod"])
        res = b.results()
    assert not np.any(res["error"])
    gpu_tables = _tables(res, len(states), n)
    obs = ("u", "rho", "var_l")
    for sampler in ("reference_algorithm", "batched_fp64"):
        rows = []
        print(f"\nGPU FAST vs {sampler}: state, observable, GPU (se), CPU (se), z")
        for (t, p), g, st in zip(states, gpu_tables, fixture["npt"]):
            for r in es.compare(g, st[sampler], obs):
                rows.append(r)
                print(f"  T={t} P={p} {r[0]:6s} {r[1]:.6g} ({r[2]:.2g})  {r[3]:.6g} ({r[4]:.2g})"
                      f"  z={r[5]:+.2f}")
        _judge(rows, f"GPU FAST vs {sampler}")


def test_uneven_batch_classes_match_fp64(gpu, fixture):
    proto = fixture["protocol"]["nvt"]
    cut = {int(k): v for k, v in fixture["protocol"]["nvt_cutoff"].items()}
    states = fixture["protocol"]["nvt_states"]
    n = proto["n"]
    chains = [abi.make_chain(n, potential=pot, ensemble=abi.JMM_NLT, cutoff=cut[pot], t=t,
                             rho=rho, max_step=proto["max_step"])
              for pot, rho, t in states for _ in range(REPLICAS)]
    cfg = abi.make_batch_config(seed=2027, precision=abi.JMM_PREC_FAST, resum_sweeps=100)
    with ChainBatch(cfg, chains) as b:
        b.run(proto["equil"])
        b.reset_stats()
        b.run(proto["prod"])
        res = b.results()
    assert not np.any(res["error"])
    rows = []
    print("\nGPU FAST vs batched FP64 (NVT): potential, rho, T, observable, GPU (se), CPU (se), z")
    for (pot, rho, t), g, st in zip(states, _tables(res, len(states), n), fixture["nvt"]):
        for r in es.compare(g, st["batched_fp64"], ("u", "var_u")):
            rows.append(r)
            print(f"  pot={pot} rho={rho} T={t} {r[0]:6s} {r[1]:.6g} ({r[2]:.2g})  "
                  f"{r[3]:.6g} ({r[4]:.2g})  z={r[5]:+.2f}")
    _judge(rows, "GPU FAST vs batched FP64, soft sphere and Gaussian core")


def test_split_chains_match_fp64(gpu, fixture):
    """The same NVT states run split (split_n = 64: every N = 128 chain cut
    into domains of 32, alternating colours, sampled once per sweep) against
    the FP64 restatement's whole chains."""
    proto = fixture["protocol"]["nvt"]
    cut = {int(k): v for k, v in fixture["protocol"]["nvt_cutoff"].items()}
    states = fixture["protocol"]["nvt_states"]
    n = proto["n"]
    chains = [abi.make_chain(n, potential=pot, ensemble=abi.JMM_NLT, cutoff=cut[pot], t=t,
                             rho=rho, max_step=proto["max_step"])
              for pot, rho, t in states for _ in range(REPLICAS)]
    cfg = abi.make_batch_config(seed=2028, precision=abi.JMM_PREC_FAST, resum_sweeps=100,
                                split_n=64)
    with ChainBatch(cfg, chains) as b:
        b.run(proto["equil"])
        b.reset_stats()
        b.run(proto["prod"])
        res = b.results()
    assert not np.any(res["error"])
    assert np.all(res["samples"] == proto["prod"])  # one sample per sweep
    rows = []
    print("\nGPU FAST split vs batched FP64 (NVT): potential, rho, T, observable, GPU (se), "
          "CPU (se), z")
    for (pot, rho, t), g, st in zip(states, _tables(res, len(states), n), fixture["nvt"]):
        for r in es.compare(g, st["batched_fp64"], ("u", "var_u")):
            rows.append(r)
            print(f"  pot={pot} rho={rho} T={t} {r[0]:6s} {r[1]:.6g} ({r[2]:.2g})  "
                  f"{r[3]:.6g} ({r[4]:.2g})  z={r[5]:+.2f}")
    _judge(rows, "GPU FAST split chains vs batched FP64")
