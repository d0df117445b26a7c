"""The ensemble fixture (tests/golden/ensemble_states.json) on the CPU.

* The two FP64 CPU samplers of the fixture agree on the batched NPT
  workload's states: the reference's move loop (linear dL moves drawn with
  probability 1/(N+1) per step, all partners) and the batched chain's FP64
  restatement (ln L moves closing every sweep, index window), on <U>/N,
  <rho> and Var(L) -- the batched algorithm samples the reference's ensemble
  at N = 256 over T x P in {0.5, 1, 2}^2.
* The fixture is the restatement's own output: one state regenerated from
  the committed generator equals it replica for replica.
* The reference's blocking error estimate (scripts/Analyze_A_SD.py:155-209,
  restated in tests/ensemble_stats.py) of each replica mean, with ten blocks
  of 800 sweeps, comes out below the spread of the independent replicas
  (0.5 - 1.0 of it): the box length decorrelates over times comparable with
  a block, which blocks of that size do not resolve.  The z tests therefore
  use the replica spread, which assumes nothing about correlation times.
"""
import json
import math
import os
import sys

import numpy as np
import pytest

from tests import ensemble_stats as es

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "ensemble_states.json")


@pytest.fixture(scope="module")
def fixture():
    with open(FIXTURE) as f:
        return json.load(f)


def test_block_sem_restates_the_reference_estimator():
    """std(block means) / sqrt(numBlocks), numpy's ddof = 0, whole blocks only."""
    x = np.arange(10, dtype=np.float64)
    means = np.array([1.0, 4.0, 7.0])  # blocks of 3; the tenth sample is left out
    assert es.block_sem(x, 3) == pytest.approx(np.std(means) / math.sqrt(3))
    with pytest.raises(ValueError):
        es.block_sem(x, 6)


def test_jackknife_of_a_mean_is_its_standard_error():
    rng = np.random.default_rng(3)
    v = rng.normal(size=40)
    val, se = es.jackknife(lambda a: float(np.mean(a)), v)
    assert val == pytest.approx(v.mean())
    assert se == pytest.approx(v.std(ddof=1) / math.sqrt(len(v)))


def test_cpu_samplers_agree_on_the_npt_grid(fixture):
    rows = []
    for st in fixture["npt"]:
        rows += es.compare(st["reference_algorithm"], st["batched_fp64"], ("u", "rho", "var_l"))
    zs = [r[5] for r in rows]
    p = es.chi2_pvalue(zs)
    print(f"reference algorithm vs batched FP64: chi2 {np.sum(np.square(zs)):.1f} over {len(zs)}, "
          f"p = {p:.3f}, max |z| = {max(abs(z) for z in zs):.2f}")
    assert max(abs(z) for z in zs) <= 3.0
    assert p >= 1e-3


def test_blocking_errors_against_replica_spread(fixture):
    """Per state and sampler, the blocking error of <U>/N, <rho> and <L>
    combined over the replicas lies between 0.4 and 1.25 of the replicas'
    spread: never much above it, and below it where a block is not many
    correlation times long."""
    ratios = []
    for st in fixture["npt"]:
        for sampler in ("reference_algorithm", "batched_fp64"):
            t = st[sampler]
            for k in ("u", "rho", "l"):
                _, se = es.replica_mean_se(t[k])
                bse = math.sqrt(np.sum(np.square(t["bsem_" + k]))) / len(t[k])
                ratios.append(bse / se)
    ratios = np.array(ratios)
    print(f"blocking / replica error: median {np.median(ratios):.2f}, "
          f"range {ratios.min():.2f} - {ratios.max():.2f}")
    assert np.all((ratios > 0.4) & (ratios < 1.25))


def test_fixture_is_the_generators_output(fixture):
    """One NVT state of the batched FP64 restatement regenerated (3 s)."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_ensemble
    k = len(fixture["nvt"]) - 1
    kind, idx, table = make_ensemble.batch_task("nvt", k, tuple(fixture["protocol"]["nvt_states"][k]))
    ref = fixture["nvt"][k]["batched_fp64"]
    for key in ("u", "e2", "l", "l2", "rho"):
        np.testing.assert_allclose(table[key], ref[key], rtol=1e-12, atol=0)
