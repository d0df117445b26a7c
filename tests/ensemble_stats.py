"""Ensemble statistics for the parity tests: standard errors of replica
averages and the z / chi-square comparison of two samplers.

Test infrastructure.  Two error estimates are formed for every average:

* replicas: R independent chains, each averaged over its production run;
  the standard error of the pooled mean is std(replica means, ddof=1)/sqrt(R)
  (each replica's mean carries its own autocorrelation, so nothing about the
  correlation time is assumed).  A non-linear average (Var L = <L^2> - <L>^2
  from pooled moments) takes its error from the jackknife over replicas.
* blocking, the reference's estimator (scripts/Analyze_A_SD.py:155-209): a
  run's samples cut into numBlocks blocks of blockSize samples, the standard
  error std(block means)/sqrt(numBlocks) with numpy's default ddof = 0.  It is
  applied to each replica's chunk averages and combined over the replicas;
  it is reported beside the replica error as a cross-check.
"""
import math

import numpy as np


def block_sem(x, block):
    """Analyze_A_SD.py's estimator at one block size (in samples of x)."""
    x = np.asarray(x, dtype=np.float64)
    nb = len(x) // block
    if nb < 2:
        raise ValueError("fewer than two blocks")
    means = x[:nb * block].reshape(nb, block).mean(axis=1)
    return float(np.std(means) / math.sqrt(nb))


def blocking_sem(x, n_blocks=10):
    """The blocking error of one run's mean with blocks sized so that the run
    holds n_blocks of them (the plateau region of Analyze_A_SD.py's scan for
    runs many correlation times long)."""
    return block_sem(x, max(1, len(x) // n_blocks))


def replica_mean_se(v):
    v = np.asarray(v, dtype=np.float64)
    return float(v.mean()), float(v.std(ddof=1) / math.sqrt(len(v)))


def pooled_variance(m1, m2, w=None):
    """<x^2> - <x>^2 from per-replica first and second moments (equal weights
    unless w is given)."""
    m1, m2 = np.asarray(m1, dtype=np.float64), np.asarray(m2, dtype=np.float64)
    w = np.ones_like(m1) if w is None else np.asarray(w, dtype=np.float64)
    a = np.sum(w * m1) / np.sum(w)
    b = np.sum(w * m2) / np.sum(w)
    return float(b - a * a)


def jackknife(fn, *arrays):
    """Value and jackknife standard error of fn over replicas (leave one out)."""
    arrays = [np.asarray(a, dtype=np.float64) for a in arrays]
    r = len(arrays[0])
    full = fn(*arrays)
    loo = np.array([fn(*[np.delete(a, k) for a in arrays]) for k in range(r)])
    se = math.sqrt((r - 1) / r * np.sum((loo - loo.mean()) ** 2))
    return float(full), float(se)


def observable(name, reps):
    """(value, replica standard error) of one observable from a replica
    table {"u": [...], "rho": [...], "l": [...], "l2": [...], "e2": [...]}."""
    if name == "var_l":
        return jackknife(pooled_variance, reps["l"], reps["l2"])
    if name == "var_u":  # per particle: (<E^2> - <E>^2) / N, from u = E/N, e2 = <E^2>
        n = float(reps["n"])
        return jackknife(lambda u, e2: pooled_variance(u * n, e2) / n, reps["u"], reps["e2"])
    return replica_mean_se(reps[name])


def compare(a, b, observables):
    """Rows (observable, value a, se a, value b, se b, z) of two replica tables."""
    rows = []
    for name in observables:
        va, sa = observable(name, a)
        vb, sb = observable(name, b)
        rows.append((name, va, sa, vb, sb, (va - vb) / math.sqrt(sa * sa + sb * sb)))
    return rows


def chi2_pvalue(zs):
    """Upper-tail probability of sum z^2 with len(zs) degrees of freedom."""
    from scipy.stats import chi2
    zs = np.asarray(zs, dtype=np.float64)
    return float(chi2.sf(np.sum(zs * zs), len(zs)))
