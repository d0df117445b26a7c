"""The batched form's three potentials and their parameter derivatives in the
FP64 oracle, against closed forms summed over all pairs with numpy (CPU).

LJ 12-6 4 eps ((s/r)^12 - (s/r)^6), soft sphere eps (s/r)^12 and Gaussian
core eps exp(-(r/s)^2), each truncated (not shifted) at the absolute cut-off
rc; on a ring, the minimum image.  The derivatives are those of the gradient
kernel: dU/deps = U/eps, dU/dsigma, and dU/dL = sum r phi'(r) / L with every
position scaled with the box.  The oracle walks index neighbours only, and
this is an independent all-pairs sum, so the two agree only if the
neighbour walk finds every pair inside the cut-off."""
import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from tests import oracle_lib

EPS, SIGMA = 1.3, 0.9
POTENTIALS = [(abi.JMM_POT_LJCUT, 3.0), (abi.JMM_POT_SOFTSPHERE, 2.5), (abi.JMM_POT_GAUSS, 4.0)]


def pair_terms(pot, r):
    """phi(r), dphi/dsigma(r), r dphi/dr(r) at eps = EPS, sigma = SIGMA."""
    e, s = EPS, SIGMA
    if pot == abi.JMM_POT_LJCUT:
        s6 = (s / r) ** 6
        phi = 4 * e * (s6 * s6 - s6)
        dsig = 4 * e * (12 * s6 * s6 - 6 * s6) / s
        rdr = 4 * e * (-12 * s6 * s6 + 6 * s6)
    elif pot == abi.JMM_POT_SOFTSPHERE:
        s12 = (s / r) ** 12
        phi = e * s12
        dsig = 12 * e * s12 / s
        rdr = -12 * e * s12
    else:
        g = np.exp(-(r / s) ** 2)
        phi = e * g
        dsig = e * g * 2 * r * r / s ** 3
        rdr = -2 * e * g * (r / s) ** 2
    return phi, dsig, rdr


def closed_form(pot, rc, x, l, periodic):
    i, j = np.triu_indices(len(x), 1)
    d = np.abs(x[j] - x[i])
    if periodic:
        d = np.minimum(d, l - d)
    r = d[d <= rc]
    phi, dsig, rdr = pair_terms(pot, r)
    u = phi.sum()
    return np.array([u, u / EPS, dsig.sum(), rdr.sum() / l])


def configuration(rng, n, rho, jitter):
    l = n / rho
    x = ((np.arange(n) + 0.5) / n - 0.5) * l + rng.uniform(-jitter, jitter, n) / rho
    return np.sort(x), l


@pytest.mark.parametrize("pot,rc", POTENTIALS)
@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("n,rho", [(97, 0.7), (96, 0.3), (33, 1.1)])
def test_oracle_energy_and_gradient_match_closed_forms(pot, rc, periodic, n, rho):
    rng = np.random.default_rng(1000 * n + pot)
    for _ in range(5):
        x, l = configuration(rng, n, rho, 0.4)
        c = abi.make_chain(n, potential=pot, cutoff=rc, eps=EPS, sigma=SIGMA, l0=l)
        want = closed_form(pot, rc, x, l, periodic)
        u = oracle_lib.energy64(c, x, l, periodic)
        got = oracle_lib.energy_grad64(c, x, l, periodic)
        scale = np.maximum(np.abs(want), 1.0)
        assert abs(u - want[0]) <= 1e-11 * scale[0]
        np.testing.assert_array_less(np.abs(got - want), 1e-11 * scale)


@pytest.mark.parametrize("pot,rc", POTENTIALS)
def test_cutoff_is_inclusive_and_absolute(pot, rc):
    """A pair exactly at rc counts (d^2 <= rc^2, as phiLJcut's <=,
    src/pot.cpp:19-101); one just beyond does not; rc is not scaled by sigma."""
    for d, counted in [(rc, True), (rc * (1 + 1e-9), False), (0.5 * rc, True)]:
        x = np.array([0.0, d])
        c = abi.make_chain(2, potential=pot, cutoff=rc, eps=EPS, sigma=SIGMA, l0=10 * rc)
        u = oracle_lib.energy64(c, x, 10 * rc, False)
        want = pair_terms(pot, np.array([d]))[0][0] if counted else 0.0
        assert u == pytest.approx(want, rel=1e-14, abs=0.0)
