"""The plain form's pair functions (oracle/plain_oracle.c) against the
reference's own phiLJcut, phiLJinfcutoff and phiHarmoniccut (src/pot.cpp:19-141,
run through oracle/pot_dump), bit for bit on all nine outputs: r over
0.8-1.2 and beyond, signed separations (the reference evaluates the signed
stored separation), one ulp either side of the cut-off, the virial switch.
Skipped where the reference's sources are absent."""
import os
import subprocess

import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from tests import oracle_lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = oracle_lib.reference_sources() or ""
DUMP = os.path.join(REPO, "oracle", "_ref", "pot_dump")


@pytest.fixture(scope="module")
def reference_phi():
    if not os.path.isdir(REF_SRC):
        pytest.skip("the reference's sources are not present")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "_ref/pot_dump",
                    f"REF_SRC={REF_SRC}"], check=True)

    def run(cases):
        text = "".join(f"{p} {d!r} {cut!r} {v} {l!r}\n" for p, d, cut, v, l in cases)
        out = subprocess.run([DUMP], input=text, capture_output=True, text=True, check=True,
                             timeout=60).stdout.splitlines()
        assert len(out) == len(cases)
        return [np.array([float.fromhex(t) for t in line.split()]) for line in out]

    return run


def separations(cut):
    core = np.linspace(0.8, 1.2, 41)
    edge = [cut, np.nextafter(cut, 0.0), np.nextafter(cut, np.inf)]
    far = [0.5, 1.5, 2.0, 2.9, 3.5, 10.0, 50.0]
    d = np.concatenate([core, edge, far])
    return [float(x) for x in np.concatenate([d, -d])]


def compare(reference_phi, cases):
    want = reference_phi(cases)
    for (p, d, cut, v, l), w in zip(cases, want):
        got = oracle_lib.phi(p, d, cut, bool(v), l)
        assert np.array_equal(got.view(np.uint64), w.view(np.uint64)), (p, d, cut, v, got, w)


@pytest.mark.parametrize("cut", [3.0, 2.5])
@pytest.mark.parametrize("virial", [0, 1])
def test_ljcut_matches_reference(reference_phi, cut, virial):
    compare(reference_phi, [(abi.JMM_POT_LJCUT, d, cut, virial, 10.0) for d in separations(cut)])


@pytest.mark.parametrize("virial", [0, 1])
def test_lj_without_cutoff_matches_reference(reference_phi, virial):
    compare(reference_phi, [(abi.JMM_POT_LJ, d, 3.0, virial, 10.0) for d in separations(3.0)])


def test_harmonic_matches_reference(reference_phi):
    cut = 1.5
    ds = [-0.1, 0.0, 0.3, 0.9, 1.0, 1.2, float(np.nextafter(cut, 0.0)), cut,
          float(np.nextafter(cut, np.inf)), 2.0]
    compare(reference_phi, [(abi.JMM_POT_HARMONIC, d, cut, 1, l) for d in ds
                            for l in (10.0, 106.66666666666667)])


def test_random_separations_match_reference(reference_phi):
    """3000 seeded separations, log-uniform over 0.3-30 with either sign,
    random cut-offs, all three functions, bit for bit."""
    rng = np.random.default_rng(11)
    cases = []
    for _ in range(3000):
        d = float(np.exp(rng.uniform(np.log(0.3), np.log(30.0))))
        d = -d if rng.random() < 0.3 else d
        cut = float(rng.uniform(1.0, 5.0))
        pot = int(rng.choice([abi.JMM_POT_LJCUT, abi.JMM_POT_LJ, abi.JMM_POT_HARMONIC]))
        virial = 1 if pot == abi.JMM_POT_HARMONIC else int(rng.integers(0, 2))
        cases.append((pot, d, cut, virial, float(rng.uniform(5.0, 500.0))))
    compare(reference_phi, cases)
