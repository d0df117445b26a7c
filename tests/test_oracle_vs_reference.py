"""The oracle (oracle/plain_oracle.c) against the reference itself.

The golden fixtures were produced by the reference's own move loop compiled
with the project's Philox stand-in for GSL (tests/golden/make_golden.py);
the restatement must reproduce every step bit for bit: trial type, trial
uniform, E/Vir/HV after the step, box length, acceptance counters, final
positions and the text of thermo.dat.mcs.
"""
import numpy as np
import pytest

from tests import golden_cases as gc
from tests import oracle_lib

CASES = gc.case_names()


@pytest.mark.parametrize("name", CASES)
def test_oracle_replays_reference(name):
    kw, params, ref = gc.load_case(name)
    chain = oracle_lib.OraclePlain(params)
    log, text = gc.run_like_driver(chain, kw)
    n = len(log)
    assert n == kw["NUMSTEPS"]
    harmonic = kw["POT"] == "HARMONIC"
    # step 0 is the driver's fad(0, 0.5)
    np.testing.assert_array_equal(log["nm"], ref["nm"][1:])
    np.testing.assert_array_equal(gc.bits(log["rn"]), gc.bits(ref["rn"][1:]))
    # a step of relaxVolume (RELAX, every 10000 steps) follows the step's own
    # record; the reference logs after it: compare the final state there
    keep = gc.unrelaxed_steps(kw, len(log))
    st_end = chain.state()
    for q, v in (("e", st_end.tot[0]), ("vir", st_end.tot[1]), ("l", st_end.l)):
        assert gc.bits(np.array([v]))[0] == gc.bits(ref[q][-1:])[0], q
    for q in ("e", "vir", "l") + (() if harmonic else ("hv",)):
        diff = np.nonzero((gc.bits(log[q]) != gc.bits(ref[q][1:])) & keep)[0]
        assert diff.size == 0, f"{q} differs first at step {diff[0] + 1}"
    acc = (log["outcome"] == 2).astype(np.int8)
    np.testing.assert_array_equal(acc, ref["accepted"][1:])
    st = chain.state()
    assert st.d_acc[0] == ref["d_acc0"][-1] and st.d_acc[1] == ref["d_acc1"][-1]
    assert st.v_acc[0] == ref["v_acc0"][-1] and st.v_acc[1] == ref["v_acc1"][-1]
    np.testing.assert_array_equal(gc.bits(chain.positions()), gc.bits(ref["r_final"]))
    ref_lines = str(ref["thermo_file"]).splitlines()
    our_lines = text.splitlines()
    assert len(our_lines) == len(ref_lines)
    for ours, theirs in zip(our_lines, ref_lines):
        if harmonic:  # HV columns are uninitialised memory in the reference
            ours, theirs = ours.split("\t")[:-2], theirs.split("\t")[:-2]
        assert ours == theirs


@pytest.mark.parametrize("name", CASES)
def test_oracle_histogram_files_equal_reference(name):
    """fgrho/ugrho/qagrho and printRho/printG: the rho.dat.mcs and g<k>.dat.mcs
    text equals the reference's, byte for byte (negative g counts, which the
    reference's stale counts after a fav volume move produce, included)."""
    kw, params, ref = gc.load_case(name)
    chain = oracle_lib.OraclePlain(params)
    _, _, files = gc.run_like_driver(chain, kw, histograms=True)
    theirs = gc.reference_histogram_files(kw, ref)
    assert sorted(files) == sorted(theirs)
    for fn, text in theirs.items():
        assert files[fn] == text, fn


def test_golden_step_zero_energy():
    """fad(0, 0.5) at set-up gives the full FP64 pair sum (src/Main.cpp:66-68)."""
    kw, params, ref = gc.load_case("nlt64_ljcut")
    chain = oracle_lib.OraclePlain(params)
    chain.fad(0, 0.5)
    st = chain.state()
    assert gc.bits(np.array([st.tot[0]]))[0] == gc.bits(ref["e"][:1])[0]
    assert st.d_acc[0] == 1  # the step-0 fad counts as an accepted displacement
