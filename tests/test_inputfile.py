"""The INPUT reader (jmmonedmc_gb300/inputfile.py) against the reference's own
readInput (src/readInput.cpp:8-262), run through oracle/input_dump on the same
files: every keyword the file names must come out with the same value
(strtod prefixes, truncation to integers, bracketed and tab-separated tokens,
unknown potentials and ensembles, RESTART spellings, repeated keywords,
unknown keywords).  Inputs on which the reference itself dereferences a null
token (blank lines, a keyword without a value) are left out; the parser's
handling of blank lines is a stated deviation.  Skipped where the
reference's sources are absent."""
import json
import math
import os
import subprocess

import numpy as np
import pytest

from jmmonedmc_gb300 import abi, inputfile
from tests import oracle_lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = oracle_lib.reference_sources() or ""
DUMP = os.path.join(REPO, "oracle", "_ref", "input_dump")
GOLDEN = os.path.join(REPO, "tests", "golden")

EDGE_CASES = {
    "prefixes_and_fallbacks": (
        "N 64.9\nNBN -1\nPOT Morse 2.0\nENSEMBLE NVT\nRESTART yes\nRELAX 0\n"
        "SEED 1e3\nMAXSTEP .3\nMAXDV 1.e-2\nT\t0.85\n[P] [1.25]\nCOMPUTE a b\n"),
    "hex_and_trailing_text": (
        "RESTART false\nN 0x40\nL 1e3x\nPOT LJcut\nENSEMBLE NLT\nT +2\n"
        "NUMSTEPS 1.5e4\nGNS 2.9\nGSW 30\nGNB 20\nGBW 0.2\nRHONB 60\nRBW 2.0\n"),
    "repeats_and_unknown_keys": (
        "RESTART False\nPOT HARMONIC 1.5 extra tokens\nP -0.5\nCPI 100\nTPI 10.9\n"
        "GPI 7\nRHOPI 8\nENGCHECK 64000\nDADJ 1e18\nVADJ 3\nFOO 1\nn 5\n"
        "ENSEMBLE NLTX\nN 10\nN 12\n"),
    "hex_float_inf_nan": (
        "RESTART FALSE\nPOT LJ 2.5\nL 0x1.8p3\nT inf\nMAXSTEP nan\nP -0x.8\n"
        "MAXDV 1e\nN 0x\n"),
    "spacing_and_long_keys": (
        "RESTART TRUE\nENSEMBLE NPT\nPOT LJcutX 3\nSEED 12345678901\n   N   7   \n"
        "ENGCHECKING 5\n[T]\t[1.5]\t\nNBN 3.99\n"),
    "computes_and_bare_relax": (
        "compute x\nCOMPUTE y z\nRELAX\nRESTART FALSE\nN 3"),
}


@pytest.fixture(scope="module")
def dump():
    if not os.path.isdir(REF_SRC):
        pytest.skip("the reference's sources are not present")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "_ref/input_dump",
                    f"REF_SRC={REF_SRC}"], check=True)
    return DUMP


def reference_read(dump, tmp_path, text):
    path = tmp_path / "INPUT"
    path.write_text(text)
    out = subprocess.run([dump, str(path)], capture_output=True, check=True,
                         timeout=30).stdout.decode("utf-8", "replace")
    fields = {}
    for line in out.split("@@ MCInput\n", 1)[1].splitlines():
        key, _, val = line.partition(" ")
        fields[key] = val
    return fields


def named_keywords(text):
    """First token of each line, split as readInput splits."""
    keys = set()
    for line in text.splitlines():
        toks = line.replace("[", " ").replace("]", " ").split()
        if toks:
            keys.add(toks[0])
    return keys


def same_float(a, b):
    return (math.isnan(a) and math.isnan(b)) or a == b


def check_against_reference(kw, ref, text):
    named = named_keywords(text)
    assert kw["RESTART"] == (ref["RESTART"] == "1")
    assert kw["ENSEMBLE"] == ref["ENSEMBLE"]
    assert len(kw["COMPUTE"]) == int(ref["COMPUTES"])
    for key in inputfile.KEYS_INT & named:
        assert kw[key] == int(ref[key]), key
    for key in set(inputfile.KEYS_FLOAT) & named:
        assert same_float(kw[key], float(ref[key])), key
    if "POT" in named:
        assert kw["POT"] == ref["POT"]
        assert same_float(kw["CUTOFF"], float(ref["CUTOFF"]))
    if "RELAX" in named:
        assert kw["RELAX"] == int(ref["RELAX"])


@pytest.mark.parametrize("name", sorted(EDGE_CASES))
def test_parser_matches_reference_readinput(dump, tmp_path, name):
    text = EDGE_CASES[name]
    check_against_reference(inputfile.parse_text(text), reference_read(dump, tmp_path, text),
                            text)


def golden_inputs():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        cases = json.load(f)["cases"]
    return sorted(c["name"] + ".npz" for c in cases)


@pytest.mark.parametrize("case", golden_inputs())
def test_golden_inputs_and_params_match_reference(dump, tmp_path, case):
    text = str(np.load(os.path.join(GOLDEN, case))["input"])
    kw = inputfile.parse_text(text)
    ref = reference_read(dump, tmp_path, text)
    check_against_reference(kw, ref, text)
    prm = inputfile.to_params(kw)
    assert prm.n == int(ref["N"]) and prm.t == float(ref["T"])
    assert prm.nbn == int(ref["NBN"]) and prm.seed == int(ref["SEED"])
    assert prm.max_step == float(ref["MAXSTEP"])
    assert prm.ensemble == (abi.JMM_NPT if ref["ENSEMBLE"] == "NPT" else abi.JMM_NLT)
    if ref["ENSEMBLE"] == "NPT":
        assert prm.p == float(ref["P"]) and prm.max_dl == float(ref["MAXDV"])
    else:
        assert prm.l == float(ref["L"])
    if ref["POT"] != "LJ":
        assert prm.cutoff == float(ref["CUTOFF"])
    else:
        assert math.isinf(prm.cutoff)
    if "ENGCHECK" in named_keywords(text):
        assert prm.eci == int(ref["ENGCHECK"])


def test_strtod_prefixes():
    """C strtod's longest-valid-prefix rule (no reference needed)."""
    s = inputfile._strtod
    assert s("1e3x") == 1000.0 and s(".5") == 0.5 and s("1.e-2") == 0.01
    assert s("0x40") == 64.0 and s("0x1.8p3") == 12.0 and s("-0x.8") == -0.5
    assert s("0x") == 0.0 and s("1e") == 1.0 and s("abc") == 0.0
    assert math.isinf(s("inf")) and math.isinf(s("-Infinity")) and math.isnan(s("nan"))


@pytest.mark.parametrize("drop, ensemble", [("N", "NPT"), ("SEED", "NPT"), ("P", "NPT"),
                                            ("MAXDV", "NPT"), ("L", "NLT"), ("POT", "NLT")])
def test_to_params_refuses_missing_keywords(drop, ensemble):
    """A keyword the move loop needs but the file omits is refused: the
    reference would read it from an uninitialised field."""
    lines = {"ENSEMBLE": ensemble, "N": "64", "P": "1.0", "L": "100.0", "T": "1.0",
             "POT": "LJcut 3.0", "NBN": "-1", "MAXSTEP": "0.3", "MAXDV": "0.5", "SEED": "1"}
    del lines[drop]
    kw = inputfile.parse_text("".join(f"{k} {v}\n" for k, v in lines.items()))
    with pytest.raises(ValueError, match=drop):
        inputfile.to_params(kw)


def _random_value(rng, integer, signed):
    """A value spelled as strtod reads it: decimal, exponent, hexadecimal,
    leading dot, trailing text.  Integer fields get no negative, huge or
    non-finite values (their conversion is undefined in the reference)."""
    mag = float(rng.choice([0.5, 3.0, 64.0, 1000.0])) * float(rng.random())
    if signed and rng.random() < 0.3:
        mag = -mag
    form = rng.integers(0, 5)
    if form == 0:
        return repr(round(mag, 6))
    if form == 1:
        return f"{mag:.3e}"
    if form == 2:
        return float(mag).hex() if not integer else hex(int(abs(mag)))
    if form == 3:
        return f"{mag:.4f}".replace("0.", ".", 1) if 0 <= mag < 1 else f"{mag:.2f}"
    return f"{mag:.3f}xyz"


def test_random_inputs_match_reference_readinput(dump, tmp_path):
    rng = np.random.default_rng(2024)
    keys_int = sorted(inputfile.KEYS_INT)
    keys_float = sorted(inputfile.KEYS_FLOAT)
    for trial in range(150):
        lines = []
        for _ in range(int(rng.integers(3, 14))):
            r = rng.random()
            if r < 0.4:
                k = str(rng.choice(keys_int))
                lines.append(f"{k} {_random_value(rng, True, k == 'NBN')}")
            elif r < 0.75:
                k = str(rng.choice(keys_float))
                lines.append(f"{k}\t{_random_value(rng, False, True)}")
            elif r < 0.82:
                pot = str(rng.choice(["LJcut", "LJ", "HARMONIC", "Morse"]))
                cut = f" {_random_value(rng, False, False)}" if rng.random() < 0.7 else ""
                lines.append(f"POT {pot}{cut}")
            elif r < 0.88:
                lines.append(f"ENSEMBLE {rng.choice(['NPT', 'NLT', 'NVT'])}")
            elif r < 0.94:
                lines.append(f"RESTART {rng.choice(['TRUE', 'FALSE', 'false', 'False', 'no'])}")
            elif r < 0.97:
                lines.append("RELAX")
            else:
                lines.append(f"[{rng.choice(keys_int)}] [{int(rng.integers(1, 500))}]")
        text = "\n".join(lines) + "\n"
        assert all(len(line) < 99 for line in lines)
        check_against_reference(inputfile.parse_text(text), reference_read(dump, tmp_path, text),
                                text)
