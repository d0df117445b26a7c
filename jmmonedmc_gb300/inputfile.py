"""The reference's INPUT keyword file, read with readInput's rules.

Restates src/readInput.cpp:8-262: one keyword and its value(s) per line,
tokens split on ``[``, `` ``, tab, newline and ``]``; numeric values go
through strtod and are truncated to integers where the reference does so;
``RELAX`` sets the flag whatever follows; an unknown ``POT`` falls back to
``LJ`` (no cut-off) and an unknown ``ENSEMBLE`` to ``NPT``; a ``POT`` line
without a cut-off means an infinite one.  Two deliberate differences: blank
lines are skipped (the reference dereferences a null token on them), and a
keyword the reference would leave uninitialised is reported as missing by
``to_params`` instead of being read as garbage.
"""
import math
import re

from . import abi

_SPLIT = re.compile(r"[\[ \t\n\]]+")

KEYS_FLOAT = {"P": "P", "L": "L", "T": "T", "MAXSTEP": "MAXSTEP", "MAXDV": "MAXDV",
              "RBW": "RBW", "GBW": "GBW", "GSW": "GSW"}
KEYS_INT = {"N", "NBN", "NUMSTEPS", "CPI", "TPI", "GPI", "RHOPI", "RHONB", "GNB",
            "GNS", "SEED", "ENGCHECK", "DADJ", "VADJ"}
POTENTIALS = {"LJcut": abi.JMM_POT_LJCUT, "LJ": abi.JMM_POT_LJ,
              "HARMONIC": abi.JMM_POT_HARMONIC}


_HEX = re.compile(r"\s*([-+]?)0[xX]([0-9a-fA-F]+\.?[0-9a-fA-F]*|\.[0-9a-fA-F]+)([pP][-+]?\d+)?")
_DEC = re.compile(r"\s*[-+]?(\d+\.?\d*([eE][-+]?\d+)?|\.\d+([eE][-+]?\d+)?|inf(inity)?|nan)",
                  re.IGNORECASE)


def _strtod(tok):
    """C strtod on the longest valid prefix: decimal, hexadecimal (0x, with an
    optional binary exponent), inf/infinity, nan; 0.0 when none."""
    m = _HEX.match(tok)
    if m:
        return float.fromhex(m.group(1) + "0x" + m.group(2) + (m.group(3) or ""))
    m = _DEC.match(tok)
    return float(m.group(0)) if m else 0.0


def parse_text(text):
    """Keyword dict with readInput's defaults (ENSEMBLE NPT, RESTART false)."""
    kw = {"ENSEMBLE": "NPT", "RESTART": False, "RELAX": 0, "COMPUTE": [], "UNKNOWN": []}
    for line in text.splitlines():
        toks = [t for t in _SPLIT.split(line) if t]
        if not toks:
            continue
        key = toks[0]
        if key == "RESTART":
            kw["RESTART"] = not (len(toks) > 1 and toks[1] in ("FALSE", "False", "false"))
        elif key in KEYS_INT:
            kw[key] = int(_strtod(toks[1])) if len(toks) > 1 else 0
        elif key in KEYS_FLOAT:
            kw[key] = _strtod(toks[1]) if len(toks) > 1 else 0.0
        elif key == "POT":
            name = toks[1] if len(toks) > 1 else ""
            if name not in POTENTIALS:
                name = "LJ"
            kw["POT"] = name
            kw["CUTOFF"] = _strtod(toks[2]) if len(toks) > 2 else math.inf
        elif key == "RELAX":
            kw["RELAX"] = 1
        elif key == "ENSEMBLE":
            name = toks[1] if len(toks) > 1 else ""
            kw["ENSEMBLE"] = name if name in ("NPT", "NLT") else "NPT"
        elif key in ("COMPUTE", "compute"):
            kw["COMPUTE"].append(toks[1:])
        else:
            kw["UNKNOWN"].append(key)
    return kw


def parse_file(path):
    with open(path) as f:
        return parse_text(f.read())


def to_params(kw):
    """abi.Params for the move loop from a parsed INPUT."""
    need = ["N", "T", "POT", "NBN", "MAXSTEP", "SEED"]
    if kw["ENSEMBLE"] == "NPT":
        need += ["P", "MAXDV"]
    else:
        need += ["L"]
    missing = [k for k in need if k not in kw]
    if missing:
        raise ValueError(f"INPUT lacks {missing}: the reference leaves them uninitialised")
    pot = POTENTIALS[kw["POT"]]
    return abi.make_params(
        n=kw["N"],
        ensemble=abi.JMM_NPT if kw["ENSEMBLE"] == "NPT" else abi.JMM_NLT,
        potential=pot,
        p=kw.get("P", 0.0),
        l=kw.get("L", float(kw["N"])),
        t=kw["T"],
        cutoff=kw.get("CUTOFF", math.inf),
        nbn=kw["NBN"],
        max_step=kw["MAXSTEP"],
        max_dl=kw.get("MAXDV", 0.0),
        seed=kw["SEED"],
        eci=kw.get("ENGCHECK", 0),
    )
