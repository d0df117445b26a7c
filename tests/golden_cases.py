"""Loading of the golden fixtures and a driver-shaped runner used by the
parity tests (test infrastructure).

``run_like_driver`` calls a chain object (the CUDA PlainChain or the
oracle's OraclePlain) in the order of the reference driver
(src/Main.cpp:66-180): fad(0, 0.5), updateThermo + printThermo at step 0,
then steps with printThermo every TPI steps, and rebuilds the text of
thermo.dat.mcs from the accumulators.
"""
import json
import os

import numpy as np

from jmmonedmc_gb300 import inputfile, thermo

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
U64 = (1 << 64) - 1


def case_names():
    with open(os.path.join(HERE, "index.json")) as f:
        return [c["name"] for c in json.load(f)["cases"]]


def load_case(name):
    z = np.load(os.path.join(HERE, name + ".npz"), allow_pickle=False)
    data = {k: z[k] for k in z.files}
    kw = inputfile.parse_text(str(data["input"]))
    return kw, inputfile.to_params(kw), data


def run_like_driver(chain, kw):
    """Returns (per-step log, thermo file text)."""
    tpi = kw["TPI"]
    nsteps = kw["NUMSTEPS"]
    chain.fad(0, 0.5)
    chain.update_thermo()
    st = chain.state()
    text = [thermo.HEADER, thermo.thermo_line(0, list(st.thermo), (0 - U64) % (1 << 64))]
    chain.reset_thermo()
    sltp = 0
    logs = [None]
    sn = 0
    while sn < nsteps:
        nxt = min(nsteps, (sn // tpi + 1) * tpi)
        logs.append(chain.steps(nxt - sn, log=True))
        sn = nxt
        if sn % tpi == 0:
            st = chain.state()
            text.append(thermo.thermo_line(sn, list(st.thermo), sn - sltp))
            chain.reset_thermo()
            sltp = sn
    return np.concatenate(logs[1:]), "".join(text)


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)
