"""Loading of the golden fixtures and a driver-shaped runner used by the
parity tests (test infrastructure).

``run_like_driver`` calls a chain object (the CUDA PlainChain or the
oracle's OraclePlain) in the order of the reference driver
(src/Main.cpp:66-180): fad(0, 0.5), relaxVolume when RELAX is set (NPT),
updateThermo + printThermo at step 0, then steps with printThermo every TPI
steps (and the rho / g prints, and relaxVolume every 10000 steps), and
rebuilds the text of thermo.dat.mcs (and of the histogram files) from the
accumulators.
"""
import json
import math
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


class Adjuster:
    """maxDisAdjust / maxDVAdjust (src/jmmMCState.cpp:2100-2139): Swendsen's
    rescale of the step toward half acceptance from the cumulative counts,
    in the reference's operand order; the volume one only when new volume
    trials have been made since its last change (its static counter)."""

    def __init__(self, kw):
        self.max_step = float(kw["MAXSTEP"])
        self.max_dl = float(kw["MAXDV"])
        self.n = int(kw["N"])
        self.v_seen = 0

    def displacement(self, chain):
        st = chain.state()
        actual = float(st.d_acc[0]) / (st.d_acc[0] + st.d_acc[1])
        ms = self.max_step * math.log(0.672924 * 0.5 + 0.0644284) / math.log(
            0.672924 * (actual + 0.0644284))
        self.max_step = 0.002 if ms < 0.002 else (0.5 if ms > 0.5 else ms)
        chain.set_step_sizes(self.max_step, self.max_dl)

    def volume(self, chain):
        st = chain.state()
        tot = st.v_acc[0] + st.v_acc[1]
        if tot - self.v_seen <= 0:
            return
        self.v_seen = tot
        actual = float(st.v_acc[0]) / tot
        md = self.max_dl * math.log(0.672924 * 0.5 + 0.0644284) / math.log(
            0.672924 * (actual + 0.0644284))
        if md < 0.002 * self.n:
            md = 0.002 * self.n
        elif md > 0.10 * self.n:
            md = 0.50 * self.n
        self.max_dl = md
        chain.set_step_sizes(self.max_step, self.max_dl)


def run_like_driver(chain, kw, histograms=False):
    """Returns (per-step log, thermo file text), and with histograms=True
    also {file name: text} of rho.dat.mcs and g<k>.dat.mcs (the histograms
    are set up from the created chain, as setupMCS does before fad)."""
    tpi, rhopi, gpi = kw["TPI"], kw["RHOPI"], kw["GPI"]
    dadj, vadj = kw["DADJ"], kw["VADJ"]
    nsteps = kw["NUMSTEPS"]
    relax = bool(kw.get("RELAX")) and kw["ENSEMBLE"] == "NPT"  # setupMCS drops it for NLT
    adjust = Adjuster(kw)
    files = {}
    if histograms:
        chain.histograms(kw["RHONB"], kw["RBW"], kw["GNS"], kw["GSW"], kw["GNB"], kw["GBW"])
    chain.fad(0, 0.5)
    if relax:
        chain.relax_volume()
    chain.update_thermo()
    st = chain.state()
    first = (0 - U64) % (1 << 64)  # the reference's "last print" starts at -1
    text = [thermo.HEADER, thermo.thermo_line(0, list(st.thermo), first)]
    chain.reset_thermo()
    if histograms:
        rho = [thermo.rho_line(0, chain.take_rho(), first, kw["RBW"])]
        gtx = [[thermo.g_line(0, row, first, kw["GSW"], kw["GBW"])] for row in chain.take_g()]
    sltp = slrho = slg = 0
    logs = [None]
    sn = 0
    while sn < nsteps:
        nxt = min(nsteps, (sn // tpi + 1) * tpi)
        if histograms:
            nxt = min(nxt, (sn // rhopi + 1) * rhopi, (sn // gpi + 1) * gpi)
        if relax:
            nxt = min(nxt, (sn // 10000 + 1) * 10000)
        nxt = min(nxt, (sn // dadj + 1) * dadj, (sn // vadj + 1) * vadj)
        logs.append(chain.steps(nxt - sn, log=True))
        sn = nxt
        if sn % tpi == 0:
            st = chain.state()
            text.append(thermo.thermo_line(sn, list(st.thermo), sn - sltp))
            chain.reset_thermo()
            sltp = sn
        if histograms and sn % rhopi == 0:
            rho.append(thermo.rho_line(sn, chain.take_rho(), sn - slrho, kw["RBW"]))
            slrho = sn
        if sn % dadj == 0:
            adjust.displacement(chain)
        if sn % vadj == 0:
            adjust.volume(chain)
        if histograms and sn % gpi == 0:
            for k, row in enumerate(chain.take_g()):
                gtx[k].append(thermo.g_line(sn, row, sn - slg, kw["GSW"], kw["GBW"]))
            slg = sn
        if relax and sn % 10000 == 0 and sn < 1000000:  # src/Main.cpp:173-176
            chain.relax_volume()
    if histograms:
        files["rho.dat.mcs"] = "".join(rho)
        for k, lines in enumerate(gtx):
            files[f"g{k}.dat.mcs"] = "".join(lines)
        return np.concatenate(logs[1:]), "".join(text), files
    return np.concatenate(logs[1:]), "".join(text)


def reference_histogram_files(kw, ref):
    """{file name: text} of the reference's rho.dat.mcs and g<k>.dat.mcs."""
    out = {"rho.dat.mcs": str(ref["rho_file"])}
    for k in range(kw["GNS"]):
        out[f"g{k}.dat.mcs"] = str(ref["g_files"][k])
    return out


def unrelaxed_steps(kw, n):
    """Mask of steps 1..n whose per-step record is not followed by a
    relaxVolume (RELAX, NPT: every 10000 steps below 10^6)."""
    sn = np.arange(1, n + 1)
    if kw.get("RELAX") and kw["ENSEMBLE"] == "NPT":
        return ~((sn % 10000 == 0) & (sn < 1000000))
    return np.ones(n, dtype=bool)


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)
