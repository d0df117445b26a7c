"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's move loop, compiled from its own sources with the
project's Philox stand-in for GSL (oracle/Makefile target ``ref``), on a set
of INPUT files, and stores per-step trajectories, final positions, thermo
accumulators and the reference's own output files as small compressed
fixtures.  It needs the reference tree, which the oracle's build recipe
(oracle/build_oracle.py: JMM_REF_SRC, or the checkout's usual place) finds,
and is run by hand:

    python tests/golden/make_golden.py

The fixtures are what the CPU and GPU parity tests compare against; nothing
at test time reads the reference tree.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(REPO, "oracle")
HARNESS = os.path.join(ORACLE, "_ref", "ref_harness")


def _recipe():
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_oracle",
                                                  os.path.join(ORACLE, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod

REF_STEP_DTYPE = np.dtype([
    ("sn", "<u8"), ("nm", "<u8"), ("rn", "<f8"), ("e", "<f8"), ("vir", "<f8"),
    ("hv", "<f8"), ("l", "<f8"), ("e12", "<f8"), ("e6", "<f8"), ("vir12", "<f8"),
    ("vir6", "<f8"), ("hv12", "<f8"), ("hv6", "<f8"), ("d_acc0", "<u8"),
    ("d_acc1", "<u8"), ("v_acc0", "<u8"), ("v_acc1", "<u8"),
])

# keyword -> value; every keyword is written because the reference leaves
# omitted ones uninitialised (src/readInput.cpp:38-57)
# histograms: 60 density bins of 2 sigma and 4 slices of 30 sigma, each with
# 20 separation bins of 0.2 sigma (x in +-60: the N = 256 box reaches beyond,
# so the range checks are exercised), printed every 250 / 400 steps
BASE = dict(ENSEMBLE="NLT", N=64, P=1.0, L=106.66666666666667, T=1.0,
            NUMSTEPS=3000, POT="LJcut 3.0", NBN=-1, MAXSTEP=0.3, MAXDV=0.5,
            CPI=1000, TPI=500, RBW=2.0, RHONB=60, RHOPI=250, GSW=30.0,
            GNS=4, GBW=0.2, GNB=20, GPI=400, SEED=1, ENGCHECK=500,
            DADJ=10**18, VADJ=10**18)

CASES = {
    # the CPU-runnable plain workload: NLT, N=64, rho=0.6, LJcut 3.0, T=1
    "nlt64_ljcut": dict(),
    # NPT with the full-energy volume move fav (src/jmmMCState.cpp:2161-2293)
    "npt64_ljcut": dict(ENSEMBLE="NPT", P=1.0, SEED=7, ENGCHECK=1000, MAXDV=0.5),
    # POT LJ with a neighbour-number limit: NPT volume move is fav
    "npt48_lj_nbn2": dict(ENSEMBLE="NPT", N=48, POT="LJ", NBN=2, SEED=11,
                          ENGCHECK=700, MAXDV=0.5),
    # HARMONIC with NBN 1, as in the reference's test/INPUTstd
    "npt10_harmonic_nbn1": dict(ENSEMBLE="NPT", N=10, P=0.7, T=0.4,
                                POT="HARMONIC", NBN=1, MAXSTEP=0.1, MAXDV=1.0,
                                SEED=125, ENGCHECK=1, NUMSTEPS=2000),
    # the per-chain size of the batched workload, NLT at rho = 0.6
    "nlt256_ljcut": dict(N=256, L=256 / 0.6, SEED=3, NUMSTEPS=2000,
                         ENGCHECK=1000, TPI=400, CPI=1000),
    # dense NPT start (L = N) with a wide volume step: many volume moves
    "npt32_ljcut_wide": dict(ENSEMBLE="NPT", N=32, P=2.0, T=1.5, MAXDV=2.0,
                             SEED=99, NUMSTEPS=4000, ENGCHECK=250),
    # maxDisAdjust / maxDVAdjust every 500 / 600 steps from a small step and a
    # wide volume step
    "npt48_ljcut_adjust": dict(ENSEMBLE="NPT", N=48, P=1.0, T=1.1, MAXSTEP=0.05, MAXDV=3.0,
                               SEED=57, NUMSTEPS=4000, ENGCHECK=800, DADJ=500, VADJ=600),
    # RELAX (as the reference's test/INPUT): relaxVolume after the step-0 fad
    # and again at step 10000
    "npt32_ljcut_relax": dict(ENSEMBLE="NPT", N=32, P=1.0, T=1.0, MAXDV=1.0, SEED=41,
                              NUMSTEPS=10000, ENGCHECK=1000, TPI=1000, RELAX=1),
}


def input_text(kw):
    lines = []
    for key in ("ENSEMBLE", "N", "P", "L", "T", "NUMSTEPS", "POT", "NBN",
                "MAXSTEP", "MAXDV", "CPI", "TPI", "RBW", "RHONB", "RHOPI",
                "GSW", "GNS", "GBW", "GNB", "GPI", "SEED", "ENGCHECK", "DADJ",
                "VADJ"):
        v = kw[key]
        if isinstance(v, float):
            v = repr(v)
        lines.append(f"{key:<10} {v}")
    if kw.get("RELAX"):
        lines.append("RELAX")
    return "\n".join(lines) + "\n"


def build_reference():
    if _recipe().build_reference_if_present() is None:
        sys.exit("make_golden: the reference tree is not present (set JMM_REF_SRC)")


def run_case(name, overrides):
    kw = dict(BASE)
    kw.update(overrides)
    text = input_text(kw)
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "INPUT"), "w") as f:
            f.write(text)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        out = subprocess.run([HARNESS, "steps.bin", "final.bin"], cwd=tmp, env=env,
                             check=True, capture_output=True, text=True)
        steps = np.fromfile(os.path.join(tmp, "steps.bin"), dtype=REF_STEP_DTYPE)
        raw = np.fromfile(os.path.join(tmp, "final.bin"), dtype="<u8", count=1)
        n = int(raw[0])
        fin = np.fromfile(os.path.join(tmp, "final.bin"), dtype="<f8")[1:]
        r_final, thermo = fin[:n], fin[n:n + 12]
        files = {}
        names = ["thermo.dat.mcs", "config.dat.mcs", "rho.dat.mcs"]
        names += [f"g{k}.dat.mcs" for k in range(kw["GNS"])]
        for fn in names:
            with open(os.path.join(tmp, fn)) as f:
                files[fn] = f.read()
    outcome = np.zeros(len(steps), dtype=np.int8)
    acc = (np.diff(steps["d_acc0"].astype(np.int64)) + np.diff(steps["v_acc0"].astype(np.int64)))
    outcome[1:] = acc
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        input=np.array(text),
        sn=steps["sn"].astype(np.uint32),
        nm=steps["nm"].astype(np.uint32),
        rn=steps["rn"],
        e=steps["e"], vir=steps["vir"], hv=steps["hv"], l=steps["l"],
        e12=steps["e12"], e6=steps["e6"],
        d_acc0=steps["d_acc0"].astype(np.uint32), d_acc1=steps["d_acc1"].astype(np.uint32),
        v_acc0=steps["v_acc0"].astype(np.uint32), v_acc1=steps["v_acc1"].astype(np.uint32),
        accepted=outcome,
        r_final=r_final, thermo_final=thermo,
        thermo_file=np.array(files["thermo.dat.mcs"]),
        config_file=np.array(files["config.dat.mcs"]),
        rho_file=np.array(files["rho.dat.mcs"]),
        g_files=np.array([files[f"g{k}.dat.mcs"] for k in range(kw["GNS"])]),
        stdout_tail=np.array("\n".join(out.stdout.splitlines()[-4:])),
    )
    return dict(name=name, input=kw, steps=len(steps) - 1)


# Restarts: a fresh run to NUMSTEPS, then the same INPUT with RESTART TRUE and
# a larger NUMSTEPS in the same directory (the reference resumes from the
# last complete frame of config.dat.mcs, src/jmmMCState.cpp:572-765).  The
# fixture holds both INPUT files and every output file after the restart.
RESTARTS = {
    "restart_nlt64": (dict(NUMSTEPS=2000), 4000),
    "restart_npt32": (dict(ENSEMBLE="NPT", N=32, P=1.5, T=1.2, MAXDV=1.0, SEED=23,
                           NUMSTEPS=3000, ENGCHECK=700), 5000),
}


def run_restart_case(name, overrides, numsteps2):
    kw = dict(BASE)
    kw.update(overrides)
    first = input_text(kw)
    second = "RESTART    TRUE\n" + input_text(dict(kw, NUMSTEPS=numsteps2))
    env = dict(os.environ, OMP_NUM_THREADS="1")
    with tempfile.TemporaryDirectory() as tmp:
        for text in (first, second):
            with open(os.path.join(tmp, "INPUT"), "w") as f:
                f.write(text)
            out = subprocess.run([HARNESS, "steps.bin", "final.bin"], cwd=tmp, env=env,
                                 check=True, capture_output=True, text=True)
        files = {}
        names = ["thermo.dat.mcs", "config.dat.mcs", "rho.dat.mcs"]
        names += [f"g{k}.dat.mcs" for k in range(kw["GNS"])]
        for fn in names:
            with open(os.path.join(tmp, fn)) as f:
                files[fn] = f.read()
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        input_first=np.array(first), input_restart=np.array(second),
        file_names=np.array(names), file_texts=np.array([files[fn] for fn in names]),
        stdout_tail=np.array("\n".join(out.stdout.splitlines()[-4:])),
    )
    return dict(name=name, input=kw, restart_numsteps=numsteps2)


def main():
    build_reference()
    index = [run_case(name, over) for name, over in CASES.items()]
    restarts = [run_restart_case(name, over, n2) for name, (over, n2) in RESTARTS.items()]
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(dict(generator="tests/golden/make_golden.py",
                       rng="Philox4x32-10, one block per step (oracle/philox.h)",
                       cases=index, restarts=restarts), f, indent=1)
    print("\n".join(f"{c['name']}: {c['steps']} steps" for c in index))
    print("\n".join(f"{c['name']}: restart to {c['restart_numsteps']}" for c in restarts))


if __name__ == "__main__":
    sys.exit(main())
