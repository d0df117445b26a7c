"""Generate tests/golden/ensemble_states.json: FP64 CPU ensemble averages
that the batched GPU chains are compared against.

Test infrastructure.  Two CPU samplers, both FP64, run on seeded replicas:

* the reference's move loop (oracle/plain_oracle.c, which replays the
  reference build's trajectories bit for bit): per-pair state, all N-1
  partners per displacement, the O(N^2) fav volume move with linear dL drawn
  with probability 1/(N+1) per step (src/jmmMCState.cpp:1758-1811,
  :1160-1464, :2161-2293), starting from the lattice at L = N;
* the batched chain's FP64 restatement (oracle/batch_oracle.c, fp64 mode):
  the batched workload's own moves, ln L steps closing every sweep.

States: the batched NPT workload's chains (N = 256, LJ 12-6 with
eps = sigma = 1 truncated at 3, hard walls, displacements up to 0.3, ln L
steps of 0.01 per sweep from the lattice at density 0.6) on a grid of
T x P in {0.5, 1, 2}^2 that holds the workload's corners; and the uneven
batch's soft-sphere (cut-off 2.5) and Gaussian-core (cut-off 4) classes at
N = 128, density 0.3 and 0.9, T = 0.5 and 2 (NVT).  For each replica the
file keeps its production averages (E/N, rho = N/L, L, L^2, E^2) and the
blocking errors of E/N, rho and L from its chunk averages
(tests/ensemble_stats.py).  Run by hand (about 30 minutes on 8 cores):

    python tests/golden/make_ensemble.py [--jobs 8]

The large-chain workload's state (N = 2^20, LJ 12-6 truncated at 2.5,
density 0.7, T = 1.2, hard walls, displacements up to 0.3, lattice start)
is a section of its own, eight chains of the FP64 restatement (sequential
single-particle Metropolis with the cut-off window, the reference's move
loop cannot hold N = 2^20); each keeps its mean E/N and acceptance ratio
over the production sweeps (about 6 minutes on 8 cores):

    python tests/golden/make_ensemble.py --parts large
"""
import argparse
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ensemble_states.json")

NPT = dict(n=256, cutoff=3.0, max_step=0.3, vol_step=0.01, rho0=0.6, equil=4000, prod=8000,
           chunk=200, ref_replicas=24, batch_replicas=48, vol_frac=0.01)
NPT_STATES = [(t, p) for t in (0.5, 1.0, 2.0) for p in (0.5, 1.0, 2.0)]
NVT = dict(n=128, max_step=0.3, equil=1000, prod=4000, chunk=100, batch_replicas=48)
SOFT, GAUSS = 3, 4  # JMM_POT_SOFTSPHERE, JMM_POT_GAUSS
NVT_CUTOFF = {SOFT: 2.5, GAUSS: 4.0}
NVT_STATES = [(pot, rho, t) for pot in (SOFT, GAUSS) for rho in (0.3, 0.9) for t in (0.5, 2.0)]
LARGE = dict(n=1 << 20, rho=0.7, t=1.2, cutoff=2.5, max_step=0.3, equil=100, prod=300, chains=8)


def _setup():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)


def _replica_table(chunks, n):
    """chunks: list over chunks of dicts of per-replica chunk means (numpy
    arrays: e, e2, l, l2, rho).  Returns the replica table."""
    import numpy as np

    from tests.ensemble_stats import blocking_sem
    stack = {k: np.stack([c[k] for c in chunks], axis=1) for k in chunks[0]}  # (R, C)
    u = stack["e"] / n
    table = {"n": n, "u": u.mean(axis=1), "e2": stack["e2"].mean(axis=1),
             "l": stack["l"].mean(axis=1), "l2": stack["l2"].mean(axis=1),
             "rho": stack["rho"].mean(axis=1)}
    for k, series in (("u", u), ("rho", stack["rho"]), ("l", stack["l"])):
        table["bsem_" + k] = np.array([blocking_sem(row) for row in series])
    return {k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in table.items()}


def batch_task(kind, idx, state):
    """All replicas of one state through the batched FP64 restatement."""
    _setup()
    import numpy as np

    from jmmonedmc_gb300 import abi
    from tests import oracle_lib
    if kind == "npt":
        t, p = state
        q = NPT
        chains = [abi.make_chain(q["n"], potential=abi.JMM_POT_LJCUT, ensemble=abi.JMM_NPT,
                                 cutoff=q["cutoff"], t=t, p=p, rho=q["rho0"],
                                 max_step=q["max_step"], vol_step=q["vol_step"])
                  for _ in range(q["batch_replicas"])]
        cfg = abi.make_batch_config(seed=500 + idx, vol_move=abi.JMM_VOLMOVE_LNL,
                                    vol_schedule=abi.JMM_VOLSCHED_SWEEP,
                                    precision=abi.JMM_PREC_EXACT, resum_sweeps=100)
    else:
        pot, rho, t = state
        q = NVT
        chains = [abi.make_chain(q["n"], potential=pot, ensemble=abi.JMM_NLT,
                                 cutoff=NVT_CUTOFF[pot], t=t, rho=rho, max_step=q["max_step"])
                  for _ in range(q["batch_replicas"])]
        cfg = abi.make_batch_config(seed=700 + idx, precision=abi.JMM_PREC_EXACT,
                                    resum_sweeps=100)
    b = oracle_lib.OracleBatch(cfg, chains, fp64=True)
    b.run(q["equil"])
    prev = b.results()
    chunks = []
    for _ in range(q["prod"] // q["chunk"]):
        b.run(q["chunk"])
        cur = b.results()
        s = (cur["samples"] - prev["samples"]).astype(np.float64)
        d = {k: (cur["sum_" + k] - prev["sum_" + k]) / s for k in ("e", "e2", "l", "l2", "rho")}
        chunks.append(d)
        prev = cur
    if np.any(cur["error"]):
        raise RuntimeError(f"batched oracle flagged an error in state {state}")
    b.close()
    return kind, idx, _replica_table(chunks, q["n"])


def large_task(k):
    """One chain of the large-chain workload through the FP64 restatement."""
    _setup()
    from jmmonedmc_gb300 import abi
    from tests import oracle_lib
    q = LARGE
    chain = abi.make_chain(q["n"], potential=abi.JMM_POT_LJCUT, ensemble=abi.JMM_NLT,
                           cutoff=q["cutoff"], t=q["t"], rho=q["rho"], max_step=q["max_step"])
    cfg = abi.make_batch_config(seed=900 + k, precision=abi.JMM_PREC_EXACT, resum_sweeps=0)
    b = oracle_lib.OracleBatch(cfg, [chain], fp64=True)
    b.run(q["equil"])
    r0 = b.results()
    b.run(q["prod"])
    r1 = b.results()
    b.close()
    s = float(r1["samples"][0] - r0["samples"][0])
    u = float(r1["sum_e"][0] - r0["sum_e"][0]) / s / q["n"]
    acc = float(r1["disp_acc"][0] - r0["disp_acc"][0]) / float(r1["disp_att"][0] - r0["disp_att"][0])
    return k, u, acc


def plain_task(idx, r, t, p, max_dl):
    """One replica of the reference's move loop (FP64 restatement)."""
    _setup()
    import numpy as np

    from jmmonedmc_gb300 import abi
    from tests import oracle_lib
    q = NPT
    n = q["n"]
    sweep = n + 1  # Step draws the trial type over N + 1 (src/jmmMCState.cpp:405,1762)
    prm = abi.make_params(n=n, ensemble=abi.JMM_NPT, potential=abi.JMM_POT_LJCUT, p=p,
                          l=float(n), t=t, cutoff=q["cutoff"], max_step=q["max_step"],
                          max_dl=max_dl, seed=1000 + 100 * idx + r, eci=0)
    c = oracle_lib.OraclePlain(prm)
    c.fad()
    c.steps(q["equil"] * sweep)
    chunks = []
    steps = q["chunk"] * sweep
    for _ in range(q["prod"] // q["chunk"]):
        c.reset_thermo()
        c.steps(steps)
        th = np.array(c.state().thermo) / steps
        # accumulator order: rhoSysA, rhoSysSA, lA, lSA, EA, ESA, ...
        chunks.append({"e": th[4:5], "e2": th[5:6], "l": th[2:3], "l2": th[3:4],
                       "rho": th[0:1]})
    c.close()
    return idx, r, chunks


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--parts", default="grid,large",
                    help="grid (the NPT and NVT states), large (the large chains), or both; "
                         "a part not made keeps the file's existing section")
    args = ap.parse_args()
    parts = set(args.parts.split(","))
    _setup()
    import numpy as np
    t0 = time.time()
    ctx = mp.get_context("spawn")
    if "grid" not in parts:
        with open(OUT) as f:
            out = json.load(f)
        with ctx.Pool(args.jobs) as pool:
            res = pool.map(large_task, range(LARGE["chains"]))
        out["protocol"]["large"] = LARGE
        out["large"] = {"u": [u for _, u, _ in sorted(res)], "acc": [a for _, _, a in sorted(res)]}
        with open(OUT, "w") as f:
            json.dump(out, f, indent=None, separators=(",", ":"))
            f.write("\n")
        print(f"wrote the large section of {OUT} in {time.time() - t0:.0f} s")
        return
    out = {"protocol": {"npt": NPT, "npt_states": NPT_STATES, "nvt": NVT,
                        "nvt_cutoff": {str(k): v for k, v in NVT_CUTOFF.items()},
                        "nvt_states": NVT_STATES},
           "npt": [None] * len(NPT_STATES), "nvt": [None] * len(NVT_STATES)}
    with ctx.Pool(args.jobs) as pool:
        jobs = [pool.apply_async(batch_task, ("npt", k, s)) for k, s in enumerate(NPT_STATES)]
        jobs += [pool.apply_async(batch_task, ("nvt", k, s)) for k, s in enumerate(NVT_STATES)]
        for j in jobs:
            kind, k, table = j.get()
            if kind == "npt":
                t, p = NPT_STATES[k]
                mean_l = float(np.mean(table["l"]))
                out["npt"][k] = {"t": t, "p": p, "batched_fp64": table,
                                 "max_dl": NPT["vol_frac"] * mean_l}
            else:
                pot, rho, t = NVT_STATES[k]
                out["nvt"][k] = {"potential": pot, "rho": rho, "t": t, "batched_fp64": table}
        print(f"batched restatement done in {time.time() - t0:.0f} s", flush=True)
        pj = [pool.apply_async(plain_task, (k, r, s["t"], s["p"], s["max_dl"]))
              for k, s in enumerate(out["npt"]) for r in range(NPT["ref_replicas"])]
        per_state = {}
        for j in pj:
            k, r, chunks = j.get()
            per_state.setdefault(k, {})[r] = chunks
        for k, reps in per_state.items():
            order = [reps[r] for r in range(NPT["ref_replicas"])]
            merged = [{key: np.concatenate([rep[c][key] for rep in order])
                       for key in order[0][c]} for c in range(len(order[0]))]
            out["npt"][k]["reference_algorithm"] = _replica_table(merged, NPT["n"])
        if "large" in parts:
            res = pool.map(large_task, range(LARGE["chains"]))
            out["protocol"]["large"] = LARGE
            out["large"] = {"u": [u for _, u, _ in sorted(res)],
                            "acc": [a for _, _, a in sorted(res)]}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=None, separators=(",", ":"))
        f.write("\n")
    print(f"wrote {OUT} in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
