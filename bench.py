#!/usr/bin/env python
"""Benchmark: attempted Monte Carlo moves per second on one GB300.

Workload (the batched NPT configuration): 4096 independent chains of N = 256
Lennard-Jones 12-6 particles (eps = sigma = 1, cut-off 3 sigma, hard walls),
T log-spaced over 0.5-2.0, P uniform over 0.5-2.0 per chain, ln L volume
moves (delta = 0.01) closing every sweep of N displacement moves (maximum
displacement 0.3 sigma), starting from the lattice at rho = 0.6; FP32 pair
energies, FP64 totals and accumulators.  Inputs are synthetic and seeded.

One bench step = one CUDA-graph launch of the persistent chain kernel over
all chains for --sweeps-per-step sweeps (default 1000, so the default 10
timed steps are the configuration's full 10^4 sweeps).  Every attempted
move (displacement or volume) counts.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own algorithm for the same chains
(the plain FP64 single-chain loop: O(N) displacement with per-pair state,
O(N^2) volume move) on the host cores, one chain per core.
Prints exactly one JSON line (rank 0).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "attempted MC moves/s (batched chains, FP32 pairs / FP64 totals)"
UNIT = "moves/s"
FLOP_PER_PAIR = 9  # d, r^2, inv2 scale, inv6 (2), inv6-1, products (2), select
# FP32 FLOP of one pair energy by potential (each also one MUFU op: the
# reciprocal, or exp for the Gaussian core): LJ 12-6 and soft sphere as
# above (soft sphere: inv6^2 in place of inv6 (inv6 - 1)); Gaussian core:
# d, r^2, r^2 / sigma^2, exp argument, scale, select, accumulate


def flop_per_pair_of(potential):
    from jmmonedmc_gb300 import abi
    return {abi.JMM_POT_LJCUT: 9, abi.JMM_POT_LJ: 9, abi.JMM_POT_SOFTSPHERE: 9,
            abi.JMM_POT_GAUSS: 7}.get(int(potential), FLOP_PER_PAIR)
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--sweeps-per-step", type=int, default=1000)
    ap.add_argument("--chains", type=int, default=4096)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=1.5,
                    help="wall seconds per host core for the CPU baseline sample")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--workload", choices=("npt", "uneven", "large", "grad"), default="npt",
                    help="npt: the batched NPT headline workload; uneven: 1024 chains of "
                         "N ~ U{32..2048}, rho ~ U(0.3, 0.9), LJ / soft sphere / Gaussian core, "
                         "T ~ U(0.5, 2), NVT; large: 64 chains of N = 2^20 LJ particles, "
                         "rho 0.7, rc 2.5, T 1.2, alternating-domain sweep; grad: 2048 chains "
                         "of N = 512 LJ at rho 0.7, T 1 (half NVT, half NPT at P 1), energy "
                         "gradient sampled every 10th sweep")
    ap.add_argument("--domain-size", type=int, default=1024,
                    help="large workload: particles per domain")
    ap.add_argument("--sample-every", type=int, default=10,
                    help="grad workload: sweeps between gradient samples")
    ap.add_argument("--split-n", type=int, default=None,
                    help="batched workloads: constant-L chains of at least this many particles "
                         "run split over a block's warps in alternating domains (0 = none; "
                         "default 512 for the uneven workload, 0 otherwise)")
    ap.add_argument("--no-sub-workloads", action="store_true",
                    help="batched NPT workload at one GPU: leave out the compact records of the "
                         "uneven, gradient and large-chain workloads")
    args = ap.parse_args()
    return apply_workload_defaults(args)


def apply_workload_defaults(args):
    """Sizes of the chosen workload where the command line left the batched
    NPT workload's defaults."""
    if getattr(args, "split_n", None) is None:
        args.split_n = 512 if args.workload == "uneven" else 0
    if args.workload == "uneven":
        if args.chains == 4096:
            args.chains = 1024
        if args.sweeps_per_step == 1000:
            args.sweeps_per_step = 500
    if args.workload == "grad":
        if args.chains == 4096:
            args.chains = 2048
        if args.n == 256:
            args.n = 512
        if args.sweeps_per_step == 1000:
            args.sweeps_per_step = 200
    if args.workload == "large":
        if args.chains == 4096:
            args.chains = 64
        if args.n == 256:
            args.n = 1 << 20
        if args.sweeps_per_step == 1000:
            args.sweeps_per_step = 20
    return args


def uneven_workload(args, seed):
    """1024 chains of uneven N, density, potential and temperature (NVT)."""
    from jmmonedmc_gb300 import abi
    from jmmonedmc_gb300.philox_host import uniforms
    n_ch = args.chains
    un, ur, ut = (uniforms(seed, n_ch, stream=s) for s in (0xC1, 0xC2, 0xC3))
    pots = [(abi.JMM_POT_LJCUT, 3.0), (abi.JMM_POT_SOFTSPHERE, 2.5), (abi.JMM_POT_GAUSS, 4.0)]
    chains = []
    for c in range(n_ch):
        n = 32 + int(un[c] * (2048 - 32 + 1))
        pot, rc = pots[c % 3]
        chains.append(abi.make_chain(n, potential=pot, ensemble=abi.JMM_NLT, eps=1.0, sigma=1.0,
                                     cutoff=rc, t=0.5 + 1.5 * ut[c], rho=0.3 + 0.6 * ur[c],
                                     max_step=0.3))
    cfg = abi.make_batch_config(seed=seed, precision=abi.JMM_PREC_FAST, resum_sweeps=100,
                                split_n=getattr(args, "split_n", 0) or 0)
    return cfg, chains


def workload(args, rank=0):
    """Chain descriptions of the batched NPT workload (rank-shifted seed)."""
    from jmmonedmc_gb300 import abi
    from jmmonedmc_gb300.philox_host import uniforms
    n_ch = args.chains
    seed = rank_seed(args, rank)
    if args.workload == "uneven":
        return uneven_workload(args, seed)
    if args.workload == "grad":
        return grad_workload(args, seed)
    temps = [0.5 * 4.0 ** (c / max(1, n_ch - 1)) for c in range(n_ch)]
    press = [0.5 + 1.5 * u for u in uniforms(seed, n_ch, stream=0xB0)]
    chains = [abi.make_chain(args.n, potential=abi.JMM_POT_LJCUT, ensemble=abi.JMM_NPT,
                             eps=1.0, sigma=1.0, cutoff=3.0, t=temps[c], p=press[c],
                             rho=0.6, max_step=0.3, vol_step=0.01) for c in range(n_ch)]
    cfg = abi.make_batch_config(seed=seed, vol_move=abi.JMM_VOLMOVE_LNL,
                                vol_schedule=abi.JMM_VOLSCHED_SWEEP,
                                precision=abi.JMM_PREC_FAST)
    return cfg, chains


def config_dict(args, extra=None):
    if args.workload == "grad":
        return grad_config(args, extra)
    if args.workload == "uneven":
        split = getattr(args, "split_n", 0) or 0
        d = {"workload": (f"uneven batch: {args.chains} chains, N ~ U{{32..2048}}, rho ~ "
                          "U(0.3,0.9), potential cycling LJ rc=3 / soft sphere rc=2.5 / Gaussian "
                          "core rc=4 (eps=sigma=1), T ~ U(0.5,2.0), NVT, hard walls, max "
                          "displacement 0.3"
                          + (f"; chains of N >= {split} split over a block's warps in "
                             "alternating domains (sampled once per sweep)" if split else "")),
             "split_n": split,
             "chains": args.chains, "sweeps_per_step": args.sweeps_per_step,
             "l2": "flushed between timed steps (256 MiB device write)",
             "precision": "FP32 pair energies, FP64 running totals and accumulators"}
        if extra:
            d.update(extra)
        return d
    d = {
        "workload": (f"batched NPT: {args.chains} chains x N={args.n}, LJ 12-6 eps=sigma=1 rc=3, "
                     "hard walls, T log-spaced 0.5-2.0, P U(0.5,2.0), ln L moves delta=0.01 "
                     "once per sweep, max displacement 0.3, start rho=0.6 lattice"),
        "chains": args.chains,
        "particles_per_chain": args.n,
        "sweeps_per_step": args.sweeps_per_step,
        "moves_per_sweep": args.n + 1,
        "l2": "flushed between timed steps (256 MiB device write); inputs 4 MiB < L2",
        "precision": "FP32 pair energies, FP64 running totals and accumulators",
    }
    if extra:
        d.update(extra)
    return d


# ---- clocks ------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                    power.append(float(parts[3]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# ---- ranks -----------------------------------------------------------------------

def reduce_over_ranks(world, device, time_ms, counts):
    """The job's figures over the ranks of one node: the slowest rank's time
    and the sum of each count (every rank runs its own chains, no data is
    exchanged).  One rank: the values unchanged."""
    if world <= 1:
        return float(time_ms), [float(c) for c in counts]
    import torch
    t = torch.tensor([time_ms] + list(counts), dtype=torch.float64, device=device)
    tmax, tsum = t.clone(), t.clone()
    torch.distributed.all_reduce(tmax, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.all_reduce(tsum, op=torch.distributed.ReduceOp.SUM)
    return float(tmax[0]), [float(v) for v in tsum[1:]]


def rank_seed(args, rank):
    """Each rank's chains draw from their own Philox key."""
    return args.seed + 1000003 * rank


# ---- CPU baseline: the reference's algorithm on the host cores -------------

def _cpu_worker(job):
    """One host core: the reference's chain (plain FP64, pair-state arrays)
    for the workload's chain `k`, run for `seconds` wall seconds."""
    k, n, t, p, seed, seconds, repo, npt, l = job
    sys.path.insert(0, repo)
    from jmmonedmc_gb300 import abi
    from tests import oracle_lib
    params = abi.make_params(n=n, ensemble=abi.JMM_NPT if npt else abi.JMM_NLT,
                             potential=abi.JMM_POT_LJCUT, p=p, t=t, l=l, cutoff=3.0,
                             max_step=0.3, max_dl=0.01 * n / 0.6, seed=seed + k, eci=0)
    chain = oracle_lib.OraclePlain(params)
    chain.fad()
    chunk = n + 1
    steps = 0
    t0 = time.perf_counter()
    while True:
        chain.steps(chunk)
        steps += chunk
        if time.perf_counter() - t0 >= seconds:
            break
    return steps, time.perf_counter() - t0


def cpu_reference_sample(chains, seconds, seed):
    """Aggregate moves/s of the reference algorithm, one chain per host core."""
    import multiprocessing as mp
    from tests import oracle_lib
    oracle_lib.load()  # build the oracle library before the workers start
    cores = os.cpu_count() or 1
    picks = [int(i * len(chains) / cores) for i in range(cores)]
    from jmmonedmc_gb300 import abi
    jobs = [(k, int(chains[k].n), float(chains[k].t), float(chains[k].p), seed, seconds, REPO,
             chains[k].ensemble == abi.JMM_NPT, float(chains[k].l0)) for k in picks]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        out = pool.map(_cpu_worker, jobs)
    wall = time.perf_counter() - t0
    steps = sum(s for s, _ in out)
    per_core_wall = max(w for _, w in out)
    return {
        "value": steps / per_core_wall,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": (f"{cores} chains of the workload (sizes {sorted(int(chains[k].n) for k in picks)}"
                   f", LJcut 3.0 for every chain: the reference has no soft-sphere or Gaussian "
                   f"potential), one per host core, each run for {seconds:.1f} s with the "
                   "reference's algorithm (oracle/plain_oracle.c: FP64, per-pair state, O(N) "
                   "displacement, O(N^2) volume move, linear dL); aggregate attempted moves / wall"),
        "steps": steps,
        "wall_s": wall,
    }


# ---- roofline inputs -----------------------------------------------------------

FIGURES = os.path.join(REPO, "profiles", "figures.json")


def profile_figures(kernel):
    """The ncu figures of one kernel (profiles/figures.json, written from the
    committed ncu summaries), or {}."""
    if not os.path.exists(FIGURES):
        return {}
    with open(FIGURES) as f:
        return json.load(f).get(kernel, {})


def profile_traffic(args, pair_evals_per_launch, sweeps):
    """DRAM bytes per launch of the chain kernel from its ncu figures
    (measured on a smaller launch and scaled by the launch's sweeps)."""
    fig = profile_figures("chains_kernel_batched_npt")
    if "dram_bytes_per_chain_sweep" not in fig:
        return None
    return args.chains * (fig["dram_bytes_per_chain_sweep"] * sweeps
                          + fig.get("dram_bytes_per_chain_launch_fixed", 0.0))


def issue_roofline(kernel, moves_per_s, clocks, dev):
    """Warp instructions issued per second by the dominant kernel against the
    issue limit (4 schedulers per SM, one warp instruction each per clock):
    the kernel's instructions per attempted move, from its ncu figures, times
    the timed moves/s of one GPU."""
    import torch
    fig = profile_figures(kernel)
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if "warp_instructions_per_move" not in fig or not mhz:
        return None
    per_move = float(fig["warp_instructions_per_move"])
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    peak = sms * 4 * float(mhz) * 1e6
    achieved = per_move * moves_per_s
    return {"achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "instructions_per_move": per_move,
            "source": f"instructions per move from the ncu capture in {fig.get('summary')} "
                      f"(profiles/figures.json); peak = 4 issue slots per SM per clock x {sms} "
                      "SMs x the sampled SM clock"}


def in_cutoff_neighbours(x_all, sizes, rc, periodic_l=None):
    """Mean number of partners within the cut-off (|x_j - x_i| <= rc, either
    side) per particle, over every chain of a sample of ordered positions
    (x_all back to back, chain k holding sizes[k]): the k of the algorithmic
    work unit, in-cut-off pairs per moved particle."""
    import numpy as np
    total_pairs, total_particles, off = 0, 0, 0
    for k, n in enumerate(sizes):
        x = np.asarray(x_all[off:off + n], dtype=np.float64)
        off += n
        r = rc[k] if hasattr(rc, "__len__") else rc
        right = np.searchsorted(x, x + r, side="right") - np.arange(1, n + 1)
        total_pairs += int(right.sum())
        total_particles += n
    return 2.0 * total_pairs / max(1, total_particles)


def algorithmic_pairs(before, after, x_all, chains):
    """Pair evaluations the moves of the timed region need (the algorithmic
    work unit): a displacement evaluates its k in-cut-off partners at the old
    and the trial position (2k), a volume move the N k / 2 in-cut-off pairs
    at the new box length; k per chain from its positions after the run."""
    ks, off = [], 0
    for c in chains:
        n = int(c.n)
        ks.append(in_cutoff_neighbours(x_all[off:off + n], [n], float(c.cutoff)))
        off += n
    total = flop = 0.0
    for c, k, d_att, v_att in zip(chains, ks, after["disp_att"] - before["disp_att"],
                                  after["vol_att"] - before["vol_att"]):
        pairs = k * (2.0 * float(d_att) + 0.5 * int(c.n) * float(v_att))
        total += pairs
        flop += pairs * flop_per_pair_of(c.potential)
    return total, sum(ks) / max(1, len(ks)), flop


# ---- the large-chain workload -------------------------------------------------------

LARGE_METRIC = "attempted MC moves/s (large chains, alternating-domain sweep, FP32 pairs)"


def large_workload(args, seed):
    """64 chains of N = 2^20 LJ 12-6 particles, rho 0.7, rc 2.5, T 1.2, NVT."""
    from jmmonedmc_gb300 import abi
    chains = [abi.make_chain(args.n, potential=abi.JMM_POT_LJCUT, ensemble=abi.JMM_NLT,
                             cutoff=2.5, t=1.2, rho=0.7, max_step=0.3)
              for _ in range(args.chains)]
    cfg = abi.make_batch_config(seed=seed, resum_sweeps=0)
    return cfg, chains


def large_config(args, extra=None):
    d = {"workload": (f"large chains: {args.chains} chains x N={args.n}, LJ 12-6 eps=sigma=1 "
                      "rc=2.5, rho=0.7, T=1.2, NVT, hard walls, max displacement 0.3, lattice "
                      f"start; alternating-domain sweep, domains of {args.domain_size}"),
         "chains": args.chains, "particles_per_chain": args.n,
         "sweeps_per_step": args.sweeps_per_step, "domain_size": args.domain_size,
         "l2": f"inputs larger than L2 ({args.chains * (args.n + 32) * 8 >> 20} MiB of int64 "
               "positions), no flush",
         "precision": "positions int64 on a 2^-k grid, FP32 step arithmetic in domain frames, "
                      "FP64 energies"}
    if extra:
        d.update(extra)
    return d


def _cpu_large_worker(job):
    """One host core: one chain of the large workload with the FP64 CPU
    restatement (cut-off window, sequential Metropolis), `seconds` of wall."""
    n, seed, seconds, repo, k = job
    sys.path.insert(0, repo)
    from jmmonedmc_gb300 import abi
    from tests import oracle_lib
    chain = abi.make_chain(n, potential=abi.JMM_POT_LJCUT, ensemble=abi.JMM_NLT, cutoff=2.5,
                           t=1.2, rho=0.7, max_step=0.3)
    ob = oracle_lib.OracleBatch(abi.make_batch_config(seed=seed + k, resum_sweeps=0), [chain],
                                fp64=True)
    steps = 0
    t0 = time.perf_counter()
    while True:
        ob.run(1)
        steps += n
        if time.perf_counter() - t0 >= seconds:
            break
    return steps, time.perf_counter() - t0


def cpu_large_sample(args, seconds):
    import multiprocessing as mp
    from tests import oracle_lib
    oracle_lib.load()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        out = pool.map(_cpu_large_worker, [(args.n, args.seed, seconds, REPO, k)
                                           for k in range(cores)])
    wall = time.perf_counter() - t0
    steps = sum(s for s, _ in out)
    per_core_wall = max(w for _, w in out)
    return {"value": steps / per_core_wall, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"{cores} chains of the workload (N={args.n} each), one per host core, "
                       f"whole sweeps for {seconds:.1f} s each with the FP64 CPU restatement "
                       "(oracle/batch_oracle.c in FP64: sequential Metropolis with the cut-off "
                       "window; the reference itself cannot hold N=2^20, its pair arrays are "
                       "O(N^2)); aggregate attempted moves / wall"),
            "steps": steps, "wall_s": wall}


def run_large(args, rank, world, local_rank):
    import numpy as np
    import torch
    import ctypes as C

    from jmmonedmc_gb300 import _native, build
    if not os.path.exists(_native.lib_path()):
        build.build_native()
    from jmmonedmc_gb300.large import LargeChains, run_host

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    cfg, chains = large_workload(args, rank_seed(args, rank))
    cpu = cpu_large_sample(args, args.cpu_seconds) if rank == 0 and world == 1 else None
    fp32_peak, rcp_peak = C.c_double(), C.c_double()
    _native.call("jmm_measure_peaks", C.byref(fp32_peak), C.byref(rcp_peak))

    h = LargeChains(cfg, chains, domain_size=args.domain_size)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    S = args.sweeps_per_step
    for _ in range(args.warmup):
        h.run_async(S, "domains", stream.cuda_stream)
    torch.cuda.synchronize(dev)
    before = h.results()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    wall0 = time.perf_counter()
    for k in range(args.steps):
        starts[k].record(stream)
        h.run_async(S, "domains", stream.cuda_stream)
        ends[k].record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    after = h.results()
    if np.any(after["error"] != 0):
        raise RuntimeError(f"chain errors: {np.unique(after['error'])}")
    moves = int((after["moves"] - before["moves"]).sum())
    pairs = int((after["pair_evals"] - before["pair_evals"]).sum())
    total_ms = float(sum(step_ms))
    total_ms, (moves_all,) = reduce_over_ranks(world, dev, total_ms, [moves])

    # the sequential plain sweep of the same chains, one sweep, beside
    seq_start, seq_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0 = h.results()
    seq_start.record(stream)
    h.run_async(1, "sequential", stream.cuda_stream)
    seq_end.record(stream)
    torch.cuda.synchronize(dev)
    seq_ms = seq_start.elapsed_time(seq_end)
    r1 = h.results()
    seq_moves = int((r1["moves"] - r0["moves"]).sum())

    # e2e: host buffers through the C ABI (jmm_large_run_host), H2D and D2H inside
    n_tot = args.chains * args.n
    x_host = torch.empty(n_tot, dtype=torch.float64, pin_memory=True).numpy()
    x_back = torch.empty(n_tot, dtype=torch.float64, pin_memory=True).numpy()
    for k in range(args.chains):
        x_host[k * args.n:(k + 1) * args.n] = h.positions(k)
    h.close()
    # k from the first four chains' positions after the timed region (NVT:
    # 2k pair energies per displacement)
    k_sample = min(4, args.chains)
    k_mean = in_cutoff_neighbours(x_host[:k_sample * args.n], [args.n] * k_sample,
                                  float(chains[0].cutoff))
    alg_pairs = 2.0 * k_mean * moves
    e2e_times, e2e_moves = [], 0
    for j in range(args.e2e_steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res_h, _ = run_host(cfg, chains, S, domain_size=args.domain_size, mode="domains",
                            x_in=x_host, x_out=x_back)
        e2e_times.append(time.perf_counter() - t0)
        e2e_moves += int(res_h["moves"].sum())
        x_host, x_back = x_back, x_host
    e2e_value = e2e_moves / sum(e2e_times) * world
    h2d = n_tot * 8 + args.chains * C.sizeof(chains[0]) + 64
    d2h = n_tot * 8 + args.chains * 120

    traffic = None
    fig = profile_figures("domain_kernel_large_chains")
    if "dram_bytes_per_particle_phase" in fig:
        traffic = float(fig["dram_bytes_per_particle_phase"]) * args.chains * args.n / 2
    launches_per_step = 3 * S
    launch_ms = total_ms / (args.steps * 2 * S)  # the two domain launches of a sweep dominate
    pairs_per_launch = alg_pairs / (args.steps * 2 * S)
    achieved = pairs_per_launch * FLOP_PER_PAIR / (launch_ms * 1e-3) / 1e12
    line = {
        "metric": LARGE_METRIC,
        "value": moves_all / (total_ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (lattice start, seeded Philox moves)",
        "config": large_config(args, {"parallelism": f"replicas{world}", "wall_s_timed": wall,
                                      "grid": float(after["grid"][0])}),
        "roofline": {
            "bound": "fp32",
            "achieved": achieved,
            "peak": fp32_peak.value,
            "unit": "TFLOP/s",
            "frac": achieved / fp32_peak.value,
            "traffic": traffic,
            "peak_source": "measured live by jmm_measure_peaks (FP32 FMA kernel; "
                           "MEASURED_PEAKS.json holds no FP32 figure)",
            "pair_evals_per_launch": pairs_per_launch,
            "pair_evals_basis": (f"algorithmic: k = {k_mean:.3f} in-cut-off partners per "
                                 f"particle (first {k_sample} chains, positions after the timed "
                                 "region); 2k pair energies per displacement"),
            "in_cutoff_partners_k": k_mean,
            "window_slots_per_launch": pairs / (args.steps * 2 * S),
            "flop_per_pair": FLOP_PER_PAIR,
            "mufu_rcp_frac": pairs_per_launch / (launch_ms * 1e-3) / (rcp_peak.value * 1e12),
            "issue": issue_roofline("domain_kernel_large_chains",
                                    moves_all / world / (total_ms * 1e-3), clocks, dev),
            "kernel": "domain_kernel (one colour phase of one sweep)",
        },
        "sequential": {"value": seq_moves / (seq_ms * 1e-3), "unit": UNIT, "ms_per_sweep": seq_ms,
                       "how": "jmm_large_run(mode SEQUENTIAL): one warp per chain, one sweep of "
                              "the same chains after the timed region"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "how": "jmm_large_run_host per step: pinned float64 host positions in, results "
                       "and positions out, handle set-up inside the timed region"},
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clocks,
    }
    if cpu is not None:
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    return line


def run_reference_large(args):
    cores = os.cpu_count() or 1
    per_step = max(0.3, args.cpu_seconds / 2)
    for _ in range(args.warmup):
        cpu_large_sample(args, 0.2)
    t_total, steps_total, last = 0.0, 0, None
    for _ in range(args.steps):
        last = cpu_large_sample(args, per_step)
        t_total += last["steps"] / last["value"]
        steps_total += last["steps"]
    value = steps_total / t_total
    return {
        "metric": LARGE_METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (same chains as the GPU arm)",
        "config": large_config(args, {"parallelism": f"host cores x{cores}"}),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": last["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---- the differentiation workload -------------------------------------------------

GRAD_METRIC = ("attempted MC moves/s with the energy gradient sampled every 10th sweep "
               "(batched chains, FP32 pairs / FP64 totals and gradient sums)")


def grad_workload(args, seed):
    """2048 chains of N = 512 LJ 12-6, rho 0.7, T 1: half NVT, half NPT (P 1)."""
    from jmmonedmc_gb300 import abi
    chains = [abi.make_chain(args.n, potential=abi.JMM_POT_LJCUT,
                             ensemble=abi.JMM_NPT if k % 2 else abi.JMM_NLT, rho=0.7, t=1.0,
                             p=1.0, cutoff=3.0, max_step=0.3, vol_step=0.02)
              for k in range(args.chains)]
    cfg = abi.make_batch_config(seed=seed, vol_move=abi.JMM_VOLMOVE_LNL,
                                vol_schedule=abi.JMM_VOLSCHED_SWEEP, resum_sweeps=10,
                                precision=abi.JMM_PREC_FAST,
                                split_n=getattr(args, "split_n", 0) or 0)
    return cfg, chains


def grad_config(args, extra=None):
    split = getattr(args, "split_n", 0) or 0
    d = {"workload": (f"differentiation: {args.chains} chains x N={args.n}, LJ 12-6 eps=sigma=1 "
                      "rc=3, rho=0.7 lattice start, T=1, half NVT and half NPT (P=1, ln L "
                      "moves delta=0.02 once per sweep), max displacement 0.3; U, dU/deps, "
                      f"dU/dsigma, dU/dL of every chain every {args.sample_every} sweeps"
                      + (f"; NVT chains of N >= {split} split over a block's warps in "
                         "alternating domains (sampled once per sweep)" if split else "")),
         "split_n": split,
         "chains": args.chains, "particles_per_chain": args.n,
         "sweeps_per_step": args.sweeps_per_step, "sample_every": args.sample_every,
         "l2": "flushed between timed steps (256 MiB device write)",
         "precision": "FP32 pair energies and pair derivatives, FP64 totals, gradients and "
                      "fluctuation sums"}
    if extra:
        d.update(extra)
    return d


def run_grad(args, rank, world, local_rank):
    import numpy as np
    import torch
    import ctypes as C

    from jmmonedmc_gb300 import _native, build
    if not os.path.exists(_native.lib_path()):
        build.build_native()
    from jmmonedmc_gb300.batch import ChainBatch, chain_array, chain_view

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    cfg, chains = grad_workload(args, rank_seed(args, rank))
    cpu = cpu_reference_sample(chains, args.cpu_seconds, args.seed) if rank == 0 and world == 1 \
        else None
    fp32_peak, rcp_peak = C.c_double(), C.c_double()
    _native.call("jmm_measure_peaks", C.byref(fp32_peak), C.byref(rcp_peak))
    b = ChainBatch(cfg, chains)
    if args.no_autotune:
        lanes, spr, cpb = 0, 0, 0
    else:
        # one untimed step first, so that the trials see equilibrated chains
        # (on the starting lattice no fourth neighbour lies within the
        # cut-off, and a window of 3 would look best); trials of a few
        # milliseconds each: the shapes' differences are a few per cent
        b.run(args.sweeps_per_step)
        lanes, spr, cpb = b.autotune(trial_sweeps=20)
    from jmmonedmc_gb300 import abi
    names = {abi.JMM_POT_LJCUT: "ljcut", abi.JMM_POT_SOFTSPHERE: "softsphere",
             abi.JMM_POT_GAUSS: "gauss"}
    class_shapes = {names[p]: "%dx%d, %d per block, window %d" % v for p, v in b.shapes().items()}
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    S, every = args.sweeps_per_step, args.sample_every
    for _ in range(args.warmup):
        b.run_sampled_async(S, every, stream.cuda_stream)
    torch.cuda.synchronize(dev)
    b.reset_stats()
    before = b.results()

    def timed(run):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        torch.cuda.synchronize(dev)
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            run()
            ends[k].record(stream)
        torch.cuda.synchronize(dev)
        return sum(s.elapsed_time(e) for s, e in zip(starts, ends))

    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    wall0 = time.perf_counter()
    total_ms = timed(lambda: b.run_sampled_async(S, every, stream.cuda_stream))
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    after = b.results()
    gstats = b.grad_stats()
    if np.any(after["error"] != 0):
        raise RuntimeError(f"chain errors: {np.unique(after['error'])}")
    moves = int((after["steps"] - before["steps"]).sum())
    pairs = int((after["pair_evals"] - before["pair_evals"]).sum())
    samples = int(gstats["samples"].sum())
    # the same sweeps without the gradient samples, for the backward's share
    plain_ms = timed(lambda: b.run_async(S, stream.cuda_stream))
    total_ms, (moves_all,) = reduce_over_ranks(world, dev, total_ms, [moves])

    # e2e: host buffers through the public API: a batch built from host
    # positions, the sampled run, the gradient statistics and results read back
    n_tot = sum(int(c.n) for c in chains)
    x_host = torch.empty(n_tot, dtype=torch.float32, pin_memory=True).numpy()
    x_host[:] = np.concatenate([b.positions(k) for k in range(len(chains))])
    alg_pairs, k_mean, alg_flop = algorithmic_pairs(before, after, x_host, chains)
    desc = chain_array(chains)
    chain_view(desc)["l0"] = b.results()["l"]  # the box lengths of these positions
    e2e_times, e2e_moves = [], 0
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        b2 = ChainBatch(cfg, desc, x=x_host)
        b2.run_sampled(S, every)
        r2, g2 = b2.results(), b2.grad_stats()
        e2e_times.append(time.perf_counter() - t0)
        e2e_moves += int(r2["steps"].sum())
        b2.close()
    e2e = {"value": e2e_moves / sum(e2e_times) * world, "unit": UNIT,
           "h2d_bytes_per_step": n_tot * 4 + len(chains) * 8,
           "d2h_bytes_per_step": len(chains) * (C.sizeof(abi_result()) + C.sizeof(abi_gstats())),
           "how": "ChainBatch from pinned host positions (jmm_batch_create_at), run_sampled, "
                  "results and grad_stats read back, all inside the timed region"}
    launch_ms = total_ms / args.steps
    achieved = alg_pairs / args.steps * FLOP_PER_PAIR / (launch_ms * 1e-3) / 1e12
    line = {
        "metric": GRAD_METRIC,
        "value": moves_all / (total_ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (lattice start, seeded Philox moves)",
        "config": grad_config(args, {"lanes_per_chain": lanes, "steps_per_round": spr,
                                     "chains_per_block": cpb, "class_shapes": class_shapes,
                                     "parallelism": f"replicas{world}",
                                     "wall_s_timed": wall}),
        "gradient_samples_per_s": samples / (total_ms * 1e-3),
        "without_gradients": {"value": moves / (plain_ms * 1e-3), "unit": UNIT,
                              "how": "the same sweeps by run_async, no gradient samples"},
        "roofline": {
            "bound": "fp32", "achieved": achieved, "peak": fp32_peak.value, "unit": "TFLOP/s",
            "frac": achieved / fp32_peak.value, "traffic": None,
            "peak_source": "measured live by jmm_measure_peaks (FP32 FMA kernel; "
                           "MEASURED_PEAKS.json holds no FP32 figure)",
            "pair_evals_per_launch": alg_pairs / args.steps,
            "pair_evals_basis": (f"algorithmic: k = {k_mean:.3f} in-cut-off partners per "
                                 "particle (mean over chains); 2k pair energies per "
                                 "displacement, N k / 2 per volume move"),
            "in_cutoff_partners_k": k_mean,
            "window_slots_per_launch": pairs / args.steps, "flop_per_pair": FLOP_PER_PAIR,
            "kernel": "jmm::batch::chains_kernel (the gradient kernel runs between)"},
        "e2e": e2e,
        "gpu_launches": args.steps * (1 + S // every),
        "clocks": clocks,
    }
    if cpu is not None:
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    return line


def abi_result():
    from jmmonedmc_gb300 import abi
    return abi.ChainResult


def abi_gstats():
    from jmmonedmc_gb300 import abi
    return abi.GradStats


# ---- our implementation ----------------------------------------------------------

def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    import ctypes as C

    from jmmonedmc_gb300 import _native, abi, build
    if not os.path.exists(_native.lib_path()):
        build.build_native()
    from jmmonedmc_gb300.batch import ChainBatch, chain_array, chain_view, run_host

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    cfg, chains = workload(args, rank)

    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_reference_sample(chains, args.cpu_seconds, args.seed)

    lib = _native.load()
    fp32_peak, rcp_peak = C.c_double(), C.c_double()
    _native.call("jmm_measure_peaks", C.byref(fp32_peak), C.byref(rcp_peak))

    b = ChainBatch(cfg, chains)
    if args.no_autotune:
        lanes, spr, cpb = 0, 0, 0
    else:
        # one untimed step first (the GPU at its clocks, the chains off the
        # lattice), then trials of about a millisecond each, the best of three
        # runs per shape and the three fastest shapes timed again
        b.run(args.sweeps_per_step)
        lanes, spr, cpb = b.autotune(trial_sweeps=20 if args.workload == "npt" else 5)
    class_names = {abi.JMM_POT_LJCUT: "ljcut", abi.JMM_POT_SOFTSPHERE: "softsphere",
                   abi.JMM_POT_GAUSS: "gauss"}
    class_shapes = {class_names[p]: "%dx%d, %d per block, window %d" % v
                    for p, v in b.shapes().items()}
    # a stream of our own: torch's default stream is the legacy stream, whose
    # handle (0) would not name it to the library
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    S = args.sweeps_per_step
    for _ in range(args.warmup):
        b.run_async(S, stream.cuda_stream)
    torch.cuda.synchronize(dev)
    before = b.results()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        b.run_async(S, stream.cuda_stream)
        ends[k].record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    after = b.results()
    if np.any(after["error"] != 0):
        raise RuntimeError(f"chain errors: {np.unique(after['error'])}")
    moves = int((after["steps"] - before["steps"]).sum())
    pairs = int((after["pair_evals"] - before["pair_evals"]).sum())
    total_ms = float(sum(step_ms))
    total_ms, (moves_all, pairs_all) = reduce_over_ranks(world, dev, total_ms, [moves, pairs])

    # e2e: host buffers through the C ABI (jmm_batch_run_host), H2D and D2H inside
    n_tot = sum(int(c.n) for c in chains)
    x_host = torch.empty(n_tot, dtype=torch.float32, pin_memory=True).numpy()
    x_off = 0
    for k, c in enumerate(chains):
        x_host[x_off:x_off + c.n] = b.positions(k)
        x_off += c.n
    alg_pairs, k_mean, alg_flop = algorithmic_pairs(before, after, x_host, chains)
    lbox = after["l"].copy()
    for k, c in enumerate(chains):
        c.l0 = float(lbox[k])
    # one class: the tuned shape; several: the library's per-class defaults
    # (a host-buffer call carries one shape only)
    one_class = len(class_shapes) == 1
    e2e_cfg = abi.make_batch_config(seed=cfg.seed + 7, vol_move=cfg.vol_move,
                                    vol_schedule=cfg.vol_schedule, precision=cfg.precision,
                                    resum_sweeps=cfg.resum_sweeps,
                                    lanes_per_chain=lanes if one_class else 0,
                                    steps_per_round=spr if one_class else 0,
                                    chains_per_block=cpb if one_class else 0,
                                    window=next(iter(b.shapes().values()))[3] if one_class else 0,
                                    split_n=cfg.split_n)
    # the chain descriptions as the C call takes them, built once like the
    # pinned positions; each step continues from the last one's box lengths
    desc = chain_array(chains)
    e2e_times, e2e_moves = [], 0
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res_h, x_out = run_host(e2e_cfg, desc, S, x_in=x_host)
        e2e_times.append(time.perf_counter() - t0)
        e2e_moves += int(res_h["steps"].sum())
        x_host[:] = x_out
        chain_view(desc)["l0"] = res_h["l"]
    e2e_value = e2e_moves / sum(e2e_times) * world
    h2d = n_tot * 4 + args.chains * C.sizeof(abi.ChainDesc) + C.sizeof(abi.BatchConfig)
    d2h = n_tot * 4 + args.chains * C.sizeof(abi.ChainResult)

    plain = plain_rate(chains[0], args) if args.workload == "npt" and rank == 0 else None

    launch_ms = total_ms / args.steps
    # the algorithmic pair evaluations (in-cut-off partners), and the window
    # slots the kernel evaluates (4W per kept displacement, in-cut-off pairs
    # of the volume moves)
    alg_per_launch = alg_pairs / args.steps
    flop_per_launch = alg_flop / args.steps  # 9 FLOP per LJ or soft-sphere pair, 7 per Gaussian
    achieved = flop_per_launch / (launch_ms * 1e-3) / 1e12
    traffic = profile_traffic(args, pairs / args.steps, S) if args.workload == "npt" else None
    line = {
        "metric": METRIC,
        "value": moves_all / (total_ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Philox: T log-spaced, P uniform, lattice start)",
        "config": config_dict(args, {"lanes_per_chain": lanes, "steps_per_round": spr,
                                     "chains_per_block": cpb, "class_shapes": class_shapes,
                                     "parallelism": f"replicas{world}",
                                     "wall_s_timed": wall}),
        "roofline": {
            "bound": "fp32",
            "achieved": achieved,
            "peak": fp32_peak.value,
            "unit": "TFLOP/s",
            "frac": achieved / fp32_peak.value,
            "traffic": traffic,
            "peak_source": "measured live by jmm_measure_peaks (FP32 FMA kernel; "
                           "MEASURED_PEAKS.json holds no FP32 figure)",
            "pair_evals_per_launch": alg_per_launch,
            "pair_evals_basis": (f"algorithmic: k = {k_mean:.3f} in-cut-off partners per "
                                 "particle (mean over chains, positions after the timed "
                                 "region); 2k pair energies per displacement (old and trial "
                                 "position), N k / 2 per volume move"),
            "in_cutoff_partners_k": k_mean,
            "flop_per_pair": alg_flop / max(alg_pairs, 1.0),
            "flop_per_pair_by_potential": {"ljcut": 9, "softsphere": 9, "gauss": 7},
            "mufu_rcp_frac": alg_per_launch / (launch_ms * 1e-3) / (rcp_peak.value * 1e12),
            "pair_evals_per_s": alg_per_launch / (launch_ms * 1e-3),
            "window_slots_per_launch": pairs / args.steps,
            "window_slot_use": alg_per_launch / max(1.0, pairs / args.steps),
            "smem": smem_roofline(alg_per_launch, launch_ms),
            "issue": issue_roofline("chains_kernel_batched_npt",
                                    moves_all / world / (total_ms * 1e-3), clocks, dev)
            if args.workload == "npt" else None,
            "kernel": "jmm::batch::chains_kernel",
        },
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "how": "jmm_batch_run_host per step: pinned host positions in, results and "
                       "positions out, batch set-up inside the timed region"},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if cpu is not None:
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    if plain is not None:
        line["plain"] = plain
    return line


SMEM_BYTES_PER_CLOCK_SM = 128
SM_COUNT = 152
SM_MAX_MHZ = 2070


def smem_roofline(pair_evals_per_launch, launch_ms):
    """Shared-memory side of the roofline: one 4-byte neighbour position read
    serves the old and the trial pair energy, so 2 B per pair evaluation,
    against the nominal 128 B/clock/SM x 152 SMs x 2.07 GHz."""
    achieved = pair_evals_per_launch * 2.0 / (launch_ms * 1e-3) / 1e9
    peak = SMEM_BYTES_PER_CLOCK_SM * SM_COUNT * SM_MAX_MHZ * 1e6 / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "basis": "4 B per neighbour position read (old and trial pair energy), nominal "
                     "peak 128 B/clock/SM x 152 SMs x 2.07 GHz"}


def plain_rate(chain, args, steps=20000):
    """The plain FP64 form (the reference's algorithm on the GPU, one chain)
    on the workload's first chain: attempted moves/s, beside the batched
    rate.  The plain form runs the reference's move set: linear dL volume
    moves (max dL = delta L) drawn with probability 1/(N+1) per step."""
    from jmmonedmc_gb300 import abi
    from jmmonedmc_gb300.plain import PlainChain
    n = int(chain.n)
    params = abi.make_params(n=n, ensemble=abi.JMM_NPT, potential=abi.JMM_POT_LJCUT, p=chain.p,
                             t=chain.t, cutoff=3.0, max_step=0.3, max_dl=0.01 * n / 0.6,
                             seed=args.seed, eci=0)
    c = PlainChain(params)
    c.fad()
    c.steps(1000)
    t0 = time.perf_counter()
    c.steps(steps)
    dt = time.perf_counter() - t0
    c.close()
    return {"value": steps / dt, "unit": UNIT, "particles": n, "steps": steps,
            "how": "jmm_plain_steps on one chain of the workload (FP64, per-pair state, the "
                   "reference's step for step), wall clock around the synchronous call"}


# ---- the reference arm -----------------------------------------------------------

def reference_config(args, cores):
    """What the reference arm runs: the reference's own move set on the GPU
    arm's chains, not the GPU arm's moves."""
    d = config_dict(args, {"parallelism": f"host cores x{cores}"})
    d["gpu_arm_workload"] = d["workload"]
    vol = ("linear dL volume moves (max dL = 0.01 N / 0.6) drawn with probability 1/(N+1) "
           "per step, each an O(N^2) full re-sum (fav)" if args.workload == "npt"
           else "constant L (NLT)")
    d["workload"] = (
        "the reference's move loop (src/jmmMCState.cpp Step / qad2 / fav: FP64, per-pair state, "
        "all N-1 partners per displacement, " + vol + "; LJcut 3.0 for every chain) on the GPU "
        "arm's chains (N, T, P), one chain per host core; oracle/plain_oracle.c, which replays "
        "the reference build's trajectories bit for bit")
    return d


def run_reference(args):
    cfg, chains = workload(args, 0)
    cores = os.cpu_count() or 1
    per_step = max(0.2, args.cpu_seconds / 2)
    vals = []
    samples = []
    for _ in range(args.warmup):
        cpu_reference_sample(chains, 0.2, args.seed)
    t_total, steps_total = 0.0, 0
    for _ in range(args.steps):
        s = cpu_reference_sample(chains, per_step, args.seed)
        vals.append(s["value"])
        samples.append(s)
        t_total += s["steps"] / s["value"]
        steps_total += s["steps"]
    value = steps_total / t_total
    return {
        "metric": GRAD_METRIC if args.workload == "grad" else METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (same chains as the GPU arm)",
        "config": reference_config(args, cores),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": samples[-1]["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


SUB_WORKLOADS = ("uneven", "grad", "large")
SUB_KEYS = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "dtype", "e2e",
            "roofline", "cpu_baseline", "clocks", "gpu_launches", "sequential", "gradients")


def sub_workload_records(args, local_rank):
    """Compact records of the uneven, gradient and large-chain workloads at
    their own full sizes, for the one-GPU line: 3 timed steps after 3 warm-up
    steps (each workload's own step: 500, 200 and 20 sweeps), two e2e steps,
    a 1 s CPU sample."""
    out = {}
    for wl in SUB_WORKLOADS:
        sub = argparse.Namespace(**vars(args))
        sub.workload, sub.chains, sub.n, sub.sweeps_per_step = wl, 4096, 256, 1000
        sub.split_n = None
        apply_workload_defaults(sub)
        sub.steps, sub.warmup, sub.e2e_steps, sub.cpu_seconds = 3, 3, 2, 1.0
        runner = {"large": run_large, "grad": run_grad}.get(wl, run_ours)
        line = runner(sub, 0, 1, local_rank)
        rec = {k: line[k] for k in SUB_KEYS if k in line}
        rec["workload"] = line["config"]["workload"]
        rec["sweeps_per_step"] = sub.sweeps_per_step
        if "class_shapes" in line["config"]:
            rec["class_shapes"] = line["config"]["class_shapes"]
        out[wl] = rec
    return out


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        ref = run_reference_large if args.workload == "large" else run_reference
        print(json.dumps(ref(args)), flush=True)
        return 0
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    runner = {"large": run_large, "grad": run_grad}.get(args.workload, run_ours)
    line = runner(args, rank, world, local_rank)
    if world == 1 and args.workload == "npt" and not args.no_sub_workloads:
        line["workloads"] = sub_workload_records(args, local_rank)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
