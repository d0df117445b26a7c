"""bench.py's host side on CPU: the workloads it builds (chain counts, sizes,
potentials, temperatures, pressures, densities), its argument defaults, the
clock-record parser, the roofline inputs it reads from the committed ncu
summaries, and the reference arm's JSON line.  Nothing here needs a GPU."""
import json
import math
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402
from jmmonedmc_gb300 import abi  # noqa: E402


def args_for(monkeypatch, *argv):
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    return bench.parse_args()


@pytest.mark.parametrize("workload, chains, n, sweeps", [
    ("npt", 4096, 256, 1000),
    ("uneven", 1024, 256, 500),
    ("grad", 2048, 512, 200),
    ("large", 64, 1 << 20, 20),
])
def test_parse_args_workload_defaults(monkeypatch, workload, chains, n, sweeps):
    a = args_for(monkeypatch, "--workload", workload)
    assert (a.chains, a.n, a.sweeps_per_step) == (chains, n, sweeps)
    assert (a.gpus, a.warmup, a.impl) == (1, 3, "ours")
    assert a.warmup >= 3  # at least three untimed steps


def test_parse_args_keeps_explicit_sizes(monkeypatch):
    a = args_for(monkeypatch, "--workload", "grad", "--chains", "64", "--n", "128",
                 "--sweeps-per-step", "7")
    assert (a.chains, a.n, a.sweeps_per_step) == (64, 128, 7)


def test_npt_workload(monkeypatch):
    """4096 chains x N = 256 LJ rc 3, T log-spaced 0.5-2.0, P ~ U(0.5, 2.0),
    ln L moves delta 0.01 once per sweep, start rho 0.6, FAST precision."""
    a = args_for(monkeypatch)
    cfg, chains = bench.workload(a, 0)
    assert len(chains) == 4096
    assert {int(c.n) for c in chains} == {256}
    assert {int(c.potential) for c in chains} == {abi.JMM_POT_LJCUT}
    assert {int(c.ensemble) for c in chains} == {abi.JMM_NPT}
    assert {float(c.cutoff) for c in chains} == {3.0}
    t = [float(c.t) for c in chains]
    assert t[0] == pytest.approx(0.5) and t[-1] == pytest.approx(2.0)
    ratios = [t[i + 1] / t[i] for i in range(len(t) - 1)]
    assert max(ratios) == pytest.approx(min(ratios), rel=1e-12)  # log-spaced
    p = [float(c.p) for c in chains]
    assert 0.5 <= min(p) < 0.6 and 1.9 < max(p) < 2.0
    assert {float(c.l0) for c in chains} == {256 / 0.6}
    assert {float(c.vol_step) for c in chains} == {0.01}
    assert {float(c.max_step) for c in chains} == {0.3}
    assert cfg.vol_move == abi.JMM_VOLMOVE_LNL and cfg.vol_schedule == abi.JMM_VOLSCHED_SWEEP
    assert cfg.precision == abi.JMM_PREC_FAST and cfg.seed == a.seed


def test_npt_workload_is_seeded_per_rank(monkeypatch):
    a = args_for(monkeypatch, "--chains", "64")
    p0 = [float(c.p) for c in bench.workload(a, 0)[1]]
    assert p0 == [float(c.p) for c in bench.workload(a, 0)[1]]
    assert p0 != [float(c.p) for c in bench.workload(a, 1)[1]]
    assert bench.rank_seed(a, 0) == a.seed and bench.rank_seed(a, 1) != a.seed


def test_uneven_workload(monkeypatch):
    """1024 chains, N ~ U{32..2048}, rho ~ U(0.3, 0.9), LJ rc 3 / soft sphere
    rc 2.5 / Gaussian core rc 4 in turn, T ~ U(0.5, 2.0), NVT."""
    a = args_for(monkeypatch, "--workload", "uneven")
    cfg, chains = bench.workload(a, 0)
    assert len(chains) == 1024
    n = [int(c.n) for c in chains]
    assert 32 <= min(n) < 100 and 1950 < max(n) <= 2048
    pots = [(abi.JMM_POT_LJCUT, 3.0), (abi.JMM_POT_SOFTSPHERE, 2.5), (abi.JMM_POT_GAUSS, 4.0)]
    for k, c in enumerate(chains):
        assert (int(c.potential), float(c.cutoff)) == pots[k % 3]
        assert int(c.ensemble) == abi.JMM_NLT
        assert 0.5 <= float(c.t) < 2.0
        rho = int(c.n) / float(c.l0)
        assert 0.3 <= rho < 0.9 + 1e-12
    rhos = [int(c.n) / float(c.l0) for c in chains]
    assert min(rhos) < 0.35 and max(rhos) > 0.85
    assert cfg.precision == abi.JMM_PREC_FAST


def test_grad_workload(monkeypatch):
    """2048 chains x N = 512 LJ rc 3 at rho 0.7, T 1; odd chains NPT at P 1."""
    a = args_for(monkeypatch, "--workload", "grad")
    cfg, chains = bench.workload(a, 0)
    assert len(chains) == 2048 and {int(c.n) for c in chains} == {512}
    assert [int(c.ensemble) for c in chains[:4]] == [abi.JMM_NLT, abi.JMM_NPT] * 2
    assert sum(int(c.ensemble) == abi.JMM_NPT for c in chains) == 1024
    assert {float(c.t) for c in chains} == {1.0} and {float(c.p) for c in chains} == {1.0}
    assert {float(c.l0) for c in chains} == {512 / 0.7}
    assert cfg.resum_sweeps == 10 and cfg.precision == abi.JMM_PREC_FAST


def test_large_workload(monkeypatch):
    """64 chains x N = 2^20 LJ rc 2.5 at rho 0.7, T 1.2, NVT."""
    a = args_for(monkeypatch, "--workload", "large")
    cfg, chains = bench.large_workload(a, a.seed)
    assert len(chains) == 64 and {int(c.n) for c in chains} == {1 << 20}
    assert {float(c.cutoff) for c in chains} == {2.5}
    assert {float(c.t) for c in chains} == {1.2}
    assert {float(c.l0) for c in chains} == {(1 << 20) / 0.7}
    assert {int(c.ensemble) for c in chains} == {abi.JMM_NLT}
    d = bench.large_config(a)
    assert d["domain_size"] == 1024 and "larger than L2" in d["l2"]


@pytest.mark.parametrize("workload", ["npt", "uneven", "grad", "large"])
def test_config_names_the_workload(monkeypatch, workload):
    a = args_for(monkeypatch, "--workload", workload)
    d = bench.large_config(a) if workload == "large" else bench.config_dict(a, {"extra": 1})
    assert d["workload"] and d["chains"] == a.chains and "l2" in d
    assert "model" not in d
    if workload != "large":
        assert d["extra"] == 1


class _DoneProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _sampler_with(tmp_path, lines):
    s = bench.ClockSampler(0)
    s.path = str(tmp_path / "clocks.csv")
    with open(s.path, "w") as f:
        f.write("\n".join(lines) + "\n")
    s.proc = _DoneProc()
    return s


def test_clock_record_median_and_reasons(tmp_path):
    """The nvidia-smi record (csv, noheader, nounits): median SM clock under
    load, the maximum, and every throttle reason seen Active."""
    idle = "Not Active"
    lines = [
        f"0, 2070, 2070, 900.1, 0x0000000000000000, {idle}, {idle}, {idle}, {idle}",
        f"0, 2055, 2070, 1350.0, 0x0000000000000004, {idle}, {idle}, {idle}, Active",
        f"0, 2070, 2070, 1380.5, 0x0000000000000000, {idle}, {idle}, {idle}, {idle}",
        "garbage line",
        f"0, [N/A], 2070, 1.0, 0x0, {idle}, {idle}, {idle}, {idle}",
    ]
    r = _sampler_with(tmp_path, lines).stop()
    assert r["sm_mhz"] == 2070 and r["sm_max_mhz"] == 2070
    assert r["reasons"] == ["sw_power_cap"] and r["samples"] == 3
    assert r["power_w_max"] == 1380.5
    assert not os.path.exists(str(tmp_path / "clocks.csv"))


def test_clock_record_flags_thermal_slowdown(tmp_path):
    lines = ["0, 1500, 2070, 1100, 0x40, Not Active, Active, Active, Not Active"]
    r = _sampler_with(tmp_path, lines).stop()
    assert r["reasons"] == ["hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_clock_record_without_nvidia_smi():
    s = bench.ClockSampler(0)
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_clock_record_empty(tmp_path):
    assert _sampler_with(tmp_path, [""]).stop()["reasons"] == ["no samples"]


def test_profile_traffic_from_committed_figures(monkeypatch):
    """DRAM bytes per launch = chains x (bytes per chain sweep x sweeps +
    fixed bytes per chain), from the chain kernel's ncu figures."""
    a = args_for(monkeypatch)
    fig = bench.profile_figures("chains_kernel_batched_npt")
    t = bench.profile_traffic(a, None, 1000)
    assert t is not None and t > 0
    assert t == pytest.approx(a.chains * (fig["dram_bytes_per_chain_sweep"] * 1000
                                          + fig["dram_bytes_per_chain_launch_fixed"]))


def test_figures_name_committed_summaries():
    """Every kernel in profiles/figures.json names a committed ncu summary."""
    with open(bench.FIGURES) as f:
        figures = json.load(f)
    assert figures
    for kernel, fig in figures.items():
        assert os.path.exists(os.path.join(REPO, fig["summary"])), kernel
        assert fig["warp_instructions_per_move"] > 0


def test_in_cutoff_neighbours():
    """k: partners within the cut-off per particle, both sides, inclusive."""
    import numpy as np
    x = np.array([0.0, 1.0, 2.0, 3.5, 10.0])
    # rc = 2: pairs (0,1) (0,2) (1,2) (2,3) -> 4 pairs, k = 8 / 5
    assert bench.in_cutoff_neighbours(x, [5], 2.0) == pytest.approx(1.6)
    # two chains back to back, per-chain cut-offs: rc = 1 adds (0,1) (1,2)
    both = np.concatenate([x, x])
    assert bench.in_cutoff_neighbours(both, [5, 5], [2.0, 1.0]) == pytest.approx(12.0 / 10)


def test_algorithmic_pairs_weigh_each_potential():
    """2k pair energies per displacement, N k / 2 per volume move; 9 FP32
    FLOP per LJ or soft-sphere pair, 7 per Gaussian-core pair."""
    import numpy as np
    from jmmonedmc_gb300 import abi
    x = np.array([0.0, 1.0, 2.0, 3.5, 10.0])  # k = 1.6 at rc 2
    chains = [abi.make_chain(5, potential=abi.JMM_POT_LJCUT, cutoff=2.0),
              abi.make_chain(5, potential=abi.JMM_POT_SOFTSPHERE, cutoff=2.0),
              abi.make_chain(5, potential=abi.JMM_POT_GAUSS, cutoff=2.0)]
    before = {"disp_att": np.zeros(3), "vol_att": np.zeros(3)}
    after = {"disp_att": np.array([10.0, 10.0, 10.0]), "vol_att": np.array([2.0, 0.0, 0.0])}
    pairs, k, flop = bench.algorithmic_pairs(before, after, np.concatenate([x, x, x]), chains)
    per = [1.6 * (2 * 10 + 0.5 * 5 * 2), 1.6 * 20, 1.6 * 20]
    assert k == pytest.approx(1.6)
    assert pairs == pytest.approx(sum(per))
    assert flop == pytest.approx(9 * per[0] + 9 * per[1] + 7 * per[2])


@pytest.mark.parametrize("profile", ["chains_kernel_batched_npt",
                                     "domain_kernel_large_chains"])
def test_issue_roofline_from_committed_figures(monkeypatch, profile):
    """Issue-slot roofline: instructions per move from the kernel's ncu
    figures x moves/s against 4 issue slots per SM per clock."""
    import torch

    class Props:
        multi_processor_count = 152

    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda dev: Props())
    r = bench.issue_roofline(profile, 2.0e10, {"sm_mhz": 2070.0}, 0)
    assert r is not None and r["instructions_per_move"] > 0
    assert r["peak"] == pytest.approx(152 * 4 * 2070e6)
    assert r["frac"] == pytest.approx(r["instructions_per_move"] * 2.0e10 / r["peak"])
    assert 0 < r["frac"] < 1.2
    assert bench.issue_roofline(profile, 1.0, {}, 0) is None  # no clock record
    assert bench.issue_roofline("no_such_kernel", 1.0, {"sm_mhz": 1.0}, 0) is None


def test_smem_roofline():
    r = bench.smem_roofline(1.0e9, 1.0)
    assert r["achieved"] == pytest.approx(2.0e9 / 1e-3 / 1e9)
    assert r["peak"] == pytest.approx(128 * 152 * 2.07e9 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])


def test_single_rank_reduce_is_identity():
    t, counts = bench.reduce_over_ranks(1, None, 2.5, [3, 4.5])
    assert (t, counts) == (2.5, [3.0, 4.5])


def _run_bench(argv, env_extra=None, timeout=300):
    env = dict(os.environ, **(env_extra or {}))
    return subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), *argv],
                          capture_output=True, text=True, timeout=timeout, env=env, cwd=REPO)


@pytest.mark.parametrize("workload", ["npt", "uneven", "grad", "large"])
def test_reference_arm_prints_one_json_line(workload):
    """--impl reference: the reference's algorithm on the host cores for the
    same chains, one JSON line with the contract's keys and e2e without copies."""
    p = _run_bench(["--impl", "reference", "--workload", workload, "--steps", "1",
                    "--warmup", "0", "--cpu-seconds", "0.4"])
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "moves/s" and d["higher_is_better"]
    assert d["value"] > 0 and math.isfinite(d["value"])
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"],
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"] and "model" not in d["config"]


def test_reference_arm_other_ranks_exit_quietly():
    p = _run_bench(["--impl", "reference", "--steps", "1", "--warmup", "0"],
                   {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""


def test_own_arm_without_a_gpu_fails_loudly():
    """No CPU fallback: without a CUDA device the GPU arm exits non-zero and
    prints no JSON line."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    p = _run_bench(["--steps", "1", "--warmup", "3", "--chains", "64"], timeout=120)
    assert p.returncode != 0
    assert not any(ln.strip().startswith("{") for ln in p.stdout.splitlines())


def test_uneven_workload_splits_long_chains_by_default(monkeypatch):
    """The uneven workload runs its chains of N >= 512 split (the batched
    config's split_n); --split-n 0 runs every chain whole; other workloads
    split nothing unless asked."""
    a = args_for(monkeypatch, "--workload", "uneven")
    cfg, _ = bench.uneven_workload(a, 1)
    assert a.split_n == 512 and cfg.split_n == 512
    assert bench.config_dict(a)["split_n"] == 512
    a = args_for(monkeypatch, "--workload", "uneven", "--split-n", "0")
    assert bench.uneven_workload(a, 1)[0].split_n == 0
    assert args_for(monkeypatch).split_n == 0
