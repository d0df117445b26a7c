"""Parity of the batched chain kernel (jmm_batch_*) with the oracle.

* EXACT precision: every field of every chain's result, and every position,
  equals the oracle's FP32 replay bit for bit, across boundaries, ensembles,
  volume moves, schedules, potentials, uneven N and lane counts, over several
  launches.
* FAST precision (hardware reciprocal/exp, the production mode): energies of
  the GPU's configurations agree with the FP64 oracle to 1e-6 relative
  (fresh sums) and 1e-5 relative (running totals, which carry the FP32 drift
  since the last re-summation); short trajectories track the FP64 chain;
  ensemble averages (<U>/N, <rho>, box-length variance) of 8 NPT states agree
  with the FP64 CPU restatement within 4 standard errors of independent
  replicas.
"""
import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.batch import ChainBatch, averages, rng_words, run_host
from tests import oracle_lib

pytestmark = pytest.mark.gpu

RESULT_FIELDS = [f for f, _ in abi.CHAIN_RESULT_DTYPE]


def _mixed_chains(rng, n_chains, nmin, nmax, ensemble=None, pots=(abi.JMM_POT_LJCUT,)):
    chains = []
    for k in range(n_chains):
        n = int(rng.integers(nmin, nmax + 1))
        pot = pots[k % len(pots)]
        cutoff = {abi.JMM_POT_LJCUT: 3.0, abi.JMM_POT_SOFTSPHERE: 2.5, abi.JMM_POT_GAUSS: 4.0}[pot]
        ens = ensemble if ensemble is not None else (abi.JMM_NPT if k % 2 else abi.JMM_NLT)
        rho = float(rng.uniform(0.3, 0.9))
        chains.append(abi.make_chain(n, potential=pot, ensemble=ens, cutoff=cutoff,
                                     t=float(rng.uniform(0.5, 2.0)),
                                     p=float(rng.uniform(0.5, 2.0)), rho=rho,
                                     max_step=0.3, vol_step=0.02))
    return chains


def _assert_same(gpu, ora, chains):
    rg, ro = gpu.results(), ora.results()
    for f in RESULT_FIELDS:
        a, b = rg[f], ro[f]
        if a.dtype.kind == "f":
            bad = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
        else:
            bad = np.nonzero(a != b)[0]
        assert bad.size == 0, f"{f} differs for chains {bad[:8]}: gpu {a[bad[:3]]} oracle {b[bad[:3]]}"
    for k in range(len(chains)):
        xg = gpu.positions(k).astype(np.float64)
        xo = ora.positions(k)
        assert np.array_equal(xg, xo), f"positions of chain {k} differ"


EXACT_CASES = {
    "npt256_lnl_sweep_walls": dict(cfg=dict(vol_move=abi.JMM_VOLMOVE_LNL,
                                            vol_schedule=abi.JMM_VOLSCHED_SWEEP),
                                   n=(256, 256), ens=abi.JMM_NPT),
    "mixed_random_linear": dict(cfg=dict(vol_move=abi.JMM_VOLMOVE_LINEAR,
                                         vol_schedule=abi.JMM_VOLSCHED_RANDOM),
                                n=(32, 300), ens=None),
    "periodic_mixed_pots": dict(cfg=dict(boundary=abi.JMM_BOUNDARY_PERIODIC, resum_sweeps=3),
                                n=(40, 200), ens=None,
                                pots=(abi.JMM_POT_LJCUT, abi.JMM_POT_SOFTSPHERE, abi.JMM_POT_GAUSS)),
    "nvt_gauss_dense": dict(cfg=dict(resum_sweeps=2), n=(64, 128), ens=abi.JMM_NLT,
                            pots=(abi.JMM_POT_GAUSS,)),
    # the smallest chains: windows reach past both ends at every step
    "tiny_walls": dict(cfg=dict(resum_sweeps=5), n=(2, 8), ens=None,
                       pots=(abi.JMM_POT_LJCUT, abi.JMM_POT_SOFTSPHERE, abi.JMM_POT_GAUSS)),
}


# (lanes, steps per round, neighbours per side; 0 = the default of the lanes)
SHAPES = [(4, 8, 0), (2, 16, 0), (4, 4, 0), (4, 2, 0), (8, 4, 0), (8, 2, 0), (16, 2, 0),
          (16, 1, 0), (32, 1, 0), (4, 8, 8), (2, 16, 8), (8, 4, 8), (2, 16, 3)]


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{g}x{s}w{w}" for g, s, w in SHAPES])
@pytest.mark.parametrize("case", sorted(EXACT_CASES))
def test_batch_exact_matches_oracle(gpu, case, shape):
    lanes, spr, window = shape
    spec = EXACT_CASES[case]
    rng = np.random.default_rng(abs(hash(case)) % (2 ** 32))
    chains = _mixed_chains(rng, 24, *spec["n"], ensemble=spec["ens"],
                           pots=spec.get("pots", (abi.JMM_POT_LJCUT,)))
    cfg = abi.make_batch_config(seed=11, precision=abi.JMM_PREC_EXACT, lanes_per_chain=lanes,
                                steps_per_round=spr, window=window, init=abi.JMM_INIT_JITTER, jitter=0.05,
                                **spec["cfg"])
    gpu = ChainBatch(cfg, chains)
    ora = oracle_lib.OracleBatch(cfg, chains)
    _assert_same(gpu, ora, chains)  # initial lattice and energies
    for sweeps in (1, 7, 30):
        gpu.run(sweeps)
        ora.run(sweeps)
        _assert_same(gpu, ora, chains)


def test_batch_rng_words_match_oracle(gpu):
    got = rng_words(0xDEADBEEF12345, 1, 77, 1000)
    for i in (0, 1, 500, 999):
        assert list(got[i]) == oracle_lib.step_words(0xDEADBEEF12345, 1 + i, 77)


def test_batch_fast_energies_within_tolerance(gpu):
    rng = np.random.default_rng(5)
    chains = _mixed_chains(rng, 64, 64, 512,
                           pots=(abi.JMM_POT_LJCUT, abi.JMM_POT_SOFTSPHERE, abi.JMM_POT_GAUSS))
    cfg = abi.make_batch_config(seed=2, precision=abi.JMM_PREC_FAST, resum_sweeps=20)
    gpu = ChainBatch(cfg, chains)
    gpu.run(60)
    res = gpu.results()
    assert np.all(res["error"] == 0)
    fresh = gpu.energies()
    for k, c in enumerate(chains):
        x = gpu.positions(k).astype(np.float64)
        e64 = oracle_lib.energy64(c, x, res["l"][k])
        scale = max(1.0, abs(e64))
        assert abs(fresh[k] - e64) <= 1e-6 * scale, (k, fresh[k], e64)
        assert abs(res["e"][k] - e64) <= 1e-5 * scale, (k, res["e"][k], e64)
        assert np.all(np.diff(x) > 0), "particles must stay ordered"
        assert np.all(np.abs(x) <= res["l"][k] / 2 + 1e-4)


def test_batch_fast_tracks_fp64_chain(gpu):
    """For a few sweeps, FAST decisions coincide with the FP64 chain's for
    nearly every chain (they part only where an FP32 rounding flips a
    near-tie decision)."""
    rng = np.random.default_rng(9)
    chains = _mixed_chains(rng, 128, 64, 64, ensemble=abi.JMM_NPT)
    cfg = abi.make_batch_config(seed=4, precision=abi.JMM_PREC_FAST)
    gpu = ChainBatch(cfg, chains)
    ora = oracle_lib.OracleBatch(cfg, chains, fp64=True)
    gpu.run(5)
    ora.run(5)
    rg, ro = gpu.results(), ora.results()
    same = (rg["disp_acc"] == ro["disp_acc"]) & (rg["vol_acc"] == ro["vol_acc"])
    assert same.mean() >= 0.95, same.mean()
    # FP32 positions (|x| up to L/2 ~ 50, ulp ~ 4e-6) move the energies of the
    # tracked chains apart by ~1e-5 relative within a few sweeps
    np.testing.assert_allclose(rg["e"][same], ro["e"][same], rtol=2e-4, atol=1e-3)
    np.testing.assert_allclose(rg["l"][same], ro["l"][same], rtol=1e-5)


def test_batch_host_entry_matches_device_run(gpu):
    chains = [abi.make_chain(100, ensemble=abi.JMM_NPT, t=1.2, p=0.8)]
    cfg = abi.make_batch_config(seed=8, precision=abi.JMM_PREC_EXACT)
    res_h, x_h = run_host(cfg, chains, 20)
    gpu = ChainBatch(cfg, chains)
    gpu.run(20)
    res_d = gpu.results()
    assert res_h["e"][0] == res_d["e"][0] and res_h["sum_e"][0] == res_d["sum_e"][0]
    assert np.array_equal(x_h, gpu.positions(0))


def test_batch_autotune_keeps_state(gpu):
    rng = np.random.default_rng(1)
    chains = _mixed_chains(rng, 40, 64, 128, ensemble=abi.JMM_NPT)
    cfg = abi.make_batch_config(seed=6, precision=abi.JMM_PREC_EXACT)
    gpu = ChainBatch(cfg, chains)
    before = gpu.results()
    g, spr, c = gpu.autotune(trial_sweeps=2)
    (w,) = {v[3] for v in gpu.shapes().values()}
    assert (g, spr) in {(a, b) for a, b, _ in SHAPES} and c * g * spr in (32, 64, 128, 256)
    after = gpu.results()
    assert np.array_equal(before["e"], after["e"]) and np.array_equal(before["steps"], after["steps"])
    # the EXACT result does not depend on the block shape, only on the lanes
    cfg2 = abi.make_batch_config(seed=6, precision=abi.JMM_PREC_EXACT, lanes_per_chain=g,
                                 steps_per_round=spr, window=w)
    ora = oracle_lib.OracleBatch(cfg2, chains)
    gpu.run(5)
    ora.run(5)
    _assert_same(gpu, ora, chains)


def test_batch_rejects_bad_input(gpu):
    from jmmonedmc_gb300._native import JmmError
    with pytest.raises(JmmError):
        ChainBatch(abi.make_batch_config(), [abi.make_chain(1)])
    with pytest.raises(JmmError):
        ChainBatch(abi.make_batch_config(boundary=abi.JMM_BOUNDARY_PERIODIC),
                   [abi.make_chain(16, cutoff=3.0, l0=5.0)])
    b = ChainBatch(abi.make_batch_config(), [abi.make_chain(16)])
    with pytest.raises(JmmError):
        b.set_positions(0, np.linspace(1, -1, 16), 30.0)  # not increasing


def test_batch_create_at_matches_set_positions(gpu):
    """A batch created from host positions (jmm_batch_create_at) runs the
    same EXACT chains as one created on the lattice whose positions are then
    set chain by chain; bad positions are refused at creation."""
    from jmmonedmc_gb300._native import JmmError
    from jmmonedmc_gb300.batch import chain_array, chain_view
    rng = np.random.default_rng(21)
    chains = _mixed_chains(rng, 12, 32, 200, ensemble=abi.JMM_NPT)
    cfg = abi.make_batch_config(seed=5, precision=abi.JMM_PREC_EXACT, init=abi.JMM_INIT_JITTER,
                                jitter=0.05)
    src = ChainBatch(cfg, chains)
    src.run(3)
    xs = [src.positions(k) for k in range(len(chains))]
    lbox = src.results()["l"].copy()
    desc = chain_array(chains)
    chain_view(desc)["l0"] = lbox
    a = ChainBatch(cfg, desc, x=np.concatenate(xs))
    b = ChainBatch(cfg, chains)
    for k in range(len(chains)):
        b.set_positions(k, xs[k], float(lbox[k]))
    ra, rb = a.results(), b.results()
    assert np.array_equal(ra["e"].view(np.uint64), rb["e"].view(np.uint64))
    a.run(5)
    b.run(5)
    _assert_same(a, b, chains)
    bad = np.concatenate(xs)
    bad[3], bad[4] = bad[4], bad[3]  # chain 0 no longer increasing
    with pytest.raises(JmmError):
        ChainBatch(cfg, desc, x=bad)
    far = np.concatenate(xs)
    far[0] = -float(lbox[0])  # beyond the left wall
    with pytest.raises(JmmError):
        ChainBatch(cfg, desc, x=far)


def test_uneven_batch_at_full_size(gpu):
    """The uneven workload (1024 chains, N 32..2048, three potentials,
    rho 0.3-0.9, T 0.5-2, NVT) runs error-free in one graph of parallel
    per-potential kernels; the energies of a sample of chains agree with the
    FP64 oracle of the GPU's own configurations."""
    import argparse
    import bench
    args = argparse.Namespace(chains=1024, seed=1, workload="uneven", n=256)
    cfg, chains = bench.uneven_workload(args, 1)
    b = ChainBatch(cfg, chains)
    b.autotune(trial_sweeps=1)
    b.run(20)
    res = b.results()
    assert np.all(res["error"] == 0)
    assert np.all(res["steps"] == 20 * np.array([c.n for c in chains]))
    fresh = b.energies()
    for k in range(0, 1024, 97):
        x = b.positions(k).astype(np.float64)
        e64 = oracle_lib.energy64(chains[k], x, res["l"][k])
        assert abs(fresh[k] - e64) <= 1e-6 * max(1.0, abs(e64)), (k, fresh[k], e64)
        assert np.all(np.diff(x) > 0)


def test_npt_batch_at_full_size(gpu):
    """The benchmark workload at its configured length (4096 chains x N =
    256, LJ rc 3, walls, T log-spaced 0.5-2, P U(0.5, 2), ln L moves once
    per sweep, 1e4 sweeps): every chain made every step without error, its
    particles stay ordered inside the walls, the running energies agree with
    fresh sums and a sample with the FP64 oracle of the GPU's own positions,
    the same seed and shape replay bit for bit, and each chain's mean density
    lies between that of hard rods of diameter sigma at its (P, T),
    P / (T + P sigma), and close packing."""
    import argparse
    import bench
    args = argparse.Namespace(chains=4096, seed=1, workload="npt", n=256)
    cfg, chains = bench.workload(args)
    cfg.lanes_per_chain, cfg.steps_per_round, cfg.chains_per_block = 4, 8, 2
    runs = []
    for _ in range(2):
        b = ChainBatch(cfg, chains)
        b.run(10000)
        runs.append((b, b.results()))
    (b, res), (_, res2) = runs
    assert np.all(res["error"] == 0)
    assert np.all(res["steps"] == 10000 * 257)
    for f in ("e", "l", "sum_e", "sum_e2", "sum_l", "disp_acc", "vol_acc"):
        assert np.array_equal(res[f], res2[f]), f
    fresh = b.energies()
    scale = np.maximum(1.0, np.abs(fresh))
    assert np.all(np.abs(res["e"] - fresh) <= 1e-5 * scale)
    for k in range(0, 4096, 409):
        x = b.positions(k).astype(np.float64)
        assert np.all(np.diff(x) > 0) and np.all(np.abs(x) <= res["l"][k] / 2 * (1 + 1e-6))
        e64 = oracle_lib.energy64(chains[k], x, res["l"][k])
        assert abs(fresh[k] - e64) <= 1e-6 * max(1.0, abs(e64)), (k, fresh[k], e64)
    avg = averages(res)
    t = np.array([c.t for c in chains])
    p = np.array([c.p for c in chains])
    rho_rods = p / (t + p)  # the LJ core keeps neighbours about sigma apart; attraction adds
    assert np.all(avg["rho"] > 0.9 * rho_rods) and np.all(avg["rho"] < 1.3)


@pytest.mark.parametrize("boundary", [abi.JMM_BOUNDARY_WALLS, abi.JMM_BOUNDARY_PERIODIC])
def test_batch_histograms_match_oracle(gpu, boundary):
    """Sampled rho(x) / g(x) histograms of a mixed batch equal the oracle's
    counts of the same positions, sample by sample; run_sampled adds one
    sample every sample_every sweeps; configuring again clears them."""
    periodic = boundary == abi.JMM_BOUNDARY_PERIODIC
    rng = np.random.default_rng(31)
    chains = _mixed_chains(rng, 16, 40, 300,
                           pots=(abi.JMM_POT_LJCUT, abi.JMM_POT_SOFTSPHERE, abi.JMM_POT_GAUSS))
    b = ChainBatch(abi.make_batch_config(seed=9, boundary=boundary, resum_sweeps=4), chains)
    hp = (30, 12.0, 3, 150.0, 25, 0.2)  # rhonb, rbw, gns, gsw, gnb, gbw
    b.histograms(*hp)
    width = 1 + hp[0] + hp[2] * hp[4]
    ref = [np.zeros(width, dtype=np.uint64) for _ in chains]
    for sweeps in (0, 3, 10):
        if sweeps:
            b.run(sweeps)
        b.sample_histograms()
        res = b.results()
        for k in range(len(chains)):
            oracle_lib.hist_sample(b.positions(k), res["l"][k], periodic, *hp, row=ref[k])
    got = b.take_histograms()
    for k in range(len(chains)):
        assert got["samples"][k] == ref[k][0] == 3
        assert np.array_equal(got["rho"][k], ref[k][1:1 + hp[0]]), k
        assert np.array_equal(got["g"][k].ravel(), ref[k][1 + hp[0]:]), k
    assert got["g"].sum() > 0 and got["rho"].sum() > 0
    b.histograms(*hp)
    b.run_sampled(20, 5)
    again = b.take_histograms()
    assert np.all(again["samples"] == 4)
    n = np.array([c.n for c in chains], dtype=np.uint64)
    assert np.all(again["rho"].sum(axis=1) <= 4 * n)


@pytest.mark.parametrize("precision", [abi.JMM_PREC_EXACT, abi.JMM_PREC_FAST])
def test_batch_checkpoint_resumes_exactly(gpu, tmp_path, precision):
    """A batch saved mid-run (after its step sizes were adjusted on the
    device) and restored continues bit for bit like the original."""
    rng = np.random.default_rng(17)
    chains = _mixed_chains(rng, 20, 40, 200)
    cfg = abi.make_batch_config(seed=12, precision=precision, lanes_per_chain=4,
                                steps_per_round=8, resum_sweeps=3)
    a = ChainBatch(cfg, chains)
    a.run(7)
    a.adjust_steps()
    a.run(5)
    path = tmp_path / "batch.npz"
    a.checkpoint(path)
    a.run(9)
    b = ChainBatch.restore(path)
    b.run(9)
    _assert_same(a, b, chains)
    np.testing.assert_array_equal(np.array(a.step_sizes()), np.array(b.step_sizes()))
    from jmmonedmc_gb300._native import JmmError
    bad = b.results()
    bad["l"][3] = 0.5  # positions would lie beyond the walls
    with pytest.raises(JmmError):
        b.set_results(bad)


def _swendsen(step, actual, ideal=0.5):
    """maxDisAdjust's rescale (src/jmmMCState.cpp:2100-2116)."""
    return step * np.log(0.672924 * ideal + 0.0644284) / np.log(0.672924 * (actual + 0.0644284))


def test_step_adjust_on_device(gpu):
    """jmm_batch_adjust_steps applies the reference's rescale per chain from its
    counts (checked against the same formula on the host), keeps the
    reference's clamps, and equilibration with it moves every chain's
    displacement acceptance toward 1/2 (or its step to the 0.5 ceiling)."""
    chains = [abi.make_chain(128, ensemble=abi.JMM_NPT, rho=0.6, t=t, p=1.0, cutoff=3.0,
                             max_step=ms, vol_step=0.05)
              for t, ms in zip(np.linspace(0.6, 2.0, 64), np.tile([0.05, 0.3, 2.0, 0.001], 16))]
    b = ChainBatch(abi.make_batch_config(seed=4), chains)
    b.run(20)
    r = b.results()
    ms0, vs0 = b.step_sizes()
    b.adjust_steps()
    ms1, vs1 = b.step_sizes()
    want = np.clip(_swendsen(ms0, r["disp_acc"] / r["disp_att"]), 0.002, 0.5)
    np.testing.assert_allclose(ms1, want.astype(np.float32).astype(np.float64) * 1.0, rtol=1e-6)
    want_v = np.clip(_swendsen(vs0, r["vol_acc"] / r["vol_att"]), 1e-4, 1.0)
    np.testing.assert_allclose(vs1, want_v, rtol=1e-6)
    # equilibration: adjust every 20 sweeps from the counts of the last window
    for _ in range(15):
        b.reset_stats()
        b.run(20)
        b.adjust_steps()
    b.reset_stats()
    b.run(50)
    r = b.results()
    acc = r["disp_acc"] / r["disp_att"]
    ms_end, _ = b.step_sizes()
    # hot chains reach the reference's 0.5 ceiling with acceptance still high
    capped = ms_end >= np.float32(0.5)
    assert np.all(((acc > 0.3) & (acc < 0.75)) | (capped & (acc >= 0.3))), (acc, ms_end)
    assert np.sum(~capped) >= 8
    # a new launch layout keeps the adjusted sizes
    ms2, _ = b.step_sizes()
    b.autotune(trial_sweeps=2)
    np.testing.assert_array_equal(b.step_sizes()[0], ms2)


def _state_averages(res, n, states, reps):
    """Per state (T, P): replica means of <E>/N, <rho> and the length
    variance <L^2> - <L>^2, and their standard errors over the replicas."""
    s = res["samples"].astype(np.float64)
    e = res["sum_e"] / s / n
    rho = res["sum_rho"] / s
    lv = res["sum_l2"] / s - (res["sum_l"] / s) ** 2
    out = {}
    for q, v in (("e", e), ("rho", rho), ("lvar", lv)):
        v = v.reshape(states, reps)
        out[q] = (v.mean(axis=1), v.std(axis=1, ddof=1) / np.sqrt(reps))
    return out


def test_fast_ensemble_averages_match_fp64_oracle(gpu):
    """The batched kernel in production precision (FP32 pairs, FP64 totals)
    against the FP64 CPU restatement of the same chains: <U>/N, <rho> and the
    box-length variance of 8 NPT states (T, P), from independent replicas on
    each side (32 on the GPU, 16 on the CPU, equilibrated 500 sweeps, sampled
    2000), agree within 4 combined standard errors; the z scores are printed."""
    n, states, gpu_reps, cpu_reps = 64, 8, 32, 16
    ts = np.linspace(0.6, 1.6, states)
    ps = np.linspace(0.5, 2.0, states)[::-1]

    def chains(reps):
        return [abi.make_chain(n, ensemble=abi.JMM_NPT, rho=0.6, t=ts[s], p=ps[s], cutoff=3.0,
                               max_step=0.3, vol_step=0.05)
                for s in range(states) for _ in range(reps)]

    cfg_g = abi.make_batch_config(seed=101, precision=abi.JMM_PREC_FAST)
    cfg_c = abi.make_batch_config(seed=202, precision=abi.JMM_PREC_FAST)
    g = ChainBatch(cfg_g, chains(gpu_reps))
    o = oracle_lib.OracleBatch(cfg_c, chains(cpu_reps), fp64=True)
    for b in (g, o):
        b.run(500)
    g.reset_stats()
    r0 = o.results()
    g.run(2000)
    o.run(2000)
    rg = g.results()
    ro = o.results()
    for f in ("sum_e", "sum_e2", "sum_l", "sum_l2", "sum_rho", "sum_rho2", "samples"):
        ro[f] = ro[f] - r0[f]
    ag = _state_averages(rg, n, states, gpu_reps)
    ac = _state_averages(ro, n, states, cpu_reps)
    worst = 0.0
    for q in ("e", "rho", "lvar"):
        (mg, sg), (mc, sc) = ag[q], ac[q]
        z = (mg - mc) / np.sqrt(sg ** 2 + sc ** 2)
        print(f"{q}: gpu {np.round(mg, 4)} cpu {np.round(mc, 4)} z {np.round(z, 2)}")
        worst = max(worst, np.abs(z).max())
    assert worst < 4.0, worst


def test_autotune_per_potential_class(gpu):
    """FAST precision: every potential class gets its own launch shape (dense
    Gaussian-core chains need a wider neighbour window than LJ chains); the
    tuned batch stays within the FP64 energy tolerance and keeps its state."""
    chains = []
    for k in range(96):
        if k % 2:
            chains.append(abi.make_chain(512, potential=abi.JMM_POT_GAUSS, cutoff=4.0, rho=0.9,
                                         t=1.0, max_step=0.3))
        else:
            chains.append(abi.make_chain(512, potential=abi.JMM_POT_LJCUT, cutoff=3.0, rho=0.6,
                                         t=1.0, max_step=0.3))
    b = ChainBatch(abi.make_batch_config(seed=3, precision=abi.JMM_PREC_FAST, resum_sweeps=5),
                   chains)
    b.run(3)
    before = b.results()
    b.autotune(trial_sweeps=2)
    after = b.results()
    assert np.array_equal(before["e"], after["e"]) and np.array_equal(before["steps"], after["steps"])
    shapes = b.shapes()
    print("per-class shapes", shapes)
    assert set(shapes) == {abi.JMM_POT_LJCUT, abi.JMM_POT_GAUSS}
    assert shapes[abi.JMM_POT_GAUSS][3] >= 8  # a window of at least 8 per side
    b.run(10)
    res = b.results()
    assert np.all(res["error"] == 0)
    fresh = b.energies()
    for k in (0, 1, 94, 95):
        x = b.positions(k).astype(np.float64)
        e64 = oracle_lib.energy64(chains[k], x, res["l"][k])
        assert abs(fresh[k] - e64) <= 1e-6 * max(1.0, abs(e64))


def test_wide_and_narrow_kernels_agree(gpu):
    """A FAST batch of at most 16 whole single-warp chains per SM runs the
    128-register chain kernel, a larger one the 72-register kernel: the same
    code with another register budget, so a chain's record and positions
    must be the same bit for bit either way (a chain's random stream depends
    only on its index).  2600 chains (more than 16 per SM on 152 SMs) run
    narrow; their first 64 alone run wide."""
    rng = np.random.default_rng(77)
    chains = _mixed_chains(rng, 2600, 40, 120)
    cfg = abi.make_batch_config(seed=5, vol_move=abi.JMM_VOLMOVE_LNL,
                                vol_schedule=abi.JMM_VOLSCHED_SWEEP, precision=abi.JMM_PREC_FAST,
                                resum_sweeps=4, lanes_per_chain=4, steps_per_round=8,
                                chains_per_block=4)
    narrow, wide = ChainBatch(cfg, chains), ChainBatch(cfg, chains[:64])
    narrow.run(12)
    wide.run(12)
    rn, rw = narrow.results()[:64], wide.results()
    for f in RESULT_FIELDS:
        a, b = rn[f], rw[f]
        assert a.tobytes() == b.tobytes(), f
    for k in range(64):
        assert np.array_equal(narrow.positions(k), wide.positions(k)), k
    narrow.close()
    wide.close()
