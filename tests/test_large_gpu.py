"""The large-chain sweeps (jmm_large_*): LJ 12-6 chains at rho = 0.7,
cut-off 2.5, T = 1.2, hard walls (the large-system workload's state point),
at sizes the FP64 CPU oracle finishes in seconds and at the full size of
64 chains x 2^20 particles through size-independent properties:

* bookkeeping: positions are multiples of a grid step, so every kernel sees
  the same FP32 separations; the running energy of either sweep equals a
  fresh FP64 sum of the final positions' pair energies up to FP32 summation
  order (5e-6 sqrt(N sweeps) + 1e-4), and that fresh energy agrees with the
  oracle's FP64 energy of the same positions (1e-6 relative);
* invariants: positions stay strictly increasing inside the walls; the same
  seed gives bit-identical positions;
* ensemble statistics: from the same lattice start, per-chain means of E/N
  and the acceptance ratio over the same sweep window, for the domain sweep,
  the sequential sweep and the FP64 CPU oracle (the batched restatement in
  FP64, one step at a time), agree within 4 combined standard errors plus
  2e-4 (FP32 pair terms);
* a configuration whose 16-particle halo does not reach beyond the cut-off
  is flagged (JMM_ERR_INVALID) and its domain skipped, while the sequential
  sweep handles it by extending its window.
"""
import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.large import LargeChains
from tests import oracle_lib

pytestmark = pytest.mark.gpu

RHO, T, RC, STEP = 0.7, 1.2, 2.5, 0.4


def _chains(n_chains, n, **kw):
    kw.setdefault("cutoff", RC)
    return [abi.make_chain(n, rho=RHO, t=T, max_step=STEP, **kw) for _ in range(n_chains)]


def _cfg(seed, resum=0):
    return abi.make_batch_config(seed=seed, resum_sweeps=resum)


def _drift_tol(n, sweeps):
    return 5e-6 * np.sqrt(n * sweeps) + 1e-4


def _check_positions(x, l):
    assert np.all(np.diff(x) > 0), "positions lost their order"
    assert np.all(np.abs(x) <= 0.5 * l)


def _window_gpu(n_chains, n, b, mode, eq, sweeps, seed):
    h = LargeChains(_cfg(seed, resum=10), _chains(n_chains, n), domain_size=b)
    h.run(eq, mode)
    h.reset_stats()
    r0 = h.results()
    h.run(sweeps, mode)
    r = h.results()
    assert np.all(r["error"] == 0)
    print(f"{mode}: largest drift at a re-sum {r['max_drift'].max():.3g}, grid {r['grid'][0]:.3g}")
    e_mean = r["sum_e"] / r["samples"] / n
    acc = (r["accepted"] - r0["accepted"]) / (r["moves"] - r0["moves"])
    fresh = h.energies()
    np.testing.assert_allclose(r["e"], fresh, rtol=0, atol=_drift_tol(n, 10))
    assert np.all(r["max_drift"] <= _drift_tol(n, 10)), r["max_drift"].max()
    for k in (0, n_chains - 1):
        _check_positions(h.positions(k), r["l"][k])
    h.close()
    return e_mean, acc


def _window_oracle(n_chains, n, eq, sweeps, seed):
    ob = oracle_lib.OracleBatch(_cfg(seed), _chains(n_chains, n), fp64=True)
    ob.run(eq)
    r0 = ob.results()
    ob.run(sweeps)
    r = ob.results()
    e_mean = (r["sum_e"] - r0["sum_e"]) / (r["samples"] - r0["samples"]) / n
    acc = (r["disp_acc"] - r0["disp_acc"]) / (r["disp_att"] - r0["disp_att"])
    return e_mean, acc


def _agree(a, b, what, slack=2e-4):
    diff = a.mean() - b.mean()
    sem = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    assert abs(diff) < 4 * sem + slack, (what, a.mean(), b.mean(), sem)


@pytest.mark.parametrize("n,b,gpu_chains,cpu_chains,eq,sweeps", [
    (256, 32, 512, 64, 300, 1200),      # many domain boundaries per chain
    (16384, 256, 64, 8, 300, 300),
])
def test_domain_and_sequential_sweeps_match_fp64_oracle(gpu, n, b, gpu_chains, cpu_chains, eq,
                                                       sweeps):
    dom = _window_gpu(gpu_chains, n, b, "domains", eq, sweeps, seed=21)
    seq = _window_gpu(gpu_chains, n, b, "sequential", eq, sweeps, seed=22)
    ora = _window_oracle(cpu_chains, n, eq, sweeps, seed=23)
    print(f"N={n} B={b}: <E>/N domains {dom[0].mean():.5f} sequential {seq[0].mean():.5f} "
          f"oracle {ora[0].mean():.5f}; acceptance {dom[1].mean():.4f} {seq[1].mean():.4f} "
          f"{ora[1].mean():.4f}")
    _agree(dom[0], ora[0], "E/N domains vs oracle")
    _agree(seq[0], ora[0], "E/N sequential vs oracle")
    _agree(dom[0], seq[0], "E/N domains vs sequential")
    _agree(dom[1], ora[1], "acceptance domains vs oracle", slack=5e-4)
    _agree(seq[1], ora[1], "acceptance sequential vs oracle", slack=5e-4)


def test_full_size_bookkeeping_and_invariants(gpu):
    n, n_chains = 1 << 20, 64
    chains = _chains(n_chains, n)
    h = LargeChains(_cfg(5, resum=0), chains, domain_size=256)
    h.run(10, "domains")
    r = h.results()
    assert np.all(r["error"] == 0)
    assert np.all(r["moves"] == 10 * n)
    assert np.all(r["sweeps"] == 10)
    fresh = h.energies()
    # running energy: FP64 base plus per-domain FP32-accumulated changes
    print(f"full size: |running - fresh| up to {np.abs(r['e'] - fresh).max():.3g}")
    np.testing.assert_allclose(r["e"], fresh, rtol=0, atol=_drift_tol(n, 10))
    for k in (0, 37, 63):
        x = h.positions(k)
        _check_positions(x, r["l"][k])
        e64 = oracle_lib.energy64(chains[k], x, r["l"][k])
        assert abs(fresh[k] - e64) <= 1e-6 * abs(e64), (k, fresh[k], e64)
    # one sequential sweep continues the same chains
    h.run(1, "sequential")
    r2 = h.results()
    assert np.all(r2["error"] == 0)
    assert np.all(r2["moves"] == 11 * n)
    np.testing.assert_allclose(r2["e"], h.energies(), rtol=0, atol=_drift_tol(n, 11))
    _check_positions(h.positions(5), r2["l"][5])
    h.close()


def test_same_seed_same_positions(gpu):
    def final(seed):
        h = LargeChains(_cfg(seed), _chains(8, 4096), domain_size=128)
        h.run(5, "domains")
        h.run(2, "sequential")
        h.run(3, "domains")
        xs = [h.positions(k) for k in (0, 7)]
        h.close()
        return xs

    a, b, c = final(9), final(9), final(10)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert not np.array_equal(a[0], c[0])


def test_set_positions_matches_oracle_energy(gpu):
    n = 8192
    chains = _chains(4, n)
    h = LargeChains(_cfg(3), chains, domain_size=256)
    rng = np.random.default_rng(4)
    l = chains[0].l0
    gaps = rng.uniform(0.8, 2.0, n + 1)
    x = np.cumsum(gaps)[:n]
    x = x - 0.5 * (x[0] + x[-1])
    assert np.all(np.abs(x) < 0.5 * l)
    h.set_positions(2, x)
    g = h.results()["grid"][2]
    x = np.rint(x / g) * g  # snapped to the grid
    assert np.array_equal(h.positions(2), x)
    e = h.energies()
    e64 = oracle_lib.energy64(chains[2], x, l)
    assert abs(e[2] - e64) <= 1e-6 * abs(e64)
    assert abs(h.results()["e"][2] - e[2]) <= 1e-9 * abs(e64)
    before = h.positions(1)
    with pytest.raises(Exception):
        h.set_positions(1, x[::-1].copy())  # decreasing: refused, chain unchanged
    assert np.array_equal(h.positions(1), before)
    h.close()


def test_run_host_continues_a_handle(gpu):
    from jmmonedmc_gb300.large import run_host
    n = 4096
    chains = _chains(4, n)
    h = LargeChains(_cfg(12), chains, domain_size=256)
    h.run(5, "domains")
    x = np.concatenate([h.positions(k) for k in range(4)])
    res, x_out = run_host(_cfg(13), chains, 3, domain_size=256, mode="domains", x_in=x)
    assert np.all(res["error"] == 0) and np.all(res["moves"] == 3 * n)
    for k in range(4):
        xk = x_out[k * n:(k + 1) * n]
        _check_positions(xk, chains[k].l0)
        e64 = oracle_lib.energy64(chains[k], xk, chains[k].l0)
        assert abs(res["e"][k] - e64) <= _drift_tol(n, 3) + 1e-6 * abs(e64)
    h.close()


def test_narrow_halo_is_flagged_and_sequential_handles_it(gpu):
    n, b = 4096, 256
    kw = dict(potential=abi.JMM_POT_GAUSS, cutoff=4.0)
    chains = _chains(1, n, **kw)
    l = chains[0].l0
    gaps = np.full(n - 1, 1.3)
    gaps[1500:1700] = 0.01  # a cluster of 200 particles within 2 sigma
    x = np.concatenate([[0.0], np.cumsum(gaps)])
    x -= 0.5 * (x[0] + x[-1])
    dom = LargeChains(_cfg(8), chains, domain_size=b)
    dom.set_positions(0, x)
    dom.run(10, "domains")
    r = dom.results()
    assert r["error"][0] == abi.JMM_ERR_INVALID
    _check_positions(dom.positions(0), l)
    np.testing.assert_allclose(r["e"], dom.energies(), rtol=1e-6)
    dom.close()
    seq = LargeChains(_cfg(8), chains, domain_size=b)
    seq.set_positions(0, x)
    seq.run(3, "sequential")
    r = seq.results()
    assert r["error"][0] == 0
    assert r["window_overflows"][0] > 0
    _check_positions(seq.positions(0), l)
    np.testing.assert_allclose(r["e"], seq.energies(), rtol=1e-6)
    seq.close()


def test_full_size_ensemble_matches_fp64_fixture(gpu):
    """The large-chain workload at its full size (64 chains x N = 2^20, LJ
    rc 2.5, rho 0.7, T 1.2, displacements up to 0.3, domains of 1024) against
    eight chains of the FP64 CPU restatement of the same state
    (tests/golden/ensemble_states.json, section "large": sequential
    single-particle Metropolis, the reference's move loop cannot hold 2^20):
    per-chain means of E/N and the acceptance ratio over sweeps 100-400 from
    the lattice, within 3 combined standard errors of the chain spreads plus
    2e-5 (FP32 pair terms)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                           "ensemble_states.json")) as f:
        fix = json.load(f)
    q = fix["protocol"]["large"]
    n = q["n"]
    chains = [abi.make_chain(n, rho=q["rho"], t=q["t"], cutoff=q["cutoff"], max_step=q["max_step"])
              for _ in range(64)]
    h = LargeChains(_cfg(41, resum=0), chains, domain_size=1024)
    h.run(q["equil"], "domains")
    h.reset_stats()
    r0 = h.results()
    h.run(q["prod"], "domains")
    r = h.results()
    h.close()
    assert np.all(r["error"] == 0)
    u = r["sum_e"] / r["samples"] / n
    acc = (r["accepted"] - r0["accepted"]) / (r["moves"] - r0["moves"])
    for name, g, c in (("E/N", u, np.array(fix["large"]["u"])),
                       ("acceptance", acc, np.array(fix["large"]["acc"]))):
        se = np.sqrt(g.var(ddof=1) / len(g) + c.var(ddof=1) / len(c))
        z = (g.mean() - c.mean()) / se
        print(f"N = 2^20 {name}: GPU domains {g.mean():.6f} (se {g.std(ddof=1) / 8:.1e}), "
              f"FP64 CPU {c.mean():.6f}, z = {z:+.2f}")
        assert abs(g.mean() - c.mean()) < 3 * se + 2e-5, (name, g.mean(), c.mean(), se)
