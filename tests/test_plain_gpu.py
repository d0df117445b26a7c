"""Parity of the plain one-chain FP64 CUDA form (jmm_plain_*) with the
reference (golden fixtures) and with the oracle, through the C ABI.

The bar is bit-exact: same trial types, same E/Vir/HV after every step,
same box length, counters, final positions and thermo.dat.mcs text.
"""
import math

import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.plain import PlainChain
from tests import golden_cases as gc
from tests import oracle_lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", gc.case_names())
def test_plain_gpu_replays_reference(gpu, name):
    kw, params, ref = gc.load_case(name)
    chain = PlainChain(params)
    log, text = gc.run_like_driver(chain, kw)
    harmonic = kw["POT"] == "HARMONIC"
    np.testing.assert_array_equal(log["nm"], ref["nm"][1:])
    # a step of relaxVolume (RELAX, every 10000 steps) follows the step's own
    # record; the reference logs after it: compare the final state there
    keep = gc.unrelaxed_steps(kw, len(log))
    st_end = chain.state()
    for q, v in (("e", st_end.tot[0]), ("vir", st_end.tot[1]), ("l", st_end.l)):
        assert gc.bits(np.array([v]))[0] == gc.bits(ref[q][-1:])[0], q
    for q in ("e", "vir", "l") + (() if harmonic else ("hv",)):
        diff = np.nonzero((gc.bits(log[q]) != gc.bits(ref[q][1:])) & keep)[0]
        if diff.size:
            k = diff[0]
            pytest.fail(f"{q} differs first at step {k + 1}: gpu {log[q][k]!r} ref {ref[q][k + 1]!r}"
                        f" (bf {log['bf'][k]!r}, ran {log['ran'][k]!r})")
    acc = (log["outcome"] == abi.JMM_OUT_ACCEPT).astype(np.int8)
    np.testing.assert_array_equal(acc, ref["accepted"][1:])
    np.testing.assert_array_equal(gc.bits(chain.positions()), gc.bits(ref["r_final"]))
    ref_lines = str(ref["thermo_file"]).splitlines()
    our_lines = text.splitlines()
    assert len(our_lines) == len(ref_lines)
    for ours, theirs in zip(our_lines, ref_lines):
        if harmonic:
            ours, theirs = ours.split("\t")[:-2], theirs.split("\t")[:-2]
        assert ours == theirs


def _compare_logs(a, b, fields=("sn", "nm", "kind", "outcome")):
    for f in fields:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    for f in ("rn", "e", "vir", "hv", "l"):
        d = np.nonzero(gc.bits(a[f]) != gc.bits(b[f]))[0]
        assert d.size == 0, f"{f} differs first at step {d[0]}"
    both_nan = np.isnan(a["ran"]) & np.isnan(b["ran"])
    assert np.all(both_nan | (gc.bits(a["ran"]) == gc.bits(b["ran"]))), "ran"
    # bf = exp(...): CUDA's exp and the host libm's may differ in the last
    # place; the decisions (outcome, above) must not.
    fa, fb = a["bf"], b["bf"]
    nan = np.isnan(fa) & np.isnan(fb)
    close = np.abs(fa - fb) <= 4 * np.spacing(np.maximum(np.abs(fa), np.abs(fb)))
    assert np.all(nan | close), "bf beyond 4 ulp"


CONFIGS = [
    dict(n=64, l=64 / 0.6, t=1.0, cutoff=3.0, max_step=0.3, seed=1, eci=0),
    dict(n=64, ensemble=abi.JMM_NPT, p=1.0, t=1.0, cutoff=3.0, max_step=0.3, max_dl=0.5,
         seed=21, eci=1000),
    dict(n=200, ensemble=abi.JMM_NPT, p=0.5, t=0.8, cutoff=2.5, max_step=0.2, max_dl=3.0,
         seed=5, eci=5000),
    dict(n=33, potential=abi.JMM_POT_LJ, nbn=3, l=40.0, t=0.7, max_step=0.25, seed=8, eci=77),
]


@pytest.mark.parametrize("cfg", CONFIGS)
def test_plain_gpu_matches_oracle(gpu, cfg):
    params = abi.make_params(**cfg)
    g, o = PlainChain(params), oracle_lib.OraclePlain(params)
    g.fad()
    o.fad()
    for chunk in (1, 7, 3000, 12000):
        _compare_logs(g.steps(chunk, log=True), o.steps(chunk, log=True))
    gs, os_ = g.state(), o.state()
    assert list(gs.d_acc) == list(os_.d_acc) and list(gs.v_acc) == list(os_.v_acc)
    assert gs.rng_block == os_.rng_block and gs.rng_slot == os_.rng_slot
    np.testing.assert_array_equal(gc.bits(np.array(gs.thermo)), gc.bits(np.array(os_.thermo)))
    np.testing.assert_array_equal(gc.bits(g.positions()), gc.bits(o.positions()))
    np.testing.assert_array_equal(gc.bits(g.separations()), gc.bits(o.separations()))


def test_plain_gpu_config1_full_length(gpu):
    """The reference's CPU-runnable case at its full length: NLT, N = 64,
    L = 64/0.6, LJcut 3.0, T 1, MAXSTEP 0.3, seed 1, 2e4 sweeps = 1.28e6
    steps, ENGCHECK 64000, RHONB 10, GNS 1, GNB 10 (bin widths covering the
    box).  The GPU plain form and the oracle end bit for bit equal: counters,
    RNG position, thermo sums, positions, separations, histogram counts."""
    params = abi.make_params(n=64, l=64 / 0.6, t=1.0, cutoff=3.0, max_step=0.3, seed=1,
                             eci=64000)
    g, o = PlainChain(params), oracle_lib.OraclePlain(params)
    for c in (g, o):
        c.fad()
        c.histograms(10, 11.0, 1, 110.0, 10, 0.5)
    for _ in range(20):
        g.steps(64000)
        o.steps(64000)
    gs, os_ = g.state(), o.state()
    assert list(gs.d_acc) == list(os_.d_acc) and list(gs.v_acc) == list(os_.v_acc)
    assert gs.rng_block == os_.rng_block and gs.rng_slot == os_.rng_slot
    np.testing.assert_array_equal(gc.bits(np.array(gs.tot)), gc.bits(np.array(os_.tot)))
    np.testing.assert_array_equal(gc.bits(np.array(gs.thermo)), gc.bits(np.array(os_.thermo)))
    np.testing.assert_array_equal(gc.bits(g.positions()), gc.bits(o.positions()))
    np.testing.assert_array_equal(gc.bits(g.separations()), gc.bits(o.separations()))
    np.testing.assert_array_equal(np.asarray(g.take_rho()), np.asarray(o.take_rho()))
    np.testing.assert_array_equal(np.asarray(g.take_g()), np.asarray(o.take_g()))


def test_plain_gpu_replay_mode(gpu):
    """Fed an explicit table of draws (nm, rn, ran), both sides consume it alike."""
    params = abi.make_params(n=48, ensemble=abi.JMM_NPT, p=1.2, t=1.1, cutoff=3.0,
                             max_step=0.3, max_dl=0.8, seed=3)
    rng = np.random.default_rng(123)
    steps = 4000
    draws = list(zip(rng.integers(0, 49, steps), rng.random(steps), rng.random(steps)))
    g, o = PlainChain(params), oracle_lib.OraclePlain(params)
    g.fad()
    o.fad()
    _compare_logs(g.steps(steps, replay=draws, log=True), o.steps(steps, replay=draws, log=True))


def test_plain_gpu_echeck_reset_path(gpu):
    """A restart frame leaves E at 1e11 until fad; an energy check before that
    finds the discrepancy and rebuilds every pair (src/jmmMCState.cpp:1998-2083)."""
    params = abi.make_params(n=40, l=60.0, t=1.0, cutoff=3.0, max_step=0.3, seed=4, eci=1)
    g, o = PlainChain(params), oracle_lib.OraclePlain(params)
    r = ((np.arange(40) + 0.5) / 40 - 0.5) * 60.0 + np.sin(np.arange(40)) * 0.1
    for c in (g, o):
        c.fad()
        c.set_config(r, 60.0, sn=10)
        et, reset = c.echeck()
        assert reset and math.isfinite(et)
    gs, os_ = g.state(), o.state()
    assert gs.echeck_resets == os_.echeck_resets == 1
    np.testing.assert_array_equal(gc.bits(np.array(gs.tot)), gc.bits(np.array(os_.tot)))
    for c in (g, o):
        c.fad()
    _compare_logs(g.steps(500, log=True), o.steps(500, log=True))


def test_plain_gpu_rejects_bad_arguments(gpu):
    from jmmonedmc_gb300._native import JmmError
    with pytest.raises(JmmError):
        PlainChain(abi.make_params(n=1))
    with pytest.raises(JmmError):
        PlainChain(abi.make_params(n=10, potential=abi.JMM_POT_GAUSS))
    c = PlainChain(abi.make_params(n=10, l=20.0))
    with pytest.raises(JmmError):
        c.steps(1)  # before fad: out of order
    with pytest.raises(JmmError):
        c.fad(nm=10)


def test_plain_gpu_direct_moves_match_oracle(gpu):
    """qad2 / fav called outside Step (jmm_plain_move), draws from the stream."""
    params = abi.make_params(n=50, ensemble=abi.JMM_NPT, p=1.0, t=1.0, cutoff=3.0,
                             max_step=0.3, max_dl=1.0, seed=17)
    g, o = PlainChain(params), oracle_lib.OraclePlain(params)
    g.fad()
    o.fad()
    rng = np.random.default_rng(2)
    for k in range(300):
        kind = abi.JMM_KIND_VOLUME if k % 7 == 0 else abi.JMM_KIND_DISPLACEMENT
        nm, rn = int(rng.integers(0, 50)), float(rng.random())
        rg, ro = g.move(kind, nm, rn), o.move(kind, nm, rn)
        assert rg.outcome == ro.outcome and rg.e == ro.e and rg.l == ro.l, k
    np.testing.assert_array_equal(gc.bits(g.positions()), gc.bits(o.positions()))


@pytest.mark.parametrize("name", gc.case_names())
def test_plain_gpu_histogram_files_equal_reference(gpu, name):
    """fgrho/ugrho/qagrho on the GPU: rho.dat.mcs and g<k>.dat.mcs built from
    the GPU's counts equal the reference's files byte for byte."""
    kw, params, ref = gc.load_case(name)
    chain = PlainChain(params)
    _, _, files = gc.run_like_driver(chain, kw, histograms=True)
    theirs = gc.reference_histogram_files(kw, ref)
    assert sorted(files) == sorted(theirs)
    for fn, text in theirs.items():
        assert files[fn] == text, fn


HIST = (50, 3.0, 5, 25.0, 40, 0.1)  # rhonb, rbw, gns, gsw, gnb, gbw


@pytest.mark.parametrize("cfg", [
    # qavLJ volume moves recount and accumulate (the reference aborts there)
    dict(n=40, potential=abi.JMM_POT_LJ, nbn=-1, ensemble=abi.JMM_NPT, p=1.0, t=1.2,
         max_step=0.4, max_dl=2.0, seed=31, eci=0),
    # wall rejections accumulate too: a narrow box and wide steps
    dict(n=60, l=70.0, t=2.0, cutoff=3.0, max_step=2.5, seed=6, eci=0),
])
def test_plain_gpu_histograms_match_oracle(gpu, cfg):
    params = abi.make_params(**cfg)
    g, o = PlainChain(params), oracle_lib.OraclePlain(params)
    for c in (g, o):
        c.histograms(*HIST)
        c.fad()
    for chunk in (1, 5, 700, 3000):
        g.steps(chunk)
        o.steps(chunk)
        for a, b in zip(g.hist_counts(), o.hist_counts()):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(g.take_rho(), o.take_rho())
        np.testing.assert_array_equal(g.take_g(), o.take_g())
    rng = np.random.default_rng(9)
    for k in range(200):  # direct moves (qad2 / qavLJ / fav outside Step)
        kind = (abi.JMM_KIND_VOLUME if (k % 9 == 0 and cfg.get("ensemble") == abi.JMM_NPT)
                else abi.JMM_KIND_DISPLACEMENT)
        nm, rn = int(rng.integers(0, cfg["n"])), float(rng.random())
        g.move(kind, nm, rn)
        o.move(kind, nm, rn)
    np.testing.assert_array_equal(g.take_rho(), o.take_rho())
    np.testing.assert_array_equal(g.take_g(), o.take_g())
