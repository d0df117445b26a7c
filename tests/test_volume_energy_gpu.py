"""The volume move's two energies and their difference against the FP64 oracle.

A volume move compares U_new, the pair energy of the positions and box scaled
by s, with U_old, that of the current ones (fav's ETrial and E,
src/jmmMCState.cpp:2193-2249, which sums both in FP64).  The batched kernel
evaluates the pairs in FP32 and forms U_new - U_old in FP64: in EXACT
precision as the difference of two FP64 sums of per-particle FP32 sums, in
FAST (production) from per-pair differences (FP32 within a lane, FP64 across
lanes), so that no FP32 sum of the size of U enters the difference.
jmm_batch_volume_energies runs the move's own code (chain_energies) on the
batch's current configurations; the FP64 oracle sums the same FP32 positions
(and the FP32 products x_i * s the kernel forms) in FP64.

Stated bounds (walls, configurations equilibrated from the batched NPT
workload's states, scale factors within the workload's ln L step of 0.01),
FAST and EXACT alike:
  |U_old - U_old(FP64)|   <= 1e-6 |U|
  |dU - dU(FP64)|          <= 1e-6 |U|
The error of dU is that of the FP32 pair energies themselves (EXACT and FAST
give nearly the same dU), measured at up to about 2e-7 |U|, largest where
|U| is small against its largest pair terms (dilute chains, steep soft
spheres).
"""
import numpy as np
import pytest

from jmmonedmc_gb300 import abi
from jmmonedmc_gb300.batch import ChainBatch
from tests import oracle_lib

pytestmark = pytest.mark.gpu

REL_U = 1e-6
REL_DU = 1e-6


def _chains():
    """Chains of the batched NPT workload's kind on its T x P corners, and
    the uneven batch's soft-sphere and Gaussian-core classes."""
    chains = []
    for t in (0.5, 1.0, 2.0):
        for p in (0.5, 1.0, 2.0):
            for _ in range(4):
                chains.append(abi.make_chain(256, potential=abi.JMM_POT_LJCUT,
                                             ensemble=abi.JMM_NPT, cutoff=3.0, t=t, p=p,
                                             rho=0.6, max_step=0.3, vol_step=0.01))
    for pot, cut in ((abi.JMM_POT_SOFTSPHERE, 2.5), (abi.JMM_POT_GAUSS, 4.0)):
        for rho in (0.3, 0.9):
            for _ in range(4):
                chains.append(abi.make_chain(128, potential=pot, ensemble=abi.JMM_NPT,
                                             cutoff=cut, t=1.0, p=1.0, rho=rho, max_step=0.3,
                                             vol_step=0.01))
    return chains


@pytest.mark.parametrize("precision", [abi.JMM_PREC_FAST, abi.JMM_PREC_EXACT],
                         ids=["fast", "exact"])
def test_volume_move_energies_match_fp64(gpu, precision):
    chains = _chains()
    cfg = abi.make_batch_config(seed=21, precision=precision, vol_move=abi.JMM_VOLMOVE_LNL,
                                vol_schedule=abi.JMM_VOLSCHED_SWEEP)
    rng = np.random.default_rng(5)
    worst_u, worst_du = 0.0, {}
    with ChainBatch(cfg, chains) as b:
        for _ in range(3):
            b.run(200)
            res = b.results()
            assert not np.any(res["error"])
            # ln s uniform in +-0.01, as the workload's volume steps
            s = np.exp(rng.uniform(-0.01, 0.01, size=len(chains))).astype(np.float32)
            out = b.volume_energies(s)
            for k, c in enumerate(chains):
                x = b.positions(k)
                l = float(res["l"][k])
                lnew = l * float(s[k])
                xs = (x * s[k]).astype(np.float32)  # the kernel's FP32 products
                u0 = oracle_lib.energy64(c, x.astype(np.float64), l)
                u1 = oracle_lib.energy64(c, xs.astype(np.float64), lnew)
                scale = max(abs(u0), 1.0)
                eu = abs(out[k, 0] - u0) / scale
                edu = abs(out[k, 2] - (u1 - u0)) / scale
                assert eu <= REL_U, (k, out[k], u0)
                assert edu <= REL_DU, (k, c.potential, out[k, 2], u1 - u0, u0)
                # U_new and the difference agree to within an ulp of U
                assert abs(out[k, 1] - out[k, 0] - out[k, 2]) <= 4e-16 * abs(out[k, 1]) + 1e-300
                worst_u = max(worst_u, eu)
                worst_du[c.potential] = max(worst_du.get(c.potential, 0.0), edu)
    print(f"largest |U_old error| / |U| = {worst_u:.2e}; |dU error| / |U| by potential "
          f"(LJ, soft sphere, Gaussian core): "
          + ", ".join(f"{worst_du[p]:.2e}" for p in sorted(worst_du)))


def test_volume_energies_leave_the_state_alone(gpu):
    chains = _chains()[:8]
    cfg = abi.make_batch_config(seed=3, precision=abi.JMM_PREC_EXACT)
    with ChainBatch(cfg, chains) as b:
        b.run(20)
        r0 = b.results()
        x0 = [b.positions(k) for k in range(len(chains))]
        b.volume_energies(np.full(len(chains), 1.01, dtype=np.float32))
        r1 = b.results()
        assert r0.tobytes() == r1.tobytes()
        for k in range(len(chains)):
            assert np.array_equal(x0[k], b.positions(k))
