"""ctypes mirror of the public C ABI in include/jmm_gpu.h.

Every structure here has the exact field order and types of its C
counterpart; ``tests/test_abi.py`` checks the sizes against the header.
"""
import ctypes as C

JMM_OK = 0
JMM_ERR_INVALID = 1
JMM_ERR_CUDA = 2
JMM_ERR_NOMEM = 3
JMM_ERR_TIMEOUT = 4
JMM_ERR_NUMERIC = 5
JMM_ERR_STATE = 6

ERROR_NAMES = {
    JMM_OK: "ok",
    JMM_ERR_INVALID: "invalid argument",
    JMM_ERR_CUDA: "CUDA error",
    JMM_ERR_NOMEM: "out of memory",
    JMM_ERR_TIMEOUT: "device wait timed out",
    JMM_ERR_NUMERIC: "non-finite value",
    JMM_ERR_STATE: "call out of order",
}

JMM_NLT = 0
JMM_NPT = 1

JMM_POT_LJCUT = 0
JMM_POT_LJ = 1
JMM_POT_HARMONIC = 2
JMM_POT_SOFTSPHERE = 3
JMM_POT_GAUSS = 4

Q_NAMES = ("e", "vir", "e12", "vir12", "e6", "vir6", "hv", "hv12", "hv6")
THERMO_NAMES = ("rhoSysA", "rhoSysSA", "lA", "lSA", "EA", "ESA", "lEA",
                "VirA", "VirSA", "EVirA", "HVA", "HVSA")

JMM_KIND_DISPLACEMENT = 0
JMM_KIND_VOLUME = 1
JMM_OUT_REJECT_WALL = 0
JMM_OUT_REJECT = 1
JMM_OUT_ACCEPT = 2


class Params(C.Structure):
    _fields_ = [
        ("n", C.c_uint64),
        ("ensemble", C.c_int32),
        ("potential", C.c_int32),
        ("p", C.c_double),
        ("l", C.c_double),
        ("t", C.c_double),
        ("cutoff", C.c_double),
        ("nbn", C.c_int32),
        ("reserved0", C.c_int32),
        ("max_step", C.c_double),
        ("max_dl", C.c_double),
        ("seed", C.c_uint64),
        ("eci", C.c_uint64),
    ]


class State(C.Structure):
    _fields_ = [
        ("sn", C.c_uint64),
        ("rng_block", C.c_uint64),
        ("rng_slot", C.c_uint32),
        ("error", C.c_uint32),
        ("l", C.c_double),
        ("tot", C.c_double * 9),
        ("d_acc", C.c_uint64 * 2),
        ("v_acc", C.c_uint64 * 2),
        ("max_step", C.c_double),
        ("max_dl", C.c_double),
        ("thermo", C.c_double * 12),
        ("echeck_count", C.c_uint64),
        ("echeck_resets", C.c_uint64),
        ("echeck_e", C.c_double),
        ("echeck_e_before", C.c_double),
    ]


class Draw(C.Structure):
    _fields_ = [("nm", C.c_uint64), ("rn", C.c_double), ("ran", C.c_double)]


class StepRecord(C.Structure):
    _fields_ = [
        ("sn", C.c_uint64),
        ("nm", C.c_uint64),
        ("rn", C.c_double),
        ("ran", C.c_double),
        ("bf", C.c_double),
        ("e", C.c_double),
        ("vir", C.c_double),
        ("hv", C.c_double),
        ("l", C.c_double),
        ("kind", C.c_int32),
        ("outcome", C.c_int32),
    ]


STEP_RECORD_DTYPE = [
    ("sn", "<u8"), ("nm", "<u8"), ("rn", "<f8"), ("ran", "<f8"), ("bf", "<f8"),
    ("e", "<f8"), ("vir", "<f8"), ("hv", "<f8"), ("l", "<f8"),
    ("kind", "<i4"), ("outcome", "<i4"),
]


def make_params(n, ensemble=JMM_NLT, potential=JMM_POT_LJCUT, p=1.0, l=None,
                t=1.0, cutoff=3.0, nbn=-1, max_step=0.3, max_dl=1.0, seed=1,
                eci=0):
    """Build a Params with the INPUT keyword meanings of src/readInput.cpp."""
    prm = Params()
    prm.n = n
    prm.ensemble = ensemble
    prm.potential = potential
    prm.p = p
    prm.l = float(n) if l is None else l
    prm.t = t
    prm.cutoff = float("inf") if potential == JMM_POT_LJ else cutoff
    prm.nbn = nbn
    prm.max_step = max_step
    prm.max_dl = max_dl
    prm.seed = seed
    prm.eci = eci
    return prm


# ---- batched form ---------------------------------------------------------
JMM_BOUNDARY_WALLS = 0
JMM_BOUNDARY_PERIODIC = 1
JMM_VOLMOVE_LINEAR = 0
JMM_VOLMOVE_LNL = 1
JMM_VOLSCHED_RANDOM = 0
JMM_VOLSCHED_SWEEP = 1
JMM_PREC_FAST = 0
JMM_PREC_EXACT = 1
JMM_INIT_LATTICE = 0
JMM_INIT_JITTER = 1


class ChainDesc(C.Structure):
    _fields_ = [
        ("n", C.c_uint32),
        ("potential", C.c_int32),
        ("ensemble", C.c_int32),
        ("reserved0", C.c_int32),
        ("eps", C.c_double),
        ("sigma", C.c_double),
        ("cutoff", C.c_double),
        ("t", C.c_double),
        ("p", C.c_double),
        ("l0", C.c_double),
        ("max_step", C.c_double),
        ("vol_step", C.c_double),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("boundary", C.c_int32),
        ("vol_move", C.c_int32),
        ("vol_schedule", C.c_int32),
        ("precision", C.c_int32),
        ("resum_sweeps", C.c_uint32),
        ("lanes_per_chain", C.c_uint32),
        ("steps_per_round", C.c_uint32),
        ("chains_per_block", C.c_uint32),
        ("init", C.c_int32),
        ("jitter", C.c_double),
        ("window", C.c_uint32),
        ("split_n", C.c_uint32),
    ]


class ChainResult(C.Structure):
    _fields_ = [
        ("e", C.c_double),
        ("l", C.c_double),
        ("steps", C.c_uint64),
        ("samples", C.c_uint64),
        ("sum_e", C.c_double),
        ("sum_e2", C.c_double),
        ("sum_l", C.c_double),
        ("sum_l2", C.c_double),
        ("sum_le", C.c_double),
        ("sum_rho", C.c_double),
        ("sum_rho2", C.c_double),
        ("disp_acc", C.c_uint64),
        ("disp_att", C.c_uint64),
        ("vol_acc", C.c_uint64),
        ("vol_att", C.c_uint64),
        ("pair_evals", C.c_uint64),
        ("max_drift", C.c_double),
        ("error", C.c_uint32),
        ("window_overflows", C.c_uint32),
    ]


CHAIN_RESULT_DTYPE = [
    ("e", "<f8"), ("l", "<f8"), ("steps", "<u8"), ("samples", "<u8"),
    ("sum_e", "<f8"), ("sum_e2", "<f8"), ("sum_l", "<f8"), ("sum_l2", "<f8"),
    ("sum_le", "<f8"), ("sum_rho", "<f8"), ("sum_rho2", "<f8"),
    ("disp_acc", "<u8"), ("disp_att", "<u8"), ("vol_acc", "<u8"), ("vol_att", "<u8"),
    ("pair_evals", "<u8"), ("max_drift", "<f8"), ("error", "<u4"),
    ("window_overflows", "<u4"),
]


def make_chain(n, potential=JMM_POT_LJCUT, ensemble=JMM_NLT, eps=1.0, sigma=1.0,
               cutoff=3.0, t=1.0, p=1.0, l0=None, rho=None, max_step=0.3, vol_step=0.01):
    d = ChainDesc()
    d.n = n
    d.potential = potential
    d.ensemble = ensemble
    d.eps = eps
    d.sigma = sigma
    d.cutoff = cutoff
    d.t = t
    d.p = p
    if l0 is None:
        l0 = n / (rho if rho is not None else 0.6)
    d.l0 = l0
    d.max_step = max_step
    d.vol_step = vol_step
    return d


def make_batch_config(seed=1, boundary=JMM_BOUNDARY_WALLS, vol_move=JMM_VOLMOVE_LNL,
                      vol_schedule=JMM_VOLSCHED_SWEEP, precision=JMM_PREC_FAST,
                      resum_sweeps=100, lanes_per_chain=0, steps_per_round=0,
                      chains_per_block=0, init=JMM_INIT_LATTICE, jitter=0.0, window=0,
                      split_n=0):
    c = BatchConfig()
    c.seed = seed
    c.boundary = boundary
    c.vol_move = vol_move
    c.vol_schedule = vol_schedule
    c.precision = precision
    c.resum_sweeps = resum_sweeps
    c.lanes_per_chain = lanes_per_chain
    c.steps_per_round = steps_per_round
    c.chains_per_block = chains_per_block
    c.init = init
    c.jitter = jitter
    c.window = window
    c.split_n = split_n
    return c


# ---- energy gradients -------------------------------------------------------
class GradChain(C.Structure):
    _fields_ = [
        ("x_off", C.c_uint64),
        ("n", C.c_uint32),
        ("potential", C.c_int32),
        ("eps", C.c_double),
        ("sigma", C.c_double),
        ("cutoff", C.c_double),
        ("l", C.c_double),
    ]


class GradStats(C.Structure):
    _fields_ = [
        ("samples", C.c_uint64),
        ("sum_u", C.c_double),
        ("sum_u2", C.c_double),
        ("sum_rho", C.c_double),
        ("sum_rho2", C.c_double),
        ("sum_l", C.c_double),
        ("sum_g", C.c_double * 3),
        ("sum_u_g", C.c_double * 3),
        ("sum_rho_g", C.c_double * 3),
        ("sum_l_g", C.c_double * 3),
    ]


GRAD_STATS_DTYPE = [
    ("samples", "<u8"), ("sum_u", "<f8"), ("sum_u2", "<f8"), ("sum_rho", "<f8"),
    ("sum_rho2", "<f8"), ("sum_l", "<f8"), ("sum_g", "<f8", (3,)), ("sum_u_g", "<f8", (3,)),
    ("sum_rho_g", "<f8", (3,)), ("sum_l_g", "<f8", (3,)),
]


JMM_LARGE_DOMAINS = 0
JMM_LARGE_SEQUENTIAL = 1


class LargeResult(C.Structure):
    _fields_ = [
        ("e", C.c_double),
        ("l", C.c_double),
        ("sweeps", C.c_uint64),
        ("samples", C.c_uint64),
        ("sum_e", C.c_double),
        ("sum_e2", C.c_double),
        ("moves", C.c_uint64),
        ("accepted", C.c_uint64),
        ("pair_evals", C.c_uint64),
        ("window_overflows", C.c_uint64),
        ("max_drift", C.c_double),
        ("grid", C.c_double),
        ("error", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


LARGE_RESULT_DTYPE = [
    ("e", "<f8"), ("l", "<f8"), ("sweeps", "<u8"), ("samples", "<u8"), ("sum_e", "<f8"),
    ("sum_e2", "<f8"), ("moves", "<u8"), ("accepted", "<u8"), ("pair_evals", "<u8"),
    ("window_overflows", "<u8"), ("max_drift", "<f8"), ("grid", "<f8"), ("error", "<u4"),
    ("reserved", "<u4"),
]


class RelaxStep(C.Structure):
    _fields_ = [("e_up", C.c_double), ("e_down", C.c_double), ("dl", C.c_double),
                ("l", C.c_double), ("e", C.c_double)]


RELAX_STEP_DTYPE = [("e_up", "<f8"), ("e_down", "<f8"), ("dl", "<f8"), ("l", "<f8"),
                    ("e", "<f8")]
