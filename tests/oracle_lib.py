"""ctypes handle on the oracle's CPU library (oracle/_build/libjmmoracle.so).

Test infrastructure: the CPU restatement that the CUDA paths are checked
against.  It shares the public structs of include/jmm_gpu.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from jmmonedmc_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(REPO, "oracle", "_build", "libjmmoracle.so")
_lib = None

P = C.POINTER
u64, i32, u32, dbl, vp = C.c_uint64, C.c_int32, C.c_uint32, C.c_double, C.c_void_p

SIGS = {
    "jmmo_plain_create": ([P(abi.Params)], vp),
    "jmmo_plain_set_config": ([vp, P(dbl), u64, dbl, u64], C.c_int),
    "jmmo_plain_fad": ([vp, u64, dbl], C.c_int),
    "jmmo_plain_steps": ([vp, u64, vp, vp], C.c_int),
    "jmmo_plain_move": ([vp, i32, u64, dbl, vp], C.c_int),
    "jmmo_plain_update_thermo": ([vp], C.c_int),
    "jmmo_plain_reset_thermo": ([vp], C.c_int),
    "jmmo_plain_echeck": ([vp, P(dbl), P(i32)], C.c_int),
    "jmmo_plain_set_step_sizes": ([vp, dbl, dbl], C.c_int),
    "jmmo_plain_get_state": ([vp, P(abi.State)], C.c_int),
    "jmmo_plain_get_positions": ([vp, P(dbl), u64], C.c_int),
    "jmmo_plain_get_separations": ([vp, P(dbl), u64], C.c_int),
    "jmmo_plain_destroy": ([vp], None),
    "jmmo_plain_histograms": ([vp, u64, dbl, i32, dbl, u64, dbl], C.c_int),
    "jmmo_plain_take_rho": ([vp, P(i32), u64], C.c_int),
    "jmmo_plain_take_g": ([vp, P(i32), u64], C.c_int),
    "jmmo_plain_hist_counts": ([vp, P(i32), u64, P(i32), u64], C.c_int),
    "jmmo_plain_trial_volume_energy": ([vp, dbl], dbl),
    "jmmo_plain_move_volume": ([vp, dbl], C.c_int),
    "jmmo_phi": ([i32, dbl, dbl, i32, dbl, P(dbl)], None),
    "jmmo_plain_relax_volume": ([vp, vp, P(i32)], C.c_int),
    "jmmo_philox_raw": ([P(u32), P(u32), P(u32)], None),
    "jmmo_step_words_export": ([u64, u64, u32, P(u32)], None),
}


def reference_sources():
    """The reference's src directory where it is present (the oracle's build
    recipe knows where), else None."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "build_oracle", os.path.join(REPO, "oracle", "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.reference_sources()


def extra_sigs(sigs):
    SIGS.update(sigs)
    if _lib is not None:
        _bind(_lib)


def _bind(lib):
    for name, (args, res) in SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res


def load():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
        _lib = C.CDLL(LIB)
        _bind(_lib)
    return _lib


def _ok(rc, name):
    if rc != 0:
        raise RuntimeError(f"{name} returned {rc}")


class OraclePlain:
    """Same surface as jmmonedmc_gb300.plain.PlainChain, on the CPU."""

    def __init__(self, params):
        self.lib = load()
        self.params = params
        self._h = self.lib.jmmo_plain_create(C.byref(params))
        if not self._h:
            raise ValueError("jmmo_plain_create rejected the parameters")

    @property
    def n(self):
        return int(self.params.n)

    def close(self):
        if self._h:
            self.lib.jmmo_plain_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def fad(self, nm=0, d=0.5):
        _ok(self.lib.jmmo_plain_fad(self._h, nm, d), "fad")

    def steps(self, n_steps, replay=None, log=False):
        rp = None
        if replay is not None:
            arr = (abi.Draw * n_steps)()
            for k in range(n_steps):
                arr[k].nm, arr[k].rn, arr[k].ran = (int(replay[k][0]), float(replay[k][1]),
                                                    float(replay[k][2]))
            rp = C.cast(arr, C.c_void_p)
        rec = (abi.StepRecord * n_steps)() if log else None
        _ok(self.lib.jmmo_plain_steps(self._h, n_steps, rp,
                                      C.cast(rec, C.c_void_p) if rec is not None else None),
            "steps")
        if rec is not None:
            return np.frombuffer(rec, dtype=np.dtype(abi.STEP_RECORD_DTYPE)).copy()
        return None

    def move(self, kind, nm, rn):
        rec = abi.StepRecord()
        _ok(self.lib.jmmo_plain_move(self._h, kind, nm, rn, C.byref(rec)), "move")
        return rec

    def set_config(self, r, l, sn=0):
        r = np.ascontiguousarray(r, dtype=np.float64)
        _ok(self.lib.jmmo_plain_set_config(self._h, r.ctypes.data_as(P(dbl)), r.size, l, sn),
            "set_config")

    def update_thermo(self):
        _ok(self.lib.jmmo_plain_update_thermo(self._h), "update_thermo")

    def reset_thermo(self):
        _ok(self.lib.jmmo_plain_reset_thermo(self._h), "reset_thermo")

    def echeck(self):
        e = C.c_double()
        reset = C.c_int32()
        _ok(self.lib.jmmo_plain_echeck(self._h, C.byref(e), C.byref(reset)), "echeck")
        return e.value, bool(reset.value)

    def set_step_sizes(self, max_step, max_dl):
        _ok(self.lib.jmmo_plain_set_step_sizes(self._h, max_step, max_dl), "set_step_sizes")

    def state(self):
        st = abi.State()
        _ok(self.lib.jmmo_plain_get_state(self._h, C.byref(st)), "get_state")
        return st

    def positions(self):
        r = np.empty(self.n, dtype=np.float64)
        _ok(self.lib.jmmo_plain_get_positions(self._h, r.ctypes.data_as(P(dbl)), self.n),
            "get_positions")
        return r

    def separations(self):
        m = self.n * (self.n - 1) // 2
        rij = np.empty(m, dtype=np.float64)
        _ok(self.lib.jmmo_plain_get_separations(self._h, rij.ctypes.data_as(P(dbl)), m),
            "get_separations")
        return rij

    def histograms(self, rhonb, rbw, gns, gsw, gnb, gbw):
        self._hist = (int(rhonb), int(gns), int(gnb))
        _ok(self.lib.jmmo_plain_histograms(self._h, rhonb, rbw, gns, gsw, gnb, gbw), "histograms")

    def take_rho(self):
        out = np.empty(self._hist[0], dtype=np.int32)
        _ok(self.lib.jmmo_plain_take_rho(self._h, out.ctypes.data_as(P(i32)), out.size),
            "take_rho")
        return out

    def take_g(self):
        rhonb, gns, gnb = self._hist
        out = np.empty(gns * gnb, dtype=np.int32)
        _ok(self.lib.jmmo_plain_take_g(self._h, out.ctypes.data_as(P(i32)), out.size), "take_g")
        return out.reshape(gns, gnb)

    def relax_volume(self):
        log = (abi.RelaxStep * 20)()
        n = C.c_int32()
        conv = self.lib.jmmo_plain_relax_volume(self._h, C.cast(log, C.c_void_p), C.byref(n))
        return np.frombuffer(log, dtype=np.dtype(abi.RELAX_STEP_DTYPE))[:n.value].copy(), bool(conv)

    def trial_volume_energy(self, dl):
        return self.lib.jmmo_plain_trial_volume_energy(self._h, dl)

    def move_volume(self, l):
        _ok(self.lib.jmmo_plain_move_volume(self._h, l), "move_volume")

    def hist_counts(self):
        rhonb, gns, gnb = self._hist
        rho = np.empty(rhonb, dtype=np.int32)
        g = np.empty(gns * gnb, dtype=np.int32)
        _ok(self.lib.jmmo_plain_hist_counts(self._h, rho.ctypes.data_as(P(i32)), rhonb,
                                            g.ctypes.data_as(P(i32)), g.size), "hist_counts")
        return rho, g.reshape(gns, gnb)



def philox_raw(ctr, key):
    lib = load()
    c = (u32 * 4)(*ctr)
    k = (u32 * 2)(*key)
    o = (u32 * 4)()
    lib.jmmo_philox_raw(c, k, o)
    return list(o)


def step_words(seed, block, chain=0):
    lib = load()
    o = (u32 * 4)()
    lib.jmmo_step_words_export(seed, block, chain, o)
    return list(o)


# ---- batched form ----------------------------------------------------------
extra_sigs({
    "jmmo_batch_create": ([P(abi.BatchConfig), P(abi.ChainDesc), u32, C.c_int], vp),
    "jmmo_batch_destroy": ([vp], None),
    "jmmo_batch_run": ([vp, u64], C.c_int),
    "jmmo_batch_run_chain": ([vp, u32, u64], C.c_int),
    "jmmo_batch_results": ([vp, P(abi.ChainResult), u32], C.c_int),
    "jmmo_batch_get_positions": ([vp, u32, P(dbl), u32], C.c_int),
    "jmmo_batch_set_positions": ([vp, u32, P(dbl), u32, dbl], C.c_int),
    "jmmo_batch_energies": ([vp, P(dbl), u32], C.c_int),
    "jmmo_energy64": ([P(abi.ChainDesc), P(dbl), dbl, C.c_int], dbl),
    "jmmo_energy_grad64": ([P(abi.ChainDesc), P(dbl), dbl, C.c_int, P(dbl)], None),
    "jmmo_batch_hist_sample": ([P(C.c_float), C.c_uint32, C.c_float, C.c_int, C.c_uint32,
                                C.c_float, C.c_uint32, C.c_float, C.c_uint32, C.c_float,
                                P(C.c_uint64)], None),
    "jmmo_portable_logf": ([C.c_float], C.c_float),
    "jmmo_portable_expf": ([C.c_float], C.c_float),
})


class OracleBatch:
    """CPU restatement of jmm_batch_*: fp64=False replays the EXACT kernel."""

    def __init__(self, config, chains, fp64=False):
        from jmmonedmc_gb300.batch import chain_array
        self.lib = load()
        self.chains = list(chains)
        self._arr = chain_array(self.chains)
        self._h = self.lib.jmmo_batch_create(C.byref(config), self._arr, len(self.chains),
                                             1 if fp64 else 0)
        if not self._h:
            raise ValueError("jmmo_batch_create failed")

    @property
    def n_chains(self):
        return len(self.chains)

    def close(self):
        if self._h:
            self.lib.jmmo_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, n_sweeps):
        _ok(self.lib.jmmo_batch_run(self._h, n_sweeps), "batch_run")

    def run_chain(self, chain, n_sweeps):
        _ok(self.lib.jmmo_batch_run_chain(self._h, chain, n_sweeps), "batch_run_chain")

    def results(self):
        from jmmonedmc_gb300.batch import results_to_numpy
        buf = (abi.ChainResult * self.n_chains)()
        _ok(self.lib.jmmo_batch_results(self._h, buf, self.n_chains), "batch_results")
        return results_to_numpy(buf)

    def positions(self, chain):
        n = self.chains[chain].n
        x = np.empty(n, dtype=np.float64)
        _ok(self.lib.jmmo_batch_get_positions(self._h, chain, x.ctypes.data_as(P(dbl)), n),
            "batch_get_positions")
        return x

    def set_positions(self, chain, x, l):
        x = np.ascontiguousarray(x, dtype=np.float64)
        _ok(self.lib.jmmo_batch_set_positions(self._h, chain, x.ctypes.data_as(P(dbl)), x.size,
                                              float(l)), "batch_set_positions")

    def energies(self):
        e = np.empty(self.n_chains, dtype=np.float64)
        _ok(self.lib.jmmo_batch_energies(self._h, e.ctypes.data_as(P(dbl)), self.n_chains),
            "batch_energies")
        return e


def energy64(chain_desc, x, l, periodic=False):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib.jmmo_energy64(C.byref(chain_desc), x.ctypes.data_as(P(dbl)), float(l),
                             1 if periodic else 0)


def hist_sample(x, l, periodic, rhonb, rbw, gns, gsw, gnb, gbw, row=None):
    """Adds one histogram sample of a chain's FP32 positions to row (the
    batched form's layout: samples, rho bins, g bins); returns row."""
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float32)
    if row is None:
        row = np.zeros(1 + rhonb + gns * gnb, dtype=np.uint64)
    lib.jmmo_batch_hist_sample(x.ctypes.data_as(P(C.c_float)), x.size, float(l),
                               1 if periodic else 0, rhonb, rbw, gns, gsw, gnb, gbw,
                               row.ctypes.data_as(P(C.c_uint64)))
    return row


def energy_grad64(chain_desc, x, l, periodic=False):
    """FP64 (U, dU/deps, dU/dsigma, dU/dL) of one configuration."""
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = (dbl * 4)()
    lib.jmmo_energy_grad64(C.byref(chain_desc), x.ctypes.data_as(P(dbl)), float(l),
                           1 if periodic else 0, out)
    return np.array(out)


def phi(potential, d, cut, virial=True, l=1.0):
    """The plain form's pair function: phi[0..8] at separation d."""
    lib = load()
    out = (dbl * 9)()
    lib.jmmo_phi(potential, float(d), float(cut), 1 if virial else 0, float(l), out)
    return np.array(out)
