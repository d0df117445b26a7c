"""Python handle on the plain one-chain FP64 form (jmm_plain_* in include/jmm_gpu.h).

Mirrors the reference's MCState API (src/jmmMCState.h:6-48) for scripting
and tests: ``PlainChain.fad`` is fad, ``steps`` is incrementStep+Step,
``echeck`` is ECheck, ``update_thermo`` is updateThermo.  The C++ drop-in
(jmmonedmc_gb300/dropin/jmmMCState.cpp) drives the same C ABI.
"""
import ctypes as C

import numpy as np

from . import _native, abi

P = C.POINTER
_native.register({
    "jmm_plain_histograms": [C.c_void_p, C.c_uint64, C.c_double, C.c_int32, C.c_double,
                             C.c_uint64, C.c_double],
    "jmm_plain_take_rho": [C.c_void_p, P(C.c_int32), C.c_uint64],
    "jmm_plain_take_g": [C.c_void_p, P(C.c_int32), C.c_uint64],
    "jmm_plain_hist_counts": [C.c_void_p, P(C.c_int32), C.c_uint64, P(C.c_int32), C.c_uint64],
    "jmm_plain_relax_volume": [C.c_void_p, C.c_void_p, P(C.c_int32), P(C.c_int32)],
    "jmm_plain_trial_volume_energy": [C.c_void_p, C.c_double, P(C.c_double)],
    "jmm_plain_move_volume": [C.c_void_p, C.c_double],
})


class PlainChain:
    def __init__(self, params: abi.Params):
        self._h = C.c_void_p()
        self.params = params
        _native.call("jmm_plain_create", C.byref(params), C.byref(self._h))

    @classmethod
    def from_kwargs(cls, **kw):
        return cls(abi.make_params(**kw))

    @property
    def n(self):
        return int(self.params.n)

    def close(self):
        if self._h:
            _native.load().jmm_plain_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- reference API -------------------------------------------------------
    def fad(self, nm=0, d=0.5):
        _native.call("jmm_plain_fad", self._h, nm, d)

    def steps(self, n_steps, replay=None, log=False):
        """Run n_steps; replay is a structured array/list of (nm, rn, ran)."""
        rp = None
        if replay is not None:
            arr = (abi.Draw * n_steps)()
            for k in range(n_steps):
                arr[k].nm, arr[k].rn, arr[k].ran = (int(replay[k][0]), float(replay[k][1]),
                                                    float(replay[k][2]))
            rp = C.cast(arr, C.c_void_p)
        rec = None
        if log:
            rec = (abi.StepRecord * n_steps)()
        _native.call("jmm_plain_steps", self._h, n_steps, rp,
                     C.cast(rec, C.c_void_p) if rec is not None else None)
        if rec is not None:
            return np.frombuffer(rec, dtype=np.dtype(abi.STEP_RECORD_DTYPE)).copy()
        return None

    def move(self, kind, nm, rn):
        """One trial outside Step (qad2 of particle nm, or the volume move)."""
        rec = abi.StepRecord()
        _native.call("jmm_plain_move", self._h, kind, nm, rn, C.byref(rec))
        return rec

    def set_config(self, r, l, sn=0):
        r = np.ascontiguousarray(r, dtype=np.float64)
        _native.call("jmm_plain_set_config", self._h,
                     r.ctypes.data_as(C.POINTER(C.c_double)), r.size, l, sn)

    def update_thermo(self):
        _native.call("jmm_plain_update_thermo", self._h)

    def reset_thermo(self):
        _native.call("jmm_plain_reset_thermo", self._h)

    def echeck(self):
        e = C.c_double()
        reset = C.c_int32()
        _native.call("jmm_plain_echeck", self._h, C.byref(e), C.byref(reset))
        return e.value, bool(reset.value)

    def set_step_sizes(self, max_step, max_dl):
        _native.call("jmm_plain_set_step_sizes", self._h, max_step, max_dl)

    def state(self):
        st = abi.State()
        _native.call("jmm_plain_get_state", self._h, C.byref(st))
        return st

    def positions(self):
        r = np.empty(self.n, dtype=np.float64)
        _native.call("jmm_plain_get_positions", self._h,
                     r.ctypes.data_as(C.POINTER(C.c_double)), self.n)
        return r

    def separations(self):
        m = self.n * (self.n - 1) // 2
        rij = np.empty(m, dtype=np.float64)
        _native.call("jmm_plain_get_separations", self._h,
                     rij.ctypes.data_as(C.POINTER(C.c_double)), m)
        return rij

    # --- rho(x) and g(x) histograms (fgrho/ugrho/qagrho, printRho/printG) ----
    def histograms(self, rhonb, rbw, gns, gsw, gnb, gbw):
        self._hist = (int(rhonb), int(gns), int(gnb))
        _native.call("jmm_plain_histograms", self._h, rhonb, rbw, gns, gsw, gnb, gbw)

    def take_rho(self):
        out = np.empty(self._hist[0], dtype=np.int32)
        _native.call("jmm_plain_take_rho", self._h, out.ctypes.data_as(P(C.c_int32)), out.size)
        return out

    def take_g(self):
        rhonb, gns, gnb = self._hist
        out = np.empty(gns * gnb, dtype=np.int32)
        _native.call("jmm_plain_take_g", self._h, out.ctypes.data_as(P(C.c_int32)), out.size)
        return out.reshape(gns, gnb)

    def hist_counts(self):
        rhonb, gns, gnb = self._hist
        rho = np.empty(rhonb, dtype=np.int32)
        g = np.empty(gns * gnb, dtype=np.int32)
        _native.call("jmm_plain_hist_counts", self._h, rho.ctypes.data_as(P(C.c_int32)), rhonb,
                     g.ctypes.data_as(P(C.c_int32)), g.size)
        return rho, g.reshape(gns, gnb)

    # --- volume relaxation (relaxVolume, calculateEnergyOfTrialVolumeChange, moveVolume)
    def relax_volume(self):
        """Returns (per-step records, converged)."""
        log = (abi.RelaxStep * 20)()
        n, conv = C.c_int32(), C.c_int32()
        _native.call("jmm_plain_relax_volume", self._h, C.cast(log, C.c_void_p), C.byref(n),
                     C.byref(conv))
        return (np.frombuffer(log, dtype=np.dtype(abi.RELAX_STEP_DTYPE))[:n.value].copy(),
                bool(conv.value))

    def trial_volume_energy(self, dl):
        e = C.c_double()
        _native.call("jmm_plain_trial_volume_energy", self._h, dl, C.byref(e))
        return e.value

    def move_volume(self, l):
        _native.call("jmm_plain_move_volume", self._h, l)


def _main(argv=None):
    """Steps/s of one plain chain: python -m jmmonedmc_gb300.plain [--n 256] [--npt]."""
    import argparse
    import time
    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--npt", action="store_true", help="NPT with linear dL moves (default NLT)")
    ap.add_argument("--rho", type=float, default=0.6)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=200)
    args = ap.parse_args(argv)
    params = abi.make_params(n=args.n, ensemble=abi.JMM_NPT if args.npt else abi.JMM_NLT,
                             l=args.n / args.rho, p=1.0, t=1.0, cutoff=3.0, max_step=0.3,
                             max_dl=1.0, seed=1, eci=0)
    chain = PlainChain(params)
    chain.fad()
    chain.steps(args.warmup)
    t0 = time.perf_counter()
    chain.steps(args.steps)
    dt = time.perf_counter() - t0
    print(f"plain form, N = {args.n} {'NPT' if args.npt else 'NLT'}: {args.steps / dt:.0f} steps/s")


if __name__ == "__main__":
    _main()
