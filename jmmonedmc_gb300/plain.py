"""Python handle on the plain one-chain FP64 form (jmm_plain_* in include/jmm_gpu.h).

Mirrors the reference's MCState API (src/jmmMCState.h:6-48) for scripting
and tests: ``PlainChain.fad`` is fad, ``steps`` is incrementStep+Step,
``echeck`` is ECheck, ``update_thermo`` is updateThermo.  The C++ drop-in
(jmmonedmc_gb300/dropin/jmmMCState.cpp) drives the same C ABI.
"""
import ctypes as C

import numpy as np

from . import _native, abi


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
