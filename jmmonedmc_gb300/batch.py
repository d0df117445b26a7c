"""Python handle on the batched chain form (jmm_batch_* in include/jmm_gpu.h).

``ChainBatch`` owns thousands of independent Metropolis chains of uneven N,
temperature, pressure and potential that run in one persistent CUDA kernel;
``run(n_sweeps)`` launches a CUDA graph holding that kernel.  Statistics come
back as a numpy structured array (``CHAIN_RESULT_DTYPE``), with helpers for
the averages the reference's analysis scripts form (scripts/Analyze_Mean.py).
"""
import ctypes as C

import numpy as np

from . import _native, abi

P = C.POINTER
_native.register({
    "jmm_batch_create": [P(abi.BatchConfig), P(abi.ChainDesc), C.c_uint32, P(C.c_void_p)],
    "jmm_batch_create_at": [P(abi.BatchConfig), P(abi.ChainDesc), C.c_uint32, P(C.c_float),
                            P(C.c_void_p)],
    "jmm_batch_histograms": [C.c_void_p, C.c_uint32, C.c_double, C.c_uint32, C.c_double,
                             C.c_uint32, C.c_double],
    "jmm_batch_sample_histograms": [C.c_void_p, C.c_void_p],
    "jmm_batch_take_histograms": [C.c_void_p, P(C.c_uint64), C.c_uint64],
    "jmm_batch_run": [C.c_void_p, C.c_uint64],
    "jmm_batch_run_async": [C.c_void_p, C.c_uint64, C.c_void_p],
    "jmm_batch_results": [C.c_void_p, P(abi.ChainResult), C.c_uint32],
    "jmm_batch_set_results": [C.c_void_p, P(abi.ChainResult), C.c_uint32],
    "jmm_batch_reset_stats": [C.c_void_p],
    "jmm_batch_get_positions": [C.c_void_p, C.c_uint32, P(C.c_float), C.c_uint32],
    "jmm_batch_set_positions": [C.c_void_p, C.c_uint32, P(C.c_float), C.c_uint32, C.c_double],
    "jmm_batch_energies": [C.c_void_p, P(C.c_double), C.c_uint32],
    "jmm_batch_volume_energies": [C.c_void_p, P(C.c_float), P(C.c_double), C.c_uint32],
    "jmm_batch_device_views": [C.c_void_p, P(C.c_void_p), P(C.c_void_p), P(C.c_uint64),
                               C.c_uint32],
    "jmm_batch_autotune": [C.c_void_p, C.c_uint32, P(C.c_uint32), P(C.c_uint32),
                           P(C.c_uint32)],
    "jmm_batch_destroy": [C.c_void_p],
    "jmm_batch_run_host": [P(abi.BatchConfig), P(abi.ChainDesc), C.c_uint32, P(C.c_float),
                           C.c_uint64, P(abi.ChainResult), P(C.c_float)],
    "jmm_rng_words": [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint64, P(C.c_uint32)],
    "jmm_batch_adjust_steps": [C.c_void_p, C.c_double, C.c_int32],
    "jmm_batch_shapes": [C.c_void_p, P(C.c_uint32), C.c_uint32],
    "jmm_batch_step_sizes": [C.c_void_p, P(C.c_double), P(C.c_double), C.c_uint32],
})


def chain_array(chains):
    """A ctypes array of jmm_chain_desc: chains itself if it already is one."""
    if isinstance(chains, C.Array) and chains._type_ is abi.ChainDesc:
        return chains
    arr = (abi.ChainDesc * len(chains))()
    for k, c in enumerate(chains):
        arr[k] = c
    return arr


def chain_view(arr):
    """A numpy structured view of a ctypes jmm_chain_desc array (shares memory)."""
    return np.frombuffer(arr, dtype=np.dtype(abi.ChainDesc))


def results_to_numpy(buf):
    return np.frombuffer(buf, dtype=np.dtype(abi.CHAIN_RESULT_DTYPE)).copy()


class ChainBatch:
    def __init__(self, config: abi.BatchConfig, chains, x=None):
        """chains: a sequence of ChainDesc or a ctypes array of them.  x: the
        chains' starting positions back to back (box lengths l0); None starts
        them on the configured lattice."""
        self.config = config
        self._arr = chain_array(chains)
        self.chains = self._arr
        self._h = C.c_void_p()
        self._hist = None
        if x is None:
            _native.call("jmm_batch_create", C.byref(config), self._arr, len(self._arr),
                         C.byref(self._h))
        else:
            x = np.ascontiguousarray(x, dtype=np.float32)
            if x.size != int(chain_view(self._arr)["n"].sum()):
                raise ValueError("x must hold every chain's positions back to back")
            _native.call("jmm_batch_create_at", C.byref(config), self._arr, len(self._arr),
                         x.ctypes.data_as(P(C.c_float)), C.byref(self._h))

    @property
    def n_chains(self):
        return len(self.chains)

    def close(self):
        if self._h:
            _native.load().jmm_batch_destroy(self._h)
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

    def run(self, n_sweeps):
        _native.call("jmm_batch_run", self._h, n_sweeps)

    def run_async(self, n_sweeps, stream=None):
        """Enqueue on a CUDA stream handle (int, e.g. torch's cuda_stream)."""
        _native.call("jmm_batch_run_async", self._h, n_sweeps,
                     C.c_void_p(stream) if stream else None)

    def results(self):
        buf = (abi.ChainResult * self.n_chains)()
        _native.call("jmm_batch_results", self._h, buf, self.n_chains)
        return results_to_numpy(buf)

    def set_results(self, res):
        """Replaces every chain's record (a structured array as results() gives)."""
        res = np.ascontiguousarray(res, dtype=np.dtype(abi.CHAIN_RESULT_DTYPE))
        if res.shape != (self.n_chains,):
            raise ValueError("one record per chain")
        buf = (abi.ChainResult * self.n_chains).from_buffer_copy(res.tobytes())
        _native.call("jmm_batch_set_results", self._h, buf, self.n_chains)

    # --- checkpoint / resume
    def checkpoint(self, path):
        """Saves the batch (configuration with its launch shape, chains with
        their current step sizes and box lengths, positions, records) to a
        .npz file; restore() continues it exactly.  (A FAST batch whose
        potential classes were tuned to different shapes restarts on the
        per-class defaults: the same chains statistically, not bit for bit.)"""
        res = self.results()
        config = abi.BatchConfig.from_buffer_copy(bytes(self.config))
        shapes = set(self.shapes().values())
        if len(shapes) == 1:
            (config.lanes_per_chain, config.steps_per_round, config.chains_per_block,
             config.window) = shapes.pop()
        desc = (abi.ChainDesc * self.n_chains).from_buffer_copy(bytes(self._arr))
        view = chain_view(desc)
        view["max_step"], view["vol_step"] = self.step_sizes()
        view["l0"] = res["l"]
        x = np.concatenate([self.positions(k) for k in range(self.n_chains)])
        np.savez(path, config=np.frombuffer(bytes(config), dtype=np.uint8),
                 chains=np.frombuffer(bytes(desc), dtype=np.uint8), positions=x, results=res)

    @classmethod
    def restore(cls, path):
        """A batch from a checkpoint() file, in the checkpointed state."""
        with np.load(path) as f:
            config = abi.BatchConfig.from_buffer_copy(f["config"].tobytes())
            raw = f["chains"].tobytes()
            n = len(raw) // C.sizeof(abi.ChainDesc)
            desc = (abi.ChainDesc * n).from_buffer_copy(raw)
            b = cls(config, desc, x=f["positions"])
            b.set_results(f["results"])
        return b

    def reset_stats(self):
        _native.call("jmm_batch_reset_stats", self._h)

    def adjust_steps(self, ideal_ratio=0.5, displacement=True, volume=True):
        """maxDisAdjust / maxDVAdjust on the device from each chain's counts."""
        what = (1 if displacement else 0) | (2 if volume else 0)
        _native.call("jmm_batch_adjust_steps", self._h, ideal_ratio, what)

    def step_sizes(self):
        """(max displacement, volume step) per chain, float64 arrays."""
        ms = np.empty(self.n_chains, dtype=np.float64)
        vs = np.empty(self.n_chains, dtype=np.float64)
        _native.call("jmm_batch_step_sizes", self._h, ms.ctypes.data_as(P(C.c_double)),
                     vs.ctypes.data_as(P(C.c_double)), self.n_chains)
        return ms, vs

    def positions(self, chain):
        n = self.chains[chain].n
        x = np.empty(n, dtype=np.float32)
        _native.call("jmm_batch_get_positions", self._h, chain,
                     x.ctypes.data_as(P(C.c_float)), n)
        return x

    def set_positions(self, chain, x, l):
        x = np.ascontiguousarray(x, dtype=np.float32)
        _native.call("jmm_batch_set_positions", self._h, chain,
                     x.ctypes.data_as(P(C.c_float)), x.size, float(l))

    def energies(self):
        e = np.empty(self.n_chains, dtype=np.float64)
        _native.call("jmm_batch_energies", self._h, e.ctypes.data_as(P(C.c_double)),
                     self.n_chains)
        return e

    def volume_energies(self, scale):
        """(U_old, U_new, U_new - U_old) per chain, float64 (n_chains, 3): the
        energies a volume move of each chain would compare, positions and box
        scaled by scale[k] (as the chain kernel's volume move forms them)."""
        scale = np.ascontiguousarray(scale, dtype=np.float32)
        if scale.shape != (self.n_chains,):
            raise ValueError("one scale factor per chain")
        out = np.empty((self.n_chains, 3), dtype=np.float64)
        _native.call("jmm_batch_volume_energies", self._h, scale.ctypes.data_as(P(C.c_float)),
                     out.ctypes.data_as(P(C.c_double)), self.n_chains)
        return out

    def device_views(self):
        """(positions device address, results device address, offsets)."""
        px, pr = C.c_void_p(), C.c_void_p()
        off = np.empty(self.n_chains, dtype=np.uint64)
        _native.call("jmm_batch_device_views", self._h, C.byref(px), C.byref(pr),
                     off.ctypes.data_as(P(C.c_uint64)), self.n_chains)
        return px.value, pr.value, off

    def energy_grad(self):
        """(U, dU/deps, dU/dsigma, dU/dL) of every chain's current configuration."""
        from . import grad  # noqa: F401  (registers the entry points)
        out = np.empty((self.n_chains, 4), dtype=np.float64)
        _native.call("jmm_batch_energy_grad", self._h, out.ctypes.data_as(P(C.c_double)),
                     self.n_chains)
        return out

    def run_sampled(self, n_sweeps, sample_every=10):
        """n_sweeps sweeps, sampling U and its gradient every sample_every sweeps."""
        from . import grad  # noqa: F401
        _native.call("jmm_batch_run_sampled", self._h, n_sweeps, sample_every)

    def run_sampled_async(self, n_sweeps, sample_every=10, stream=None):
        """Enqueue run_sampled on a CUDA stream handle (int, None = the batch's)."""
        from . import grad  # noqa: F401
        _native.call("jmm_batch_run_sampled_async", self._h, n_sweeps, sample_every,
                     C.c_void_p(stream) if stream else None)

    def grad_stats(self):
        from . import grad  # noqa: F401
        buf = (abi.GradStats * self.n_chains)()
        _native.call("jmm_batch_grad_stats", self._h, buf, self.n_chains)
        return np.frombuffer(buf, dtype=np.dtype(abi.GRAD_STATS_DTYPE)).copy()

    # --- sampled rho(x) / g(x) histograms
    def histograms(self, rhonb, rbw, gns, gsw, gnb, gbw):
        """Configures (and clears) the chains' sampled histograms: rhonb
        position bins of width rbw, gns slices of width gsw x gnb separation
        bins of width gbw (the reference's RHONB/RBW/GNS/GSW/GNB/GBW)."""
        _native.call("jmm_batch_histograms", self._h, rhonb, rbw, gns, gsw, gnb, gbw)
        self._hist = (rhonb, gns, gnb)

    def sample_histograms(self, stream=None):
        """Adds the current configuration of every chain (enqueued)."""
        _native.call("jmm_batch_sample_histograms", self._h,
                     C.c_void_p(stream) if stream else None)

    def take_histograms(self):
        """{"samples": (chains,), "rho": (chains, rhonb), "g": (chains, gns, gnb)}."""
        if self._hist is None:
            raise RuntimeError("take_histograms: histograms() has not configured this batch")
        rhonb, gns, gnb = self._hist
        width = 1 + rhonb + gns * gnb
        out = np.empty(self.n_chains * width, dtype=np.uint64)
        _native.call("jmm_batch_take_histograms", self._h, out.ctypes.data_as(P(C.c_uint64)),
                     out.size)
        rows = out.reshape(self.n_chains, width)
        return {"samples": rows[:, 0].copy(), "rho": rows[:, 1:1 + rhonb].copy(),
                "g": rows[:, 1 + rhonb:].reshape(self.n_chains, gns, gnb).copy()}

    def autotune(self, trial_sweeps=4):
        """(lanes_per_chain, steps_per_round, chains_per_block) chosen."""
        g, s, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        _native.call("jmm_batch_autotune", self._h, trial_sweeps, C.byref(g), C.byref(s),
                     C.byref(c))
        return g.value, s.value, c.value

    def shapes(self):
        """{potential: (lanes, steps per round, chains per block, neighbours
        per side)} of the classes present (LJcut, soft sphere, Gaussian core)."""
        out = (C.c_uint32 * 12)()
        _native.call("jmm_batch_shapes", self._h, out, 12)
        pots = (abi.JMM_POT_LJCUT, abi.JMM_POT_SOFTSPHERE, abi.JMM_POT_GAUSS)
        return {p: tuple(out[4 * k:4 * k + 4]) for k, p in enumerate(pots) if out[4 * k]}


def run_host(config, chains, n_sweeps, x_in=None):
    """Create, run and read back in one call through host buffers.  chains is
    a sequence of ChainDesc or a ctypes array of them (passed as it is)."""
    arr = chain_array(chains)
    n_tot = int(chain_view(arr)["n"].sum())
    res = (abi.ChainResult * len(chains))()
    x_out = np.empty(n_tot, dtype=np.float32)
    xin_ptr = None
    if x_in is not None:
        x_in = np.ascontiguousarray(x_in, dtype=np.float32)
        if x_in.size != n_tot:
            raise ValueError(f"x_in holds {x_in.size} positions, the chains {n_tot}")
        xin_ptr = x_in.ctypes.data_as(P(C.c_float))
    _native.call("jmm_batch_run_host", C.byref(config), arr, len(chains), xin_ptr, n_sweeps,
                 res, x_out.ctypes.data_as(P(C.c_float)))
    return results_to_numpy(res), x_out


def rng_words(seed, block0, chain, count):
    out = np.empty(4 * count, dtype=np.uint32)
    _native.call("jmm_rng_words", seed, block0, chain, count,
                 out.ctypes.data_as(P(C.c_uint32)))
    return out.reshape(count, 4)


def averages(res):
    """Per-chain <E>, <E^2>, <L>, <L^2>, <LE>, <rho>, <rho^2> from the sums."""
    s = res["samples"].astype(np.float64)
    out = {}
    for k in ("e", "e2", "l", "l2", "le", "rho", "rho2"):
        out[k] = res["sum_" + k] / s
    return out
