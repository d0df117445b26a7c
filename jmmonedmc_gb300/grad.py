"""Energy gradients for torch: the backward of the chains' total energy.

``chain_energy(x, l, eps, sigma, layout)`` returns U per chain and is
differentiable (through ``ChainEnergy``, a ``torch.autograd.Function``)
with respect to the positions (forces), the box lengths (the virial term,
positions scaled with the box) and the potential parameters eps and sigma.
Forward and backward both come from one launch of the hand-written kernel
behind ``jmm_energy_grad`` (include/jmm_gpu.h): FP32 pair terms, FP64 sums.
This module is the thin PyTorch layer of the gradient tooling; the Monte
Carlo kernels do not depend on it.

``fluctuation_gradients`` turns a sampled batch run's statistics
(``ChainBatch.run_sampled``) into d<A>/dtheta = <dA/dtheta>
- beta (<A dU/dtheta> - <A><dU/dtheta>) for A = U, rho, L and
theta = eps, sigma.
"""
import ctypes as C

import numpy as np

from . import _native, abi

P = C.POINTER
_native.register({
    "jmm_energy_grad": [C.c_void_p, C.c_uint32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                        C.c_void_p],
    "jmm_batch_energy_grad": [C.c_void_p, P(C.c_double), C.c_uint32],
    "jmm_batch_run_sampled": [C.c_void_p, C.c_uint64, C.c_uint32],
    "jmm_batch_run_sampled_async": [C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p],
    "jmm_batch_grad_stats": [C.c_void_p, P(abi.GradStats), C.c_uint32],
})


class Layout:
    """Where each chain's positions sit in one flat float32 tensor."""

    def __init__(self, sizes, potential=abi.JMM_POT_LJCUT, cutoff=3.0,
                 boundary=abi.JMM_BOUNDARY_WALLS):
        self.sizes = [int(n) for n in sizes]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.uint64)
        self.potential = potential
        self.cutoff = float(cutoff)
        self.boundary = boundary

    @property
    def n_chains(self):
        return len(self.sizes)

    def chain_index(self, device):
        import torch
        idx = np.repeat(np.arange(self.n_chains), self.sizes)
        return torch.as_tensor(idx, device=device)

    def table(self, l, eps, sigma, device):
        """The device array of jmm_grad_chain for these parameters."""
        import torch
        arr = (abi.GradChain * self.n_chains)()
        lv, ev, sv = (t.detach().double().cpu().numpy() for t in (l, eps, sigma))
        for k in range(self.n_chains):
            arr[k].x_off = int(self.offsets[k])
            arr[k].n = self.sizes[k]
            arr[k].potential = self.potential
            arr[k].eps = float(ev[k])
            arr[k].sigma = float(sv[k])
            arr[k].cutoff = self.cutoff
            arr[k].l = float(lv[k])
        raw = np.frombuffer(arr, dtype=np.uint8).copy()
        return torch.as_tensor(raw, device=device)


def _check(layout, x, l, eps, sigma):
    """The kernel reads x and the table on the device with no sizes of its
    own, so shapes and the device are checked here, before any launch."""
    n_pos = sum(layout.sizes)
    if x.numel() != n_pos:
        raise ValueError(f"x holds {x.numel()} positions, the layout {n_pos}")
    for name, t in (("l", l), ("eps", eps), ("sigma", sigma)):
        if t.numel() != layout.n_chains:
            raise ValueError(f"{name} needs one value per chain ({layout.n_chains})")
    if not x.is_cuda:
        raise ValueError("x must be a CUDA tensor: the gradient kernel reads it on the device")


def _launch(layout, x, l, eps, sigma, want_forces):
    import torch
    _check(layout, x, l, eps, sigma)
    dev = x.device
    table = layout.table(l, eps, sigma, dev)
    out = torch.empty((layout.n_chains, 4), dtype=torch.float64, device=dev)
    forces = torch.empty_like(x) if want_forces else None
    stream = torch.cuda.current_stream(dev).cuda_stream
    _native.call("jmm_energy_grad", table.data_ptr(), layout.n_chains, x.data_ptr(),
                 layout.boundary, out.data_ptr(), forces.data_ptr() if want_forces else None,
                 stream or None)
    return out, forces


def energy_and_gradients(x, l, eps, sigma, layout, forces=False):
    """(U, dU/deps, dU/dsigma, dU/dL) per chain, and -dU/dx if asked."""
    x = x.contiguous().float()
    return _launch(layout, x, l, eps, sigma, forces)


def _autograd_function():
    import torch

    class ChainEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, l, eps, sigma, layout):
            x = x.contiguous().float()
            out, forces = _launch(layout, x, l, eps, sigma, True)
            ctx.layout = layout
            ctx.save_for_backward(out, forces)
            return out[:, 0].clone()

        @staticmethod
        def backward(ctx, g_u):
            out, forces = ctx.saved_tensors
            layout = ctx.layout
            g = g_u.double()
            idx = layout.chain_index(forces.device)
            g_x = (-forces.double() * g[idx]).to(forces.dtype)
            return g_x, g * out[:, 3], g * out[:, 1], g * out[:, 2], None

    return ChainEnergy


_ChainEnergy = None


def chain_energy(x, l, eps, sigma, layout):
    """U per chain (float64), differentiable in x, l, eps and sigma."""
    global _ChainEnergy
    if _ChainEnergy is None:
        _ChainEnergy = _autograd_function()
    return _ChainEnergy.apply(x, l, eps, sigma, layout)


def fluctuation_gradients(stats, t, n=None):
    """d<A>/dtheta per chain from jmm_grad_stats (numpy structured array).

    Returns a dict with keys like 'dU_deps', 'dU_dsigma', 'drho_deps',
    'drho_dsigma', 'dL_deps', 'dL_dsigma' (A does not depend on theta
    explicitly except U: d<U>/dtheta adds <dU/dtheta>)."""
    s = stats["samples"].astype(np.float64)
    beta = 1.0 / np.asarray(t, dtype=np.float64)
    mean = lambda key: stats[key] / (s if stats[key].ndim == 1 else s[:, None])
    g = mean("sum_g")
    out = {}
    names = ("eps", "sigma")
    for k, th in enumerate(names):
        cov_u = mean("sum_u_g")[:, k] - mean("sum_u") * g[:, k]
        cov_rho = mean("sum_rho_g")[:, k] - mean("sum_rho") * g[:, k]
        cov_l = mean("sum_l_g")[:, k] - mean("sum_l") * g[:, k]
        out[f"dU_d{th}"] = g[:, k] - beta * cov_u
        out[f"drho_d{th}"] = -beta * cov_rho
        out[f"dL_d{th}"] = -beta * cov_l
    return out
