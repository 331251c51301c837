"""Spectral post-processing on the GPU: Gaussian line-spread function and rotational broadening.

``apply_LSF``, ``compute_LSF_matrix`` and ``apply_rotation`` mirror Korg's functions of the same
names (src/utils.jl:45-240: same arguments and meaning, wavelengths in A or cm as in Korg, R a
number or a function of wavelength in A).  Flux may be one spectrum or a stack (nspec, nwl): the
kernels share each output's weights across the stack.  ``LSF`` and ``Rotation`` are torch
autograd functions on device tensors (the reverse modes are the transposed maps), so fitting
code can differentiate through the post-processing after ``korg_gb300.autograd.Synthesis``.
Device memory is torch (plumbing); the work is the C library's.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .wavelengths import Wavelengths


def _grid(wls):
    return wls if isinstance(wls, Wavelengths) else Wavelengths(wls)


def _obs_cm(obs):
    o = np.asarray(obs, dtype=np.float64)
    return o * 1e-8 if o.size and o[0] >= 1 else o


def _R_values(R, out_cm):
    if callable(R):
        return np.array([float(R(w * 1e8)) for w in out_cm])
    return np.array([float(R)])


def _ranges(g: Wavelengths):
    arr = (_lib.WlRange * len(g.ranges))()
    for k, (start, step, n) in enumerate(g.ranges):
        arr[k] = _lib.WlRange(n, start, step)
    return arr


class _Ctx:
    def __init__(self, ctx):
        import torch
        self.torch = torch
        self.ctx = ctx or _lib.default_context()
        self.dev = torch.device("cuda", torch.cuda.current_device())

    def t(self, a):
        return self.torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(self.dev)

    @property
    def stream(self):
        return self.torch.cuda.current_stream(self.dev).cuda_stream


def _as_stack(flux):
    f = np.asarray(flux, dtype=np.float64)
    return (f[None, :], True) if f.ndim == 1 else (f, False)


def apply_LSF(flux, wls, R, window_size=4, obs_wls=None, ctx=None):
    """apply_LSF(flux, wls, R; window_size=4) (src/utils.jl:94-106); with ``obs_wls`` the
    product compute_LSF_matrix(wls, obs_wls, R) * flux (:132-155) without forming the matrix."""
    if R == math.inf and obs_wls is None:
        return np.array(flux, dtype=np.float64, copy=True)
    c = _Ctx(ctx)
    g = _grid(wls)
    out_cm = g.all_wls if obs_wls is None else _obs_cm(obs_wls)
    f, one = _as_stack(flux)
    Rv = _R_values(R, out_cm)
    tw, to, tR, tf = c.t(g.all_wls), c.t(out_cm), c.t(Rv), c.t(f)
    out = c.torch.empty((f.shape[0], len(out_cm)), dtype=c.torch.float64, device=c.dev)
    c.ctx.check(c.ctx.lib.korg_apply_lsf_dev(c.ctx.h, tw.data_ptr(), len(g), to.data_ptr(), len(out_cm),
                                             tR.data_ptr(), len(Rv), float(window_size), tf.data_ptr(), f.shape[0],
                                             out.data_ptr(), c.stream))
    o = out.cpu().numpy()
    return o[0] if one else o


def compute_LSF_matrix(synth_wls, obs_wls, R, window_size=4, ctx=None):
    """compute_LSF_matrix(synth_wls, obs_wls, R; window_size=4) (src/utils.jl:132-155) as a
    scipy.sparse CSR matrix of shape (len(obs_wls), len(synth_wls))."""
    import scipy.sparse
    c = _Ctx(ctx)
    g = _grid(synth_wls)
    out_cm = _obs_cm(obs_wls)
    Rv = _R_values(R, out_cm)
    tw, to, tR = c.t(g.all_wls), c.t(out_cm), c.t(Rv)
    n = len(out_cm)
    lb = c.torch.empty(n, dtype=c.torch.int64, device=c.dev)
    ub = c.torch.empty_like(lb)
    args = (c.ctx.h, tw.data_ptr(), len(g), to.data_ptr(), n, tR.data_ptr(), len(Rv), float(window_size))
    c.ctx.check(c.ctx.lib.korg_lsf_windows_dev(*args, lb.data_ptr(), ub.data_ptr(), c.stream))
    nnz = (ub - lb + 1).clamp(min=0)
    row_ptr = c.torch.zeros(n + 1, dtype=c.torch.int64, device=c.dev)
    row_ptr[1:] = c.torch.cumsum(nnz, 0)
    total = int(row_ptr[-1].item())
    vals = c.torch.empty(max(total, 1), dtype=c.torch.float64, device=c.dev)
    c.ctx.check(c.ctx.lib.korg_lsf_matrix_values_dev(*args, row_ptr.data_ptr(), vals.data_ptr(), c.stream))
    rp, lbh, nz = row_ptr.cpu().numpy(), lb.cpu().numpy(), nnz.cpu().numpy()
    cols = np.repeat(lbh, nz) + (np.arange(total) - np.repeat(rp[:-1], nz))
    return scipy.sparse.csr_matrix((vals[:total].cpu().numpy(), cols, rp), shape=(n, len(g)))


def apply_rotation(flux, wls, vsini, eps=0.6, ctx=None):
    """apply_rotation(flux, wls, vsini, ε=0.6) (src/utils.jl:168-192)."""
    c = _Ctx(ctx)
    g = _grid(wls)
    f, one = _as_stack(flux)
    rg = _ranges(g)
    tw, tf = c.t(g.all_wls), c.t(f)
    out = c.torch.empty_like(tf)
    c.ctx.check(c.ctx.lib.korg_apply_rotation_dev(c.ctx.h, tw.data_ptr(), len(g), rg, len(g.ranges), float(vsini),
                                                  float(eps), tf.data_ptr(), f.shape[0], out.data_ptr(), c.stream))
    o = out.cpu().numpy()
    return o[0] if one else o


def _autograd():
    import torch

    class LSF(torch.autograd.Function):
        """flux (nspec, nwl) device tensor -> LSF-convolved (nspec, nout); reverse mode L^T."""

        @staticmethod
        def forward(fctx, flux, wls, out_wls, R, window_size=4.0, ctx=None):
            c = _Ctx(ctx)
            f = flux.contiguous()
            out = torch.empty((f.shape[0], out_wls.numel()), dtype=torch.float64, device=f.device)
            args = (c.ctx.h, wls.data_ptr(), wls.numel(), out_wls.data_ptr(), out_wls.numel(), R.data_ptr(),
                    R.numel(), float(window_size))
            c.ctx.check(c.ctx.lib.korg_apply_lsf_dev(*args, f.data_ptr(), f.shape[0], out.data_ptr(), c.stream))
            fctx.args, fctx.c, fctx.nwl = args, c, f.shape[1]
            fctx.keep = (wls, out_wls, R)
            return out

        @staticmethod
        def backward(fctx, g):
            g = g.contiguous()
            d = torch.zeros((g.shape[0], fctx.nwl), dtype=torch.float64, device=g.device)
            fctx.c.ctx.check(fctx.c.ctx.lib.korg_apply_lsf_vjp_dev(*fctx.args, g.data_ptr(), g.shape[0], d.data_ptr(),
                                                                   fctx.c.stream))
            return d, None, None, None, None, None

    class Rotation(torch.autograd.Function):
        """flux (nspec, nwl) device tensor -> rotationally broadened; reverse mode R^T."""

        @staticmethod
        def forward(fctx, flux, wls, grid: Wavelengths, vsini, eps=0.6, ctx=None):
            c = _Ctx(ctx)
            f = flux.contiguous()
            rg = _ranges(grid)
            out = torch.empty_like(f)
            args = (c.ctx.h, wls.data_ptr(), wls.numel(), rg, len(grid.ranges), float(vsini), float(eps))
            c.ctx.check(c.ctx.lib.korg_apply_rotation_dev(*args, f.data_ptr(), f.shape[0], out.data_ptr(), c.stream))
            fctx.args, fctx.c, fctx.keep = args, c, (wls, rg)
            return out

        @staticmethod
        def backward(fctx, g):
            g = g.contiguous()
            d = torch.zeros_like(g)
            fctx.c.ctx.check(fctx.c.ctx.lib.korg_apply_rotation_vjp_dev(*fctx.args, g.data_ptr(), g.shape[0],
                                                                        d.data_ptr(), fctx.c.stream))
            return d, None, None, None, None, None

    return LSF, Rotation


def __getattr__(name):
    if name in ("LSF", "Rotation"):
        LSF, Rotation = _autograd()
        globals().update(LSF=LSF, Rotation=Rotation)
        return globals()[name]
    raise AttributeError(name)
