"""Fitting through the GPU path: synthesis, rectification, rotation and LSF, differentiated end
to end.

Korg's Fit module (src/Fit/fit_via_synthesis.jl:304-390) minimises the squared residual between
an observed spectrum and synthesize -> rectify -> apply_rotation -> LSF matrix, with gradients
from ForwardDiff.  :func:`fit_log_gf` does the same for the line strengths of chosen lines
(the hot-path parameter a line-list calibration fits): every stage is a GPU kernel with a
hand-written reverse mode (korg_synthesize_vjp_dev, korg_apply_rotation_vjp_dev,
korg_apply_lsf_vjp_dev), chained by torch autograd, and scipy's L-BFGS-B drives the loop.
"""
from __future__ import annotations

import numpy as np

from .api import SynthesisInputs


def _obs_cm(obs):
    o = np.asarray(obs, dtype=np.float64)
    return o * 1e-8 if o.size and o[0] >= 1 else o


class SpectrumModel:
    """Rectified model spectrum of prepared inputs as a differentiable function of the log gf of
    the lines ``line_idx``: flux / continuum, then rotation (vsini > 0) and a Gaussian LSF of
    resolving power R onto ``obs_wls`` (the synthesis grid when None; no LSF when R is None)."""

    def __init__(self, inp: SynthesisInputs, line_idx, obs_wls=None, R=None, vsini=0.0, eps=0.6,
                 precision="mixed", ctx=None):
        import torch
        from .autograd import Synthesis
        self.torch = torch
        self.inp = inp
        self.synth = Synthesis(inp, precision=precision, ctx=ctx)
        self.dev = self.synth.dev
        self.x = self.synth.initial()
        self.idx = torch.as_tensor(np.asarray(line_idx, dtype=np.int64), device=self.dev)
        self.vsini, self.eps, self.R = float(vsini), float(eps), R
        if R is not None:
            out_cm = inp.wls.all_wls if obs_wls is None else _obs_cm(obs_wls)
            Rv = np.array([float(R(w * 1e8)) for w in out_cm]) if callable(R) else np.array([float(R)])
            self.out_wls = torch.as_tensor(np.ascontiguousarray(out_cm), device=self.dev)
            self.Rv = torch.as_tensor(Rv, device=self.dev)

    def initial(self):
        """The prepared log gf of the fitted lines."""
        return self.x["log_gf"][self.idx].cpu().numpy()

    def __call__(self, log_gf):
        """Model spectrum (device tensor) for a device tensor of the fitted lines' log gf."""
        from .postprocess import LSF, Rotation
        x = dict(self.x)
        x["log_gf"] = self.x["log_gf"].index_put((self.idx,), log_gf)
        flux, cntm = self.synth(**x)
        y = (flux / cntm)[None]
        if self.vsini > 0:
            y = Rotation.apply(y, self.synth.wls, self.inp.wls, self.vsini, self.eps, self.synth.ctx)
        if self.R is not None:
            y = LSF.apply(y, self.synth.wls, self.out_wls, self.Rv, 4.0, self.synth.ctx)
        return y[0]


def fit_log_gf(inp: SynthesisInputs, obs, line_idx, obs_wls=None, R=None, vsini=0.0, eps=0.6, precision="mixed",
               maxiter=100, ctx=None):
    """Least-squares fit of the log gf of lines ``line_idx`` to the rectified observed spectrum
    ``obs`` (on ``obs_wls``, or on the synthesis grid), through :class:`SpectrumModel`.
    Returns (fitted log gf, final loss, scipy OptimizeResult)."""
    import scipy.optimize
    model = SpectrumModel(inp, line_idx, obs_wls=obs_wls, R=R, vsini=vsini, eps=eps, precision=precision, ctx=ctx)
    torch = model.torch
    tobs = torch.as_tensor(np.ascontiguousarray(obs, dtype=np.float64), device=model.dev)

    def loss_and_grad(v):
        lg = torch.as_tensor(v, dtype=torch.float64, device=model.dev).requires_grad_(True)
        loss = torch.sum((model(lg) - tobs) ** 2)
        loss.backward()
        return float(loss.item()), lg.grad.detach().cpu().numpy()

    res = scipy.optimize.minimize(loss_and_grad, model.initial(), jac=True, method="L-BFGS-B",
                                  options={"maxiter": int(maxiter), "ftol": 1e-15, "gtol": 1e-12})
    return res.x, float(res.fun), res
