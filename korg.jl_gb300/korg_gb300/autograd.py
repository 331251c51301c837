"""torch.autograd entry of the synthesis hot path (the juliacall-Python route to gradients).

:class:`Synthesis` holds one prepared spectrum's fixed inputs on the GPU; calling it with
torch tensors of the differentiable inputs returns (flux, cntm) tensors whose backward runs
korg_synthesize_vjp_dev (the hand-written reverse-mode kernels).  The differentiable inputs
are the hot-path inputs of korg_synthesize: per-layer T, n_e, n_eff_vdW, xi, the n/U rows,
per-line log gf, the continuum interpolant knots and the reference-wavelength continuum
opacity (all float64, on the device).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .api import SynthesisInputs, _prec

FIELDS = ("T", "ne", "n_eff_vdW", "xi", "n_div_U", "log_gf", "cntm_vals", "alpha_ref_cntm")


def _ptr(t, kind=_lib._dp):
    return C.cast(t.data_ptr(), kind)


class Synthesis:
    def __init__(self, inp: SynthesisInputs, precision="mixed", device=0, ctx=None, hydrogen_gradient=True):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.inp = inp
        self.prec = _prec(precision)
        self.ctx = ctx or _lib.Context(device)
        if inp.hydrogen_lines:
            self.ctx.ensure_stark()
        self.flags = _lib.KORG_VJP_HYDROGEN if hydrogen_gradient else 0
        t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(self.dev)
        self.wls = t(inp.wls.all_wls)
        self.fixed = {k: t(getattr(inp, k)) for k in ("tau_ref", "nH_I", "nHe_I", "UH_I", "cntm_knots")}
        ll, l5 = inp.linelist, inp.linelist5
        self.l1 = {k: t(getattr(ll, k)) for k in ("wl", "E_lower", "gamma_rad", "gamma_stark", "vdW1", "vdW2", "mass")}
        self.l1["is_mol"] = t(ll.is_mol, torch.int32)
        self.l1["species"] = t(ll.species_idx, torch.int32)
        self.l5 = {k: t(getattr(l5, k)) for k in ("wl", "log_gf", "E_lower", "gamma_rad", "gamma_stark", "vdW1",
                                                   "vdW2", "mass")}
        self.l5["is_mol"] = t(l5.is_mol, torch.int32)
        self.l5["species"] = t(l5.species_idx, torch.int32)
        self.L, self.nwl = len(inp.T), len(inp.wls)

    def initial(self):
        """The prepared values of the differentiable inputs, as device tensors."""
        torch = self.torch
        return {k: torch.as_tensor(np.ascontiguousarray(self.inp.linelist.log_gf if k == "log_gf" else
                                                        getattr(self.inp, k))).to(self.dev) for k in FIELDS}

    def _structs(self, x):
        inp = self.inp
        lay = _lib.Layers(self.L, x["n_div_U"].shape[0], _ptr(x["T"]), _ptr(x["ne"]), _ptr(x["n_eff_vdW"]),
                          _ptr(x["xi"]), _ptr(x["n_div_U"]))
        f = self.fixed
        s = _lib.SynthInputs(lay, _ptr(f["tau_ref"]), _ptr(x["alpha_ref_cntm"]), _ptr(f["nH_I"]), _ptr(f["nHe_I"]),
                             _ptr(f["UH_I"]), inp.ref_wl, _lib.Cntm(len(inp.cntm_knots), _ptr(f["cntm_knots"]),
                                                                     _ptr(x["cntm_vals"])),
                             int(inp.hydrogen_lines), int(inp.use_MHD), inp.hydrogen_window, inp.cutoff_threshold)

        def lines(d, log_gf, n):
            return _lib.Lines(n, _ptr(d["wl"]), _ptr(log_gf), _ptr(d["E_lower"]), _ptr(d["gamma_rad"]),
                              _ptr(d["gamma_stark"]), _ptr(d["vdW1"]), _ptr(d["vdW2"]), _ptr(d["mass"]),
                              _ptr(d["is_mol"], _lib._ip), _ptr(d["species"], _lib._ip))

        return s, lines(self.l1, x["log_gf"], len(inp.linelist)), lines(self.l5, self.l5["log_gf"], len(inp.linelist5))

    def forward_raw(self, x):
        torch = self.torch
        x = {k: v.detach().contiguous() for k, v in x.items()}
        s, l1, l5 = self._structs(x)
        flux = torch.empty(self.nwl, dtype=torch.float64, device=self.dev)
        cntm = torch.empty_like(flux)
        st = torch.cuda.current_stream(self.dev).cuda_stream
        self.ctx.check(self.ctx.lib.korg_synthesize_dev(self.ctx.h, C.byref(s), C.byref(l1), C.byref(l5),
                                                        self.wls.data_ptr(), self.nwl, self.prec, flux.data_ptr(),
                                                        cntm.data_ptr(), None, st))
        return flux, cntm

    def vjp_raw(self, x, dflux, dcntm):
        torch = self.torch
        x = {k: v.detach().contiguous() for k, v in x.items()}
        s, l1, l5 = self._structs(x)
        out = {k: torch.zeros_like(x[k]) for k in FIELDS}
        g = _lib.SynthGrads(_ptr(out["T"]), _ptr(out["ne"]), _ptr(out["n_eff_vdW"]), _ptr(out["xi"]),
                            _ptr(out["n_div_U"]), None, None, None, _ptr(out["log_gf"]), _ptr(out["cntm_vals"]),
                            _ptr(out["alpha_ref_cntm"]))
        st = torch.cuda.current_stream(self.dev).cuda_stream
        df = None if dflux is None else dflux.detach().contiguous().to(torch.float64)
        dc = None if dcntm is None else dcntm.detach().contiguous().to(torch.float64)
        self.ctx.check(self.ctx.lib.korg_synthesize_vjp_dev(
            self.ctx.h, C.byref(s), C.byref(l1), C.byref(l5), self.wls.data_ptr(), self.nwl, self.prec,
            None if df is None else df.data_ptr(), None if dc is None else dc.data_ptr(), C.byref(g), self.flags, st))
        return out

    def __call__(self, **x):
        """flux, cntm = synth(T=..., ne=..., n_eff_vdW=..., xi=..., n_div_U=..., log_gf=...,
        cntm_vals=..., alpha_ref_cntm=...) with autograd."""
        fn = _make_function(self.torch)
        return fn.apply(self, *[x[k] for k in FIELDS])


_FN = None


def _make_function(torch):
    global _FN
    if _FN is None:
        class SynthesizeFunction(torch.autograd.Function):
            @staticmethod
            def forward(ctx, synth, *xs):
                x = dict(zip(FIELDS, xs))
                ctx.synth = synth
                ctx.save_for_backward(*xs)
                return synth.forward_raw(x)

            @staticmethod
            def backward(ctx, dflux, dcntm):
                x = dict(zip(FIELDS, ctx.saved_tensors))
                g = ctx.synth.vjp_raw(x, dflux, dcntm)
                return (None, *[g[k] if ctx.needs_input_grad[i + 1] else None for i, k in enumerate(FIELDS)])

        _FN = SynthesizeFunction
    return _FN
