"""Batched synthesis through ``korg_synthesize_batch_dev``.

Korg's Fit module (src/Fit/fit_via_synthesis.jl:304-390) and grid builders call ``synthesize``
over and over for many atmospheres and abundance sets.  :class:`BatchSynthesis` keeps a batch
of prepared spectra resident on the GPU and runs them together: every spectrum's prologue, one
persistent tile launch over the (spectrum, wavelength-tile) queue, every spectrum's transfer.
With ``use_graph`` the second and later runs of the same batch replay a CUDA graph.

All device memory here is torch tensors (plumbing only); the work is the C library's.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .api import SynthesisInputs, _prec


class _Packer:
    """Lays out many host arrays in one byte buffer (256-byte aligned pieces), so a batch moves
    host -> device in one copy."""

    def __init__(self):
        self.items = []
        self.size = 0

    def add(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        off = (self.size + 255) & ~255
        self.items.append((off, a))
        self.size = off + max(a.nbytes, 1)
        return off


class BatchSynthesis:
    """A batch of prepared spectra on one wavelength grid, resident on ``device``.

    ``run()`` synthesises all of them (device flux and continuum, shape (n, nwl));
    ``upload()`` copies the host inputs again (after they were edited in place through
    ``host_array``) with one host-to-device copy; ``results()`` returns numpy copies."""

    def __init__(self, inputs: list[SynthesisInputs], precision="mixed", ctx=None, device=0, use_graph=True,
                 autotune=False, max_scratch_bytes=0):
        import torch
        if not inputs:
            raise ValueError("empty batch")
        wls = inputs[0].wls.all_wls
        for inp in inputs[1:]:
            if len(inp.wls) != len(wls) or not np.array_equal(inp.wls.all_wls, wls):
                raise ValueError("all spectra of a batch need the same wavelength grid")
            if len(inp.T) != len(inputs[0].T):
                raise ValueError("all spectra of a batch need the same number of layers")
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.ctx = ctx or _lib.Context(device)
        if any(inp.hydrogen_lines for inp in inputs):
            self.ctx.ensure_stark()
        self.ctx.check(self.ctx.lib.korg_set_batch_options(self.ctx.h, int(use_graph), int(autotune),
                                                           int(max_scratch_bytes)))
        self.inputs = inputs
        self.prec = _prec(precision)
        self.nwl, self.n = len(wls), len(inputs)
        pk = _Packer()
        self._wls_off = pk.add(wls, np.float64)
        self._layout = []
        for inp in inputs:
            self._layout.append(self._pack_one(pk, inp))
        self.host = torch.empty(pk.size, dtype=torch.uint8, pin_memory=True)
        hv = self.host.numpy()
        for off, a in pk.items:
            hv[off:off + a.nbytes] = a.view(np.uint8).reshape(-1)
        self.dbuf = torch.empty(pk.size, dtype=torch.uint8, device=self.dev)
        self.dbuf.copy_(self.host)
        self.flux = torch.empty((self.n, self.nwl), dtype=torch.float64, device=self.dev)
        self.cntm = torch.empty_like(self.flux)
        base = self.dbuf.data_ptr()
        self.items = (_lib.BatchItem * self.n)()
        for k, (inp, lay) in enumerate(zip(inputs, self._layout)):
            self.items[k] = self._item(inp, lay, base, k)
        self.wls_ptr = base + self._wls_off
        self.h2d_bytes = pk.size
        self._pk = pk

    @staticmethod
    def _pack_one(pk, inp):
        f, i = np.float64, np.int32
        o = {}
        for name in ("T", "ne", "n_eff_vdW", "xi", "n_div_U", "tau_ref", "alpha_ref_cntm", "nH_I", "nHe_I", "UH_I",
                     "cntm_knots", "cntm_vals"):
            o[name] = pk.add(getattr(inp, name), f)
        for tag, ll in (("l", inp.linelist), ("l5", inp.linelist5)):
            for name in ("wl", "log_gf", "E_lower", "gamma_rad", "gamma_stark", "vdW1", "vdW2", "mass"):
                o[f"{tag}.{name}"] = pk.add(getattr(ll, name), f)
            o[f"{tag}.is_mol"] = pk.add(ll.is_mol, i)
            o[f"{tag}.species"] = pk.add(ll.species_idx, i)
        return o

    def _item(self, inp, o, base, k):
        dp = lambda name: C.cast(base + o[name], _lib._dp)
        ip = lambda name: C.cast(base + o[name], _lib._ip)
        L = len(inp.T)
        lay = _lib.Layers(L, inp.n_div_U.shape[0], dp("T"), dp("ne"), dp("n_eff_vdW"), dp("xi"), dp("n_div_U"))
        s = _lib.SynthInputs(lay, dp("tau_ref"), dp("alpha_ref_cntm"), dp("nH_I"), dp("nHe_I"), dp("UH_I"),
                             inp.ref_wl, _lib.Cntm(len(inp.cntm_knots), dp("cntm_knots"), dp("cntm_vals")),
                             int(inp.hydrogen_lines), int(inp.use_MHD), inp.hydrogen_window, inp.cutoff_threshold)

        def lines(tag, ll):
            return _lib.Lines(len(ll), *[dp(f"{tag}.{n}") for n in ("wl", "log_gf", "E_lower", "gamma_rad",
                                                                   "gamma_stark", "vdW1", "vdW2", "mass")],
                              ip(f"{tag}.is_mol"), ip(f"{tag}.species"))

        fl = C.cast(self.flux.data_ptr() + 8 * self.nwl * k, _lib._dp)
        cn = C.cast(self.cntm.data_ptr() + 8 * self.nwl * k, _lib._dp)
        return _lib.BatchItem(s, lines("l", inp.linelist), lines("l5", inp.linelist5), fl, cn)

    def host_array(self, k, name):
        """Writable view of spectrum k's host copy of input ``name`` (e.g. "T", "n_div_U")."""
        off = self._layout[k][name]
        src = getattr(self.inputs[k], name)
        return self.host.numpy()[off:off + src.nbytes].view(np.float64).reshape(src.shape)

    def upload(self, stream=None):
        """One host-to-device copy of every spectrum's inputs (pinned, asynchronous)."""
        self.dbuf.copy_(self.host, non_blocking=True)

    def run(self, stream=None):
        stream = stream or self.torch.cuda.current_stream(self.dev)
        self.ctx.check(self.ctx.lib.korg_synthesize_batch_dev(self.ctx.h, self.n, self.items, self.wls_ptr, self.nwl,
                                                              self.prec, stream.cuda_stream))
        return self.flux, self.cntm

    def vjp(self, dflux, dcntm=None, hydrogen=True, reuse_forward=True, stream=None):
        """Reverse mode of the batch (korg_synthesize_batch_vjp_dev): for every spectrum k the
        gradient of sum(dflux[k] * flux[k] + dcntm[k] * cntm[k]) with respect to its hot-path
        inputs, as a list of dicts of device tensors keyed like api.GRAD_FIELDS (T, ne, n_eff_vdW,
        xi, nH_I, nHe_I, UH_I [L]; n_div_U [S, L]; log_gf [lines]; cntm_vals [L, nk];
        alpha_ref_cntm [L]).  dflux, dcntm: device tensors (n, nwl) or None.  reuse_forward: the
        last call was run() of this batch (in one chunk), whose opacity is reused."""
        from .api import GRAD_FIELDS
        torch = self.torch
        stream = stream or torch.cuda.current_stream(self.dev)
        L = len(self.inputs[0].T)
        out, cot = [], (_lib.BatchVjpItem * self.n)()
        keep = [dflux, dcntm]
        for k, inp in enumerate(self.inputs):
            shapes = {"n_div_U": inp.n_div_U.shape, "log_gf": (len(inp.linelist),), "cntm_vals": inp.cntm_vals.shape}
            g = {f: torch.zeros(shapes.get(f, (L,)), dtype=torch.float64, device=self.dev) for f in GRAD_FIELDS}
            out.append(g)
            ptr = lambda t: C.cast(t.data_ptr(), _lib._dp)
            cot[k] = _lib.BatchVjpItem(None if dflux is None else C.cast(dflux[k].data_ptr(), _lib._dp),
                                       None if dcntm is None else C.cast(dcntm[k].data_ptr(), _lib._dp),
                                       _lib.SynthGrads(*[ptr(g[f]) for f in GRAD_FIELDS]))
        flags = (_lib.KORG_VJP_HYDROGEN if hydrogen else 0) | (_lib.KORG_VJP_REUSE_FORWARD if reuse_forward else 0)
        self.ctx.check(self.ctx.lib.korg_synthesize_batch_vjp_dev(self.ctx.h, self.n, self.items, cot, self.wls_ptr,
                                                                  self.nwl, self.prec, flags, stream.cuda_stream))
        self._vjp_keep = (keep, cot)
        return out

    def results(self):
        self.torch.cuda.synchronize(self.dev)
        return self.flux.cpu().numpy(), self.cntm.cpu().numpy()

    def tile_config(self):
        tw, st, sp, tu = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        self.ctx.check(self.ctx.lib.korg_get_tile_config(self.ctx.h, len(self.inputs[0].T), self.prec, C.byref(tw),
                                                         C.byref(st), C.byref(sp), C.byref(tu)))
        return {"tw": tw.value, "stage": st.value, "split": bool(sp.value), "tuned": bool(tu.value)}
