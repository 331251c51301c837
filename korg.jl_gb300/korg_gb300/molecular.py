"""Precomputed molecular cross-sections on the GPU.

``MolecularCrossSection`` restates src/molecular_cross_sections.jl:51-88: the absorption
cross-section per molecule of one species' lines on a (vmic, T, wavelength) grid, computed with
the line-opacity kernels (the temperatures play the role of layers, with n_e = 0, continuum 1,
cutoff threshold 1 and n/U = 1/(cutoff_alpha U(T)), so each line is truncated where its
absorption coefficient per molecule falls to cutoff_alpha).  ``interpolate_into`` restates
interpolate_molecular_cross_sections! (:101-117): trilinear interpolation in (vmic, log10 T,
wavelength), zero outside the table, times the molecule's number density, added to alpha.
The table stays on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .data import default_partition_funcs
from .wavelengths import Wavelengths

DEFAULT_VMIC = np.array([0.0, 1 / 3, 2 / 3, 1.0, 1.5, 2.0, 2 + 2 / 3, 2 + 4 / 3, 4.0, 4 + 2 / 3, 4 + 4 / 3])
DEFAULT_LOGT = np.arange(3.0, 5.0 + 1e-9, 0.04)


class MolecularCrossSection:
    def __init__(self, linelist, wavelengths, cutoff_alpha=1e-32, vmic_vals=DEFAULT_VMIC, log_temp_vals=DEFAULT_LOGT,
                 precision="fp64", ctx=None, device=0):
        import torch
        species = {linelist.species[k] for k in np.unique(linelist.species_idx)}
        if len(species) != 1:
            raise ValueError("All lines must be of the same species")
        self.species = species.pop()
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.ctx = ctx or _lib.default_context()
        self.wls = wavelengths if isinstance(wavelengths, Wavelengths) else Wavelengths(wavelengths)
        self.vmic_vals = np.asarray(vmic_vals, np.float64)
        self.log_temp_vals = np.asarray(log_temp_vals, np.float64)
        T = 10.0 ** self.log_temp_vals
        U = default_partition_funcs()[self.species](np.log(T))
        t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(self.dev)
        self._T, self._invU = t(T), t(1.0 / U)
        self._twls = t(self.wls.all_wls)
        self._vm, self._lt = t(self.vmic_vals), t(self.log_temp_vals)
        ll = linelist
        keep = [t(getattr(ll, k)) for k in ("wl", "log_gf", "E_lower", "gamma_rad", "gamma_stark", "vdW1", "vdW2",
                                            "mass")]
        keep += [t(ll.is_mol, torch.int32), t(np.zeros(len(ll)), torch.int32)]  # species row 0
        lines = _lib.Lines(len(ll), *[C.cast(x.data_ptr(), _lib._dp) for x in keep[:8]],
                           C.cast(keep[8].data_ptr(), _lib._ip), C.cast(keep[9].data_ptr(), _lib._ip))
        nT, nv, nw = len(T), len(self.vmic_vals), len(self.wls)
        self.table = torch.empty((nv, nw, nT), dtype=torch.float64, device=self.dev)
        prec = _lib.KORG_MIXED if precision == "mixed" else _lib.KORG_FP64
        st = torch.cuda.current_stream(self.dev).cuda_stream
        self.ctx.check(self.ctx.lib.korg_molecular_cross_section_dev(
            self.ctx.h, C.byref(lines), self._twls.data_ptr(), nw, self._T.data_ptr(), self._invU.data_ptr(), nT,
            self._vm.data_ptr(), nv, float(cutoff_alpha), prec, self.table.data_ptr(), st))
        torch.cuda.synchronize(self.dev)

    def table_numpy(self):
        """(vmic, wavelength, T) array of the cross-section per molecule (cm^2)."""
        return self.table.cpu().numpy()

    def interpolate_into(self, alpha, wls, T, vmic, n):
        """alpha (device tensor, (nwl, L) C order = Korg's L x nwl) += sigma(vmic, T, wl) * n; the
        other arguments are device tensors of wavelengths (cm), per-layer T, vmic (km/s) and the
        molecule's number density."""
        L = alpha.shape[1]
        st = self.torch.cuda.current_stream(self.dev).cuda_stream
        nT, nv, nw = len(self.log_temp_vals), len(self.vmic_vals), len(self.wls)
        self.ctx.check(self.ctx.lib.korg_interpolate_molecular_cross_section_dev(
            self.ctx.h, alpha.data_ptr(), wls.data_ptr(), alpha.shape[0], L, T.data_ptr(), vmic.data_ptr(),
            n.data_ptr(), self.table.data_ptr(), self._twls.data_ptr(), nw, self._vm.data_ptr(), nv,
            self._lt.data_ptr(), nT, st))
