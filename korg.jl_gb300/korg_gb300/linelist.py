"""Line lists as structure-of-arrays, with Korg's ``Line`` conversion rules.

Korg's ``Line`` (src/linelist.jl:5-100) stores wl in cm, log gf, species, E_lower (eV),
gamma_rad, gamma_stark and a vdW pair that is either ``(gamma_vdW, -1)`` or ABO ``(sigma,
alpha)``.  :class:`LineList` holds the same fields as contiguous float64 / int32 arrays (the
layout the CUDA entry points take), sorted by wavelength.
"""
from __future__ import annotations

import math

import numpy as np

from .constants import (RydbergH_eV, Rydberg_eV, bohr_radius_cgs, c_cgs, electron_charge_cgs,
                        electron_mass_cgs, hplanck_eV, kboltz_cgs)
from .data import _npz, ionization_energies
from .species import Species, parse_species


def approximate_radiative_gamma(wl, log_gf):
    """src/linelist.jl:124-129"""
    e, m, c = electron_charge_cgs, electron_mass_cgs, c_cgs
    return 8 * math.pi ** 2 * e ** 2 / (m * c * wl ** 2) * 10 ** log_gf


def approximate_gammas(wl, species: Species, E_lower):
    """(gamma_stark, log10 gamma_vdW) per Unsold / Cowley at 10,000 K (src/linelist.jl:149-183)."""
    Z = species.charge + 1
    if species.ismolecule() or Z > 3:
        return 0.0, 0.0
    chi = ionization_energies()[species.atoms[0]][Z - 1]
    c, h, k = c_cgs, hplanck_eV, kboltz_cgs
    E_upper = E_lower + (h * c / wl)
    nstar4_upper = (Z ** 2 * RydbergH_eV / (chi - E_upper)) ** 2
    if Z == 1:
        gstark = 2.25910152e-7 * nstar4_upper
    else:
        gstark = 5.42184365e-7 * nstar4_upper / (Z + 1) ** 2
    drbar2 = (5 / 2) * Rydberg_eV ** 2 * Z ** 2 * (1 / (chi - E_upper) ** 2 - 1 / (chi - E_lower) ** 2)
    if chi < E_upper:
        log_gvdW = 0.0
    else:
        log_gvdW = 6.33 + 0.4 * math.log10(drbar2) + 0.3 * math.log10(10_000) + math.log10(k)
    return gstark, log_gvdW


def make_line(wl, log_gf, species, E_lower, gamma_rad=None, gamma_stark=None, vdW=None):
    """One line's fields after Korg's Line constructor rules (src/linelist.jl:56-100).
    Returns (wl_cm, log_gf, species, E_lower, gamma_rad, gamma_stark, vdW1, vdW2)."""
    if isinstance(species, str):
        species = parse_species(species)
    if wl >= 1:
        wl *= 1e-8
    isnan = lambda x: x is None or (not isinstance(x, tuple) and math.isnan(x))
    if isnan(gamma_stark) or isnan(vdW):
        gs_approx, vdW_approx = approximate_gammas(wl, species, E_lower)
        if isnan(gamma_stark):
            gamma_stark = gs_approx
        if isnan(vdW):
            vdW = vdW_approx
    if isnan(gamma_rad):
        gamma_rad = approximate_radiative_gamma(wl, log_gf)
    if not isinstance(vdW, tuple):
        if vdW < 0:
            vdW = (10 ** vdW, -1.0)
        elif vdW == 0:
            vdW = (0.0, -1.0)
        elif 0 < vdW < 20:
            vdW = (vdW * 10 ** approximate_gammas(wl, species, E_lower)[1], -1.0)
        else:
            vdW = (math.floor(vdW) * bohr_radius_cgs * bohr_radius_cgs, vdW - math.floor(vdW))
    return (wl, log_gf, species, E_lower, gamma_rad, gamma_stark, float(vdW[0]), float(vdW[1]))


class LineList:
    """Structure-of-arrays line list.  ``species`` is a list of :class:`Species`; ``species_idx``
    maps each line to a row of ``species``."""

    fields = ("wl", "log_gf", "E_lower", "gamma_rad", "gamma_stark", "vdW1", "vdW2")

    def __init__(self, wl, log_gf, species_idx, species, E_lower, gamma_rad, gamma_stark, vdW1, vdW2):
        self.wl = np.ascontiguousarray(wl, dtype=np.float64)
        self.log_gf = np.ascontiguousarray(log_gf, dtype=np.float64)
        self.species_idx = np.ascontiguousarray(species_idx, dtype=np.int32)
        self.species = list(species)
        self.E_lower = np.ascontiguousarray(E_lower, dtype=np.float64)
        self.gamma_rad = np.ascontiguousarray(gamma_rad, dtype=np.float64)
        self.gamma_stark = np.ascontiguousarray(gamma_stark, dtype=np.float64)
        self.vdW1 = np.ascontiguousarray(vdW1, dtype=np.float64)
        self.vdW2 = np.ascontiguousarray(vdW2, dtype=np.float64)
        self.mass = np.array([s.mass() for s in self.species], dtype=np.float64)[self.species_idx] \
            if len(self.species) else np.zeros(len(self.wl))
        self.is_mol = np.array([s.ismolecule() for s in self.species], dtype=np.int32)[self.species_idx] \
            if len(self.species) else np.zeros(len(self.wl), np.int32)

    @classmethod
    def from_lines(cls, lines):
        """From tuples produced by :func:`make_line`."""
        specs, idx = [], {}
        cols = [[] for _ in range(8)]
        for ln in lines:
            for k, v in enumerate(ln):
                cols[k].append(v)
        sidx = []
        for s in cols[2]:
            if s not in idx:
                idx[s] = len(specs)
                specs.append(s)
            sidx.append(idx[s])
        return cls(cols[0], cols[1], sidx, specs, cols[3], cols[4], cols[5], cols[6], cols[7])

    def __len__(self):
        return len(self.wl)

    def subset(self, sel):
        return LineList(self.wl[sel], self.log_gf[sel], self.species_idx[sel], self.species,
                        self.E_lower[sel], self.gamma_rad[sel], self.gamma_stark[sel],
                        self.vdW1[sel], self.vdW2[sel])

    def is_sorted(self):
        return bool(np.all(np.diff(self.wl) >= 0))

    def sorted(self):
        return self.subset(np.argsort(self.wl, kind="stable"))

    def concat(self, other):
        specs = list(self.species)
        remap = []
        for s in other.species:
            if s not in specs:
                specs.append(s)
            remap.append(specs.index(s))
        remap = np.asarray(remap, dtype=np.int32)
        return LineList(np.concatenate([self.wl, other.wl]), np.concatenate([self.log_gf, other.log_gf]),
                        np.concatenate([self.species_idx, remap[other.species_idx]]), specs,
                        np.concatenate([self.E_lower, other.E_lower]),
                        np.concatenate([self.gamma_rad, other.gamma_rad]),
                        np.concatenate([self.gamma_stark, other.gamma_stark]),
                        np.concatenate([self.vdW1, other.vdW1]), np.concatenate([self.vdW2, other.vdW2]))


def filter_linelist(linelist: LineList, wls, line_buffer):
    """Lines within ``line_buffer`` (cm) of each wavelength window (src/synthesize.jl:331-350)."""
    last = -1
    keep = []
    for lo, hi in wls.eachwindow():
        first = int(np.searchsorted(linelist.wl, lo - line_buffer, side="left"))
        first = max(first, last + 1)
        last = int(np.searchsorted(linelist.wl, hi + line_buffer, side="right")) - 1
        keep.append(np.arange(first, last + 1))
    sel = np.concatenate(keep) if keep else np.zeros(0, np.int64)
    return linelist.subset(sel)


def alpha_5000_linelist() -> LineList:
    """Korg's built-in reference-wavelength line list (src/linelist.jl:970-993)."""
    d = _npz("alpha_5000_lines.npz")
    lines = []
    for i in range(len(d["wl"])):
        v1, v2 = d["vdW"][i]
        vdW = float(v1) if np.isnan(v2) else (float(v1), float(v2))
        lines.append(make_line(float(d["wl"][i]), float(d["log_gf"][i]), str(d["species"][i]),
                               float(d["E_lower"][i]), float(d["gamma_rad"][i]),
                               float(d["gamma_stark"][i]), vdW))
    return LineList.from_lines(lines)
