"""Bundled data tables (converted from Korg.jl's data directory by data/make_data.py)."""
from __future__ import annotations

import functools
import os

import numpy as np

from .cubic_spline import CubicSpline
from .species import parse_species

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


@functools.lru_cache(maxsize=None)
def _npz(name):
    with np.load(os.path.join(DATA_DIR, name), allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


@functools.lru_cache(maxsize=None)
def default_partition_funcs():
    """Species -> CubicSpline over ln T, as Korg's default_partition_funcs
    (src/read_statmech_quantities.jl:137-198): atomic tables on a uniform ln T grid without
    extrapolation, Barklem & Collet diatomics with flat extrapolation."""
    d = _npz("partition_funcs.npz")
    n = int(np.floor((d["logT_max"] - d["logT_min"]) / d["logT_step"] + 1 + 1e-9))
    logTs = d["logT_min"] + np.arange(n) * d["logT_step"]
    out = {}
    for name, U in zip(d["atomic_names"], d["U_atomic"]):
        out[parse_species(str(name))] = CubicSpline(logTs, U)
    ones = np.ones(n)
    out[parse_species("H II")] = CubicSpline(logTs, ones)
    out[parse_species("He III")] = CubicSpline(logTs, ones)
    lnT = np.log(d["mol_temps"])
    for name, U in zip(d["mol_names"], d["U_mol"]):
        try:
            spec = parse_species(str(name))
        except (KeyError, ValueError):
            continue
        out[spec] = CubicSpline(lnT, U, extrapolate=True)
    e = _npz("equilibrium_constants.npz")  # ExoMol polyatomics, astrophysical convention (:203-226)
    for k, name in enumerate(e["poly_names"]):
        a, b = e["poly_off"][k], e["poly_off"][k + 1]
        with np.errstate(divide="ignore", invalid="ignore"):  # H3+'s table starts at T = 0 (a NaN spline)
            out[parse_species(str(name))] = CubicSpline(np.log(e["poly_T"][a:b]), e["poly_U"][a:b] / e["poly_g_ns"][k],
                                                        extrapolate=True)
    return out


class PolyatomicLogK:
    """log10 of the partial-pressure equilibrium constant of a polyatomic molecule from its
    atomization energy D00 (kJ/mol) and partition functions (src/read_statmech_quantities.jl:66-89)."""

    def __init__(self, spec, D00_kJmol, partition_funcs):
        from .constants import hplanck_cgs, kboltz_cgs
        from .species import Species, atomic_masses
        self.spec, self.D00 = spec, D00_kJmol * 0.01036  # kJ/mol -> eV
        self.Zs = spec.atoms
        self.U_atoms = [partition_funcs[Species([Z], 0)] for Z in self.Zs]
        self.U_mol = partition_funcs[spec]
        self.log_masses_ratio = sum(np.log10(atomic_masses[Z - 1]) for Z in self.Zs) - np.log10(spec.mass())
        self._h, self._k = hplanck_cgs, kboltz_cgs

    def log_nK(self, logT):
        """log10 of the number-density equilibrium constant n(A)n(B).../n(mol)."""
        from .constants import kboltz_eV
        n = len(self.Zs)
        prod = 1.0
        for U in self.U_atoms:
            prod = prod * U(logT)
        log_Us_ratio = np.log10(prod / self.U_mol(logT))
        T = np.exp(logT)
        log_tU = 1.5 * np.log10(2 * np.pi * self._k * T / self._h ** 2)
        return ((n - 1) * log_tU + 1.5 * self.log_masses_ratio + log_Us_ratio
                - self.D00 / (kboltz_eV * T * np.log(10)))

    def __call__(self, logT):
        return self.log_nK(logT) + (len(self.Zs) - 1) * np.log10(self._k * np.exp(logT))


C2_CORRECTION_EV = 6.24 - 6.371  # Visser+ 2019 minus Barklem & Collet D0 of C2 (eV)


@functools.lru_cache(maxsize=None)
def barklem_collet_log_K_tables():
    """[(Species, ln T knots, log10 K)] of the Barklem & Collet molecules with the C2 dissociation
    energy corrected to Visser+ 2019 (src/read_statmech_quantities.jl:101-130): the non-finite
    knots of each molecule are dropped."""
    from .constants import kboltz_eV
    e = _npz("equilibrium_constants.npz")
    out = []
    for name, lnT, logK in zip(e["bc_mols"], e["bc_lnTs"], e["bc_logKs"]):
        spec = parse_species(str(name))
        logK = logK.copy()
        if spec == parse_species("C2"):
            logK += np.log10(np.e) / (kboltz_eV * np.exp(lnT)) * C2_CORRECTION_EV
        mask = np.isfinite(lnT)
        out.append((spec, lnT[mask], logK[mask]))
    return out


@functools.lru_cache(maxsize=None)
def default_log_equilibrium_constants():
    """Species -> log10 K(ln T) in partial-pressure form, as Korg's
    default_log_equilibrium_constants (src/read_statmech_quantities.jl:53-98): flat-extrapolated
    cubic splines for the Barklem & Collet diatomics, PolyatomicLogK for the polyatomics."""
    out = {spec: CubicSpline(lnT, logK, extrapolate=True) for spec, lnT, logK in barklem_collet_log_K_tables()}
    e = _npz("equilibrium_constants.npz")
    pf = default_partition_funcs()
    for name, D00 in zip(e["atomization_names"], e["atomization_kJmol"]):
        spec = parse_species(str(name))
        out[spec] = PolyatomicLogK(spec, float(D00), pf)
    return out


@functools.lru_cache(maxsize=None)
def ionization_energies():
    """Z -> [chi1, chi2, chi3] in eV (Barklem & Collet 2016)."""
    d = _npz("partition_funcs.npz")
    return {int(z): [float(x) for x in e] for z, e in zip(d["ion_Z"], d["ion_E"])}


@functools.lru_cache(maxsize=None)
def stark_profiles():
    """Stehle & Hutcheon tables packed as flat arrays with per-transition offsets; the profile
    is stored as log P with -Inf replaced by -700 and the first delta-nu knot as -floatmax
    (src/hydrogen_line_absorption.jl:6-37)."""
    d = _npz("stark_profiles.npz")
    nT, nNe, nD = d["nT"].astype(np.int32), d["nNe"].astype(np.int32), d["nD"].astype(np.int32)
    t_off = np.concatenate([[0], np.cumsum(nT)[:-1]]).astype(np.int64)
    ne_off = np.concatenate([[0], np.cumsum(nNe)[:-1]]).astype(np.int64)
    d_off = np.concatenate([[0], np.cumsum(nD)[:-1]]).astype(np.int64)
    p_sz = nT.astype(np.int64) * nNe * nD
    p_off = np.concatenate([[0], np.cumsum(p_sz)[:-1]]).astype(np.int64)
    l_sz = nT.astype(np.int64) * nNe
    l_off = np.concatenate([[0], np.cumsum(l_sz)[:-1]]).astype(np.int64)
    with np.errstate(divide="ignore"):
        logP = np.log(d["profile"])
    logP[logP == -np.inf] = -700.0
    logdnu = np.empty_like(d["dnu"])
    for t in range(len(nD)):
        seg = d["dnu"][d_off[t]:d_off[t] + nD[t]]
        logdnu[d_off[t]] = -np.finfo(np.float64).max
        logdnu[d_off[t] + 1:d_off[t] + nD[t]] = np.log(seg[1:])
    return dict(ntrans=len(nT), lower=d["lower"].astype(np.int32), upper=d["upper"].astype(np.int32),
                nT=nT, nNe=nNe, nD=nD, t_off=t_off, ne_off=ne_off, d_off=d_off, p_off=p_off,
                l_off=l_off, log_gf=d["log_gf"].astype(np.float64), temps=d["temps"], nes=d["nes"],
                logdnu=logdnu, logP=logP, lambda0=d["lambda0"] * 1e-8, names=d["names"])


@functools.lru_cache(maxsize=None)
def continuum_tables():
    """The continuum-absorption tables of src/ContinuumAbsorption/ (see make_data.continuum):
    arrays keyed as in continuum_tables.npz, all float64."""
    return {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in _npz("continuum_tables.npz").items()}
