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
