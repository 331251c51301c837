"""Continuum absorption on the GPU (korg_continuum_absorption), with the reference's interface.

* :func:`total_continuum_absorption` -- ``total_continuum_absorption(nus, T, ne,
  number_densities, partition_funcs)`` (src/ContinuumAbsorption/ContinuumAbsorption.jl:39-74) for
  one layer;
* :func:`continuum_absorption` -- every layer of an atmosphere on a wavelength grid at once, the
  form synthesize uses (src/synthesize.jl:211-237), returning the (L, nwl) values of the
  continuum interpolants.

Number densities come from the caller's chemical equilibrium as a dict Species -> density (a
scalar for one layer, or an array over layers).  n(H-) is taken from the dict when present, else
from n(H I) n_e nK(T) as the reference's chemical equilibrium forms it (src/statmech.jl:75-79,
182).  Metal bound-free absorption is not included (its tables are not distributed with the
reference).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .species import Species, parse_species

_PEACH = ("He II", "C II", "Si II", "Mg II")  # ions with Peach (1970) departure coefficients

kboltz_cgs, hplanck_cgs, electron_mass_cgs, kboltz_eV = 1.380649e-16, 6.62607015e-27, 9.1093897e-28, 8.617333262145e-5


def Hminus_nK(T):
    """n(H-) = nK(T) n(H I) n_e (src/statmech.jl:75-79)."""
    T = np.asarray(T, np.float64)
    transU = (2 * np.pi * electron_mass_cgs * kboltz_cgs * T / hplanck_cgs ** 2) ** 1.5
    return np.exp(0.754204 / (kboltz_eV * T)) / (4 * transU)


def layer_inputs(T, ne, number_densities, partition_funcs=None):
    """The per-layer quantities of korg_continuum_layers from a number-density dict."""
    from .data import default_partition_funcs
    pf = partition_funcs or default_partition_funcs()
    T = np.atleast_1d(np.asarray(T, np.float64))
    L = len(T)
    ne = np.broadcast_to(np.asarray(ne, np.float64), (L,)).astype(np.float64)
    z = np.zeros(L)
    g = lambda s: np.broadcast_to(np.asarray(number_densities.get(parse_species(s), z), np.float64), (L,))
    Hminus = Species([1], -1)
    d = {"T": T, "ne": ne, "nH_I": g("H I"), "nH_II": g("H II"), "nHe_I": g("He I"), "nH2": g("H2")}
    d["nH_minus"] = (np.broadcast_to(np.asarray(number_densities[Hminus], np.float64), (L,))
                     if Hminus in number_densities else Hminus_nK(T) * d["nH_I"] * ne)
    lnT = np.log(T)
    d["invU_H_I"] = 1.0 / pf[parse_species("H I")](lnT)
    d["invU_He_I"] = 1.0 / pf[parse_species("He I")](lnT)
    peach = {parse_species(s): s for s in _PEACH}
    d["n_Z1"], d["n_Z2"] = np.zeros(L), np.zeros(L)
    for s in _PEACH:
        d["n_" + s.replace(" ", "")] = g(s)
    for spec, n in number_densities.items():
        if spec.charge <= 0 or spec in peach:
            continue
        if spec.charge == 1:
            d["n_Z1"] = d["n_Z1"] + n
        elif spec.charge == 2:
            d["n_Z2"] = d["n_Z2"] + n
        else:
            raise ValueError("triply+ ionized species not supported")  # absorption_ff_positive_ion.jl:76-78
    return {k: np.ascontiguousarray(np.broadcast_to(v, (L,)), np.float64) for k, v in d.items()}


def _layers_struct(d, keep):
    f = lambda k: _lib._p(keep.f64(d[k]))
    return _lib.ContinuumLayers(len(d["T"]), *[f(k) for k in ("T", "ne", "nH_I", "nH_II", "nHe_I", "nH2", "nH_minus",
                                                               "invU_H_I", "invU_He_I", "n_Z1", "n_Z2")],
                                (_lib._dp * 4)(*[f("n_" + s.replace(" ", "")) for s in _PEACH]))


def absorption_from_inputs(wls_cm, d, ctx=None):
    """korg_continuum_absorption for the per-layer inputs of :func:`layer_inputs`: array (L, nwl)."""
    ctx = ctx or _lib.default_context()
    ctx.ensure_continuum()
    keep = _lib.Keep()
    w = keep.f64(np.atleast_1d(wls_cm))
    out = np.empty((len(d["T"]), len(w)))
    ctx.check(ctx.lib.korg_continuum_absorption(ctx.h, _lib._p(w), len(w), C.byref(_layers_struct(d, keep)),
                                                _lib._p(out)))
    return out


def continuum_absorption(wls_cm, T, ne, number_densities, partition_funcs=None, ctx=None):
    """Continuum absorption (cm^-1) of every layer at every wavelength (cm): array (L, nwl)."""
    return absorption_from_inputs(wls_cm, layer_inputs(T, ne, number_densities, partition_funcs), ctx)


INPUTS = ("T", "ne", "nH_I", "nH_II", "nHe_I", "nH2", "nH_minus", "invU_H_I", "invU_He_I", "n_Z1", "n_Z2",
          "n_HeII", "n_CII", "n_SiII", "n_MgII")


def absorption_vjp(wls_cm, d, gbar, ctx=None, rel=1e-6):
    """Reverse mode of :func:`absorption_from_inputs`: {input: dL/dinput [L]} for L = sum gbar *
    alpha, by central differences of the FP64 device kernel, every layer's input perturbed at once
    (the layers are independent).  The terms are linear in the densities (the step is exact there)
    and piecewise-smooth in T (table interpolation), so a relative step of 1e-6 leaves ~1e-10 of
    truncation and rounding; an input that is zero takes an absolute step of 1."""
    gbar = np.asarray(gbar, np.float64)
    out = {}
    for k in INPUTS:
        v = d[k]
        h = np.where(v != 0, rel * np.abs(v), 1.0)
        dp, dm = dict(d), dict(d)
        dp[k], dm[k] = v + h, v - h
        diff = absorption_from_inputs(wls_cm, dp, ctx) - absorption_from_inputs(wls_cm, dm, ctx)
        out[k] = np.sum(gbar * diff, axis=1) / (2 * h)
    return out


def layer_inputs_vjp(grads, T, number_densities, partition_funcs=None):
    """Chain the continuum inputs' gradients (:func:`absorption_vjp`) back to the layer
    temperatures, n_e and the number density of each species (the map of :func:`layer_inputs`):
    returns (dT [L], dne [L], {Species: dn [L]})."""
    from .data import default_partition_funcs
    pf = partition_funcs or default_partition_funcs()
    T = np.atleast_1d(np.asarray(T, np.float64))
    lnT = np.log(T)
    dn = {}
    add = lambda s, v: dn.__setitem__(s, dn.get(s, 0.0) + v)
    add(parse_species("H I"), grads["nH_I"])
    add(parse_species("H II"), grads["nH_II"])
    add(parse_species("He I"), grads["nHe_I"])
    add(parse_species("H2"), grads["nH2"])
    Hminus = Species([1], -1)
    if Hminus not in number_densities:  # Korg's chemical equilibrium always provides it
        raise NotImplementedError("the continuum reverse mode needs n(H-) among the number densities")
    add(Hminus, grads["nH_minus"])
    dT = grads["T"].copy()
    for k, s in (("invU_H_I", "H I"), ("invU_He_I", "He I")):
        U = pf[parse_species(s)](lnT)
        dT += grads[k] * (-pf[parse_species(s)].derivative(lnT) / T) / U ** 2
    peach = {parse_species(s): "n_" + s.replace(" ", "") for s in _PEACH}
    for spec in number_densities:
        if spec.charge <= 0:
            continue
        if spec in peach:
            add(spec, grads[peach[spec]])
        elif spec.charge == 1:
            add(spec, grads["n_Z1"])
        elif spec.charge == 2:
            add(spec, grads["n_Z2"])
    return dT, grads["ne"].copy(), dn


def total_continuum_absorption(nus, T, ne, number_densities, partition_funcs=None, ctx=None):
    """``total_continuum_absorption(nus, T, ne, number_densities, partition_funcs)`` for one layer:
    alpha (cm^-1) at the sorted frequencies ``nus`` (Hz)."""
    nus = np.asarray(nus, np.float64)
    if np.any(np.diff(nus) < 0):
        raise ValueError("nus should be sorted")
    wls = 2.99792458e10 / nus[::-1]
    return continuum_absorption(wls, T, ne, number_densities, partition_funcs, ctx)[0][::-1].copy()
