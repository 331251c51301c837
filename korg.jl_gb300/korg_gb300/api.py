"""Python mirror of Korg's hot-path API, backed by the CUDA library.

* :func:`line_absorption_`   -- ``line_absorption!`` (src/line_absorption.jl:33-129)
* :func:`hydrogen_line_absorption_` -- ``hydrogen_line_absorption!``
  (src/hydrogen_line_absorption.jl:75-163)
* :func:`radiative_transfer` -- ``RadiativeTransfer.radiative_transfer`` for a planar
  atmosphere with the default schemes (RadiativeTransfer.jl:62-139)
* :func:`synthesize`         -- ``synthesize`` (src/synthesize.jl:138-324)

Arrays follow Korg's memory layout: alpha is (layers x wavelengths) column-major, i.e. a numpy
array of shape (L, nwl) in Fortran order (equivalently (nwl, L) in C order).  ``precision`` is
``"fp64"`` (the plain form) or ``"mixed"``.
"""
from __future__ import annotations

import ctypes as C
import functools
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .constants import c_cgs
from .data import default_partition_funcs
from .linelist import LineList, alpha_5000_linelist, filter_linelist
from .species import Species, atomic_masses, parse_species
from .wavelengths import Wavelengths

_PREC = {"fp64": _lib.KORG_FP64, "mixed": _lib.KORG_MIXED}

# line_absorption.jl:54-58: perturber-density coefficients of He and H2 relative to H
_a_H, _a_He, _a_H2 = 4.50711, 1.38375, 5.503
C_HE = (_a_He / _a_H) ** 0.4 * (atomic_masses[1] / atomic_masses[0]) ** -0.3
C_H2 = (_a_H2 / _a_H) ** 0.4 * 2 ** -0.3


def _prec(p):
    try:
        return _PREC[p]
    except KeyError:
        raise ValueError(f"precision must be 'fp64' or 'mixed', got {p!r}") from None


def _alpha_buffer(alpha, L, nwl):
    """View alpha as a contiguous buffer in Korg's layout; returns (buffer, writeback)."""
    a = np.asarray(alpha)
    if a.dtype != np.float64:
        raise TypeError("alpha must be float64")
    if a.shape == (L, nwl) and a.flags.f_contiguous:
        return a.T, None  # (nwl, L) C-contiguous view of the same memory
    if a.shape == (nwl, L) and a.flags.c_contiguous:
        return a, None
    if a.shape == (L, nwl):
        buf = np.ascontiguousarray(a.T)
        return buf, lambda: np.copyto(a, buf.T)
    raise ValueError(f"alpha must have shape (L, nwl) = ({L}, {nwl})")


def n_div_U_matrix(species, n_densities, partition_fns, temps):
    """Rows n(species)/U(species, ln T) per layer (line_absorption.jl:42-44)."""
    lnT = np.log(np.asarray(temps, np.float64))
    rows = []
    for s in species:
        if s not in n_densities:
            raise KeyError(f"no number density for {s}")
        rows.append(np.asarray(n_densities[s], np.float64) / partition_fns[s](lnT))
    return np.ascontiguousarray(np.array(rows).reshape(len(species), len(lnT)))


def n_eff_vdW(n_densities, L):
    """line_absorption.jl:59-60"""
    z = np.zeros(L)
    g = lambda s: np.asarray(n_densities.get(parse_species(s), z), np.float64)
    return g("H I") + C_HE * g("He I") + C_H2 * g("H2")


class ContinuumInterpolant:
    """The per-layer continuum callables alpha_cntm[l](wl): piecewise linear over ``knots`` (cm)
    with ``vals`` of shape (L, nk) (src/synthesize.jl:226-228).  A 1-knot interpolant is a
    constant per layer."""

    def __init__(self, knots, vals):
        self.knots = np.ascontiguousarray(knots, np.float64)
        self.vals = np.ascontiguousarray(vals, np.float64)

    @classmethod
    def constant(cls, values):
        v = np.asarray(values, np.float64)
        return cls(np.zeros(1), v.reshape(-1, 1))


def line_absorption_(alpha, linelist: LineList, wls, temps, ne, n_densities, partition_fns, xi, alpha_cntm,
                     cutoff_threshold=3e-4, precision="fp64", ctx=None):
    """``line_absorption!``: add line opacity to ``alpha`` (L x nwl) in place.  Returns the
    number of line-layer-wavelength profile evaluations."""
    wls = Wavelengths(wls) if not isinstance(wls, Wavelengths) else wls
    temps = np.asarray(temps, np.float64)
    L, nwl = len(temps), len(wls)
    if len(linelist) == 0:
        return 0  # line_absorption.jl:35-37
    if parse_species("H I") in linelist.species:
        import warnings
        warnings.warn("Atomic hydrogen should not be in the linelist. Korg has built-in hydrogen lines.")
    ctx = ctx or _lib.default_context()
    keep = _lib.Keep()
    nU = n_div_U_matrix(linelist.species, n_densities, partition_fns, temps)
    xi_l = np.broadcast_to(np.asarray(xi, np.float64), (L,))
    lay = _lib.Layers(L, nU.shape[0], _lib._p(keep.f64(temps)), _lib._p(keep.f64(ne)),
                      _lib._p(keep.f64(n_eff_vdW(n_densities, L))), _lib._p(keep.f64(xi_l)), _lib._p(keep.f64(nU)))
    if isinstance(alpha_cntm, ContinuumInterpolant):
        ci = alpha_cntm
    else:
        ci = ContinuumInterpolant.constant(alpha_cntm)
    cn = _lib.Cntm(len(ci.knots), _lib._p(keep.f64(ci.knots)), _lib._p(keep.f64(ci.vals)))
    lines = _lib.lines_struct(linelist, keep)
    buf, wb = _alpha_buffer(alpha, L, nwl)
    n = C.c_int64(0)
    ctx.check(ctx.lib.korg_line_absorption(ctx.h, _lib._p(buf), _lib._p(keep.f64(wls.all_wls)), nwl, C.byref(lines),
                                           C.byref(lay), C.byref(cn), cutoff_threshold, _prec(precision),
                                           C.byref(n)))
    if wb:
        wb()
    return n.value


def hydrogen_line_absorption_(alphas, wls, T, ne, nH_I, nHe_I, UH_I, xi, window_size, use_MHD=True,
                              precision="fp64", ctx=None):
    """``hydrogen_line_absorption!`` for one layer: add to ``alphas`` (nwl) in place."""
    wls = Wavelengths(wls) if not isinstance(wls, Wavelengths) else wls
    ctx = ctx or _lib.default_context()
    ctx.ensure_stark()
    a = np.asarray(alphas)
    if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != (len(wls),):
        raise ValueError("alphas must be a contiguous float64 vector over the wavelengths")
    w = np.ascontiguousarray(wls.all_wls)
    ctx.check(ctx.lib.korg_hydrogen_line_absorption(ctx.h, _lib._p(a), _lib._p(w), len(w), float(T), float(ne),
                                                    float(nH_I), float(nHe_I), float(UH_I), float(xi),
                                                    float(window_size), int(bool(use_MHD)), _prec(precision)))


def generate_mu_grid(mu_points):
    """RadiativeTransfer.jl:13-30: Gauss-Legendre on [0, 1] for an integer, trapezoid weights for
    an explicit sorted grid in [0, 1]."""
    if np.ndim(mu_points) == 0:
        mu, w = np.polynomial.legendre.leggauss(int(mu_points))
        return mu / 2 + 0.5, w / 2
    mu = np.asarray(mu_points, np.float64)
    if len(mu) == 1:
        return mu, np.array([1.0])
    if np.any(np.diff(mu) < 0) or mu[0] < 0 or mu[-1] > 1:
        raise ValueError("mu_grid must be sorted and bounded between 0 and 1")
    d = np.diff(mu)
    return mu, 0.5 * np.concatenate([[d[0]], d[:-1] + d[1:], [d[-1]]])


_TAU = {"anchored": 0, "bezier": 1}
_ISCHEME = {"linear": 0, "linear_flux_only": 1, "bezier": 2}


def radiative_transfer(atm, alpha, S, mu_points, alpha_ref=None, tau_ref=None, tau_scheme="anchored",
                       I_scheme=None, include_inward_rays=False, spherical=None, spatial_coord=None, R=None,
                       ctx=None):
    """``RadiativeTransfer.radiative_transfer(atm, alpha, S, mu_points; alpha_ref, tau_ref,
    tau_scheme, I_scheme)`` (RadiativeTransfer.jl:62-139).  ``atm`` supplies tau_ref and the
    heights (``atm.z``); ``spherical=True`` with radius ``R`` makes it a shell atmosphere
    (radii R + z, default I_scheme "linear" and the photosphere correction of :73).  Returns
    (F, I_surface (n_mu x nwl), mu_grid, mu_weights).  The planar default (anchored tau,
    linear_flux_only) is the exponential-integral flux on one ray (:81-84); every other
    combination runs korg_radiative_transfer_general."""
    if tau_scheme not in _TAU:
        raise ValueError('tau_scheme must be one of "anchored" or "bezier"')
    spherical = bool(R is not None) if spherical is None else spherical
    I_scheme = I_scheme or ("linear" if spherical else "linear_flux_only")
    if I_scheme not in _ISCHEME:
        raise ValueError('I_scheme must be one of "linear", "bezier", or "linear_flux_only"')
    tau_ref = atm.tau_ref if tau_ref is None else tau_ref
    tau_ref = np.asarray(tau_ref, np.float64)
    L = len(tau_ref)
    a = np.asarray(alpha)
    nwl = a.size // L
    abuf, _ = _alpha_buffer(a, L, nwl)
    sbuf, _ = _alpha_buffer(np.asarray(S), L, nwl)
    ctx = ctx or _lib.default_context()
    keep = _lib.Keep()
    F = np.empty(nwl)
    if I_scheme == "linear_flux_only" and tau_scheme == "anchored" and not spherical:
        ctx.check(ctx.lib.korg_radiative_transfer(ctx.h, _lib._p(abuf), _lib._p(sbuf), L, nwl,
                                                  _lib._p(keep.f64(tau_ref)), _lib._p(keep.f64(alpha_ref)),
                                                  _lib._p(F)))
        return F, (F / (2 * np.pi)).reshape(1, nwl), np.array([1.0]), np.array([1.0])
    mu, w = generate_mu_grid(mu_points)
    if spatial_coord is None:
        z = np.asarray(atm.z, np.float64)
        spatial_coord = (R + z) if spherical else z
    spatial_coord = keep.f64(spatial_coord)
    Isurf = np.empty((len(mu), nwl))
    ctx.check(ctx.lib.korg_radiative_transfer_general(
        ctx.h, _lib._p(abuf), _lib._p(sbuf), L, nwl, _lib._p(spatial_coord), int(spherical),
        _lib._p(keep.f64(tau_ref)), _lib._p(keep.f64(alpha_ref)), _lib._p(keep.f64(mu)), _lib._p(keep.f64(w)),
        len(mu), int(bool(include_inward_rays)), _TAU[tau_scheme], _ISCHEME[I_scheme], _lib._p(F),
        _lib._p(Isurf)))
    if spherical and R is not None:
        F = F * (spatial_coord[0] ** 2 / R ** 2)  # photosphere correction (:73)
    return F, Isurf, mu, w


# ---------------------------------------------------------------------------------- synthesize


@dataclass
class SynthesisInputs:
    """Everything synthesize() computes on the host before the hot path
    (src/synthesize.jl:159-262), for one atmosphere."""

    wls: Wavelengths
    linelist: LineList
    linelist5: LineList
    T: np.ndarray
    ne: np.ndarray
    tau_ref: np.ndarray
    xi: np.ndarray
    n_eff_vdW: np.ndarray
    n_div_U: np.ndarray          # (S, L), rows follow linelist.species (shared with linelist5)
    nH_I: np.ndarray
    nHe_I: np.ndarray
    UH_I: np.ndarray
    alpha_ref_cntm: np.ndarray
    cntm_knots: np.ndarray
    cntm_vals: np.ndarray        # (L, nk)
    ref_wl: float = 5e-5
    hydrogen_lines: bool = True
    use_MHD: bool = True
    hydrogen_window: float = 150e-8
    cutoff_threshold: float = 3e-4
    number_densities: dict = field(default_factory=dict)
    # what the chemical equilibrium was solved from (chemistry="gpu"): n_tot, the model n_e and the
    # normalised abundances, per layer / per element; None otherwise
    chemistry: tuple | None = None

    def struct(self, keep):
        L = len(self.T)
        lay = _lib.Layers(L, self.n_div_U.shape[0], _lib._p(keep.f64(self.T)), _lib._p(keep.f64(self.ne)),
                          _lib._p(keep.f64(self.n_eff_vdW)), _lib._p(keep.f64(self.xi)),
                          _lib._p(keep.f64(self.n_div_U)))
        return _lib.SynthInputs(lay, _lib._p(keep.f64(self.tau_ref)), _lib._p(keep.f64(self.alpha_ref_cntm)),
                                _lib._p(keep.f64(self.nH_I)), _lib._p(keep.f64(self.nHe_I)),
                                _lib._p(keep.f64(self.UH_I)), self.ref_wl,
                                _lib.Cntm(len(self.cntm_knots), _lib._p(keep.f64(self.cntm_knots)),
                                          _lib._p(keep.f64(self.cntm_vals))),
                                int(self.hydrogen_lines), int(self.use_MHD), self.hydrogen_window,
                                self.cutoff_threshold)


@dataclass
class SynthesisResult:
    """src/synthesize.jl:30-41 (alpha only when requested)."""

    flux: np.ndarray
    cntm: np.ndarray
    alpha: np.ndarray | None
    alpha_ref: np.ndarray | None
    wavelengths: np.ndarray
    subspectra: list
    line_evals: int = 0


def _merge_windows(wins):
    wins = sorted(wins)
    out = [list(wins[0])]
    for a, b in wins[1:]:
        if a <= out[-1][1]:
            out[-1][1] = max(out[-1][1], b)
        else:
            out.append([a, b])
    return [tuple(w) for w in out]


def prepare_synthesis(atm, linelist: LineList, A_X, wavelengths, vmic=1.0, line_buffer=10.0, cntm_step=1.0,
                      hydrogen_lines=True, use_MHD_for_hydrogen_lines=None, hydrogen_line_window_size=150,
                      line_cutoff_threshold=3e-4, use_internal_reference_linelist=True,
                      chemical_equilibrium=None, continuum_opacity=None, continuum="standin", chemistry="standin",
                      ctx=None):
    """The host part of synthesize (src/synthesize.jl:159-262).  Chemical equilibrium:
    ``chemistry="gpu"`` solves Korg's chemical equilibrium for every layer on the device
    (:func:`korg_gb300.statmech.chemical_equilibrium`, src/synthesize.jl:207-219), starting from
    the atmosphere's n_e; a callable ``chemistry(T, n_tot, ne_model, absolute_abundances) ->
    (ne, {Species: n})`` over the layers (the reference's argument order) does the same with
    another solver; ``"standin"`` (the default, CPU only) uses the compact stand-in of
    :mod:`korg_gb300.standin`; a ``chemical_equilibrium(T, n_tot, A_X) -> (ne, {Species: n})``
    callable overrides all of them.  The continuum: ``continuum="gpu"`` evaluates Korg's
    continuum absorption (every term but metal bound-free) on the device
    (:mod:`korg_gb300.continuum`); ``"standin"`` (the default, CPU only) the compact stand-in; a
    ``continuum_opacity(wls_cm, T, ne, n_HI, n_HII) -> alpha`` callable overrides both."""
    from . import standin
    if chemical_equilibrium is not None:
        chem = chemical_equilibrium
    elif chemistry == "standin":
        chem = standin.chemical_equilibrium
    elif chemistry == "gpu" or callable(chemistry):
        def chem(T, n_tot, A_X):
            if chemistry == "gpu":
                from .statmech import chemical_equilibrium
                solve = functools.partial(chemical_equilibrium, ctx=ctx)
            else:
                solve = chemistry
            ab = 10.0 ** (np.asarray(A_X, np.float64) - 12)  # :204-209
            return solve(T, n_tot, np.asarray(atm.ne, np.float64), ab / ab.sum())
    else:
        raise ValueError(f'chemistry must be "gpu", "standin" or a callable, got {chemistry!r}')
    cont = continuum_opacity or standin.continuum_opacity
    wls = wavelengths if isinstance(wavelengths, Wavelengths) else Wavelengths(wavelengths)
    use_MHD = (wls.all_wls[-1] < 13_000e-8) if use_MHD_for_hydrogen_lines is None else use_MHD_for_hydrogen_lines
    if wls.all_wls[0] < 1300e-8:  # :170-177
        raise ValueError("Requested wavelength range extends blue-ward of 1300 A, the lowest allowed wavelength.")
    cstep, lbuf = cntm_step * 1e-8, line_buffer * 1e-8
    wins = _merge_windows([(a - lbuf - cstep, b + lbuf + cstep) for a, b in wls.eachwindow()])
    cntm_wls = Wavelengths([(a, b, cstep) for a, b in wins])
    if not linelist.is_sorted():  # :191-194
        linelist = linelist.sorted()
    if atm.reference_wavelength == 5e-5 and use_internal_reference_linelist:
        ll5 = alpha_5000_linelist()
    else:
        raise NotImplementedError("only the built-in 5000 A reference line list is supported")
    linelist = filter_linelist(linelist, wls, lbuf)
    # one species table for both lists
    ll = linelist.concat(ll5.subset(np.zeros(0, dtype=np.int64)))
    species = list(ll.species)
    remap = []
    for s in ll5.species:
        if s not in species:
            species.append(s)
        remap.append(species.index(s))
    ll = LineList(ll.wl, ll.log_gf, ll.species_idx, species, ll.E_lower, ll.gamma_rad, ll.gamma_stark, ll.vdW1,
                  ll.vdW2)
    remap = np.asarray(remap, np.int32)
    ll5 = LineList(ll5.wl, ll5.log_gf, remap[ll5.species_idx], species, ll5.E_lower, ll5.gamma_rad,
                   ll5.gamma_stark, ll5.vdW1, ll5.vdW2)
    T = np.asarray(atm.T, np.float64)
    L = len(T)
    ne, nd = chem(T, atm.n_tot, A_X)
    pf = default_partition_funcs()
    for s in species:  # species the stand-in does not form get zero density
        nd.setdefault(s, np.zeros(L))
    H1, H2, He1 = parse_species("H I"), parse_species("H II"), parse_species("He I")
    if continuum_opacity is None and continuum == "gpu":  # src/synthesize.jl:225-235 on the device
        from .continuum import continuum_absorption
        vals = continuum_absorption(cntm_wls.all_wls, T, ne, nd, pf, ctx=ctx)
        aref = continuum_absorption(np.array([atm.reference_wavelength]), T, ne, nd, pf, ctx=ctx)[:, 0].copy()
    elif continuum_opacity is None and continuum != "standin":
        raise ValueError(f'continuum must be "gpu" or "standin", got {continuum!r}')
    else:
        vals = np.empty((L, len(cntm_wls)))
        aref = np.empty(L)
        for l in range(L):
            vals[l] = cont(cntm_wls.all_wls, T[l], ne[l], nd[H1][l], nd[H2][l])
            aref[l] = cont(np.array([atm.reference_wavelength]), T[l], ne[l], nd[H1][l], nd[H2][l])[0]
    xi = np.broadcast_to(np.asarray(vmic, np.float64) * 1e5, (L,)).copy()
    return SynthesisInputs(
        wls=wls, linelist=ll, linelist5=ll5, T=T, ne=np.asarray(ne, np.float64),
        tau_ref=np.asarray(atm.tau_ref, np.float64), xi=xi, n_eff_vdW=n_eff_vdW(nd, L),
        n_div_U=n_div_U_matrix(species, nd, pf, T), nH_I=nd[H1], nHe_I=nd[He1],
        UH_I=pf[H1](np.log(T)), alpha_ref_cntm=aref, cntm_knots=cntm_wls.all_wls, cntm_vals=vals,
        ref_wl=atm.reference_wavelength, hydrogen_lines=hydrogen_lines, use_MHD=bool(use_MHD),
        hydrogen_window=hydrogen_line_window_size * 1e-8, cutoff_threshold=line_cutoff_threshold,
        number_densities=nd,
        chemistry=(np.asarray(atm.n_tot, np.float64), np.asarray(atm.ne, np.float64),
                   10.0 ** (np.asarray(A_X, np.float64) - 12) / np.sum(10.0 ** (np.asarray(A_X, np.float64) - 12)))
        if chemical_equilibrium is None and chemistry == "gpu" else None)


def synthesize_prepared(inp: SynthesisInputs, precision="mixed", return_alpha=False, ctx=None) -> SynthesisResult:
    """Run the hot path (src/synthesize.jl:249-318) on prepared inputs through korg_synthesize."""
    ctx = ctx or _lib.default_context()
    if inp.hydrogen_lines:
        ctx.ensure_stark()
    keep = _lib.Keep()
    s = inp.struct(keep)
    lines = _lib.lines_struct(inp.linelist, keep)
    lines5 = _lib.lines_struct(inp.linelist5, keep)
    nwl, L = len(inp.wls), len(inp.T)
    flux, cntm = np.empty(nwl), np.empty(nwl)
    alpha = np.empty((nwl, L)) if return_alpha else None
    aref = np.empty(L)
    w = keep.f64(inp.wls.all_wls)
    ctx.check(ctx.lib.korg_synthesize(ctx.h, C.byref(s), C.byref(lines), C.byref(lines5), _lib._p(w), nwl,
                                      _prec(precision), _lib._p(flux), _lib._p(cntm), _lib._p(alpha), _lib._p(aref)))
    return SynthesisResult(flux=flux, cntm=cntm, alpha=None if alpha is None else alpha.T, alpha_ref=aref,
                           wavelengths=inp.wls.all_wls_angstrom, subspectra=inp.wls.subspectrum_indices(),
                           line_evals=ctx.stats().line_evals)


def synthesize(atm, linelist, A_X, wavelengths, precision="mixed", return_alpha=False, ctx=None, continuum="gpu",
               chemistry="gpu", **kwargs):
    """``synthesize(atm, linelist, A_X, wavelengths; kwargs...)`` (src/synthesize.jl:138-324), with
    chemical equilibrium and continuum absorption evaluated on the device by default (see
    :func:`prepare_synthesis`)."""
    inp = prepare_synthesis(atm, linelist, A_X, wavelengths, continuum=continuum, chemistry=chemistry, ctx=ctx,
                            **kwargs)
    return synthesize_prepared(inp, precision=precision, return_alpha=return_alpha, ctx=ctx)


# ---------------------------------------------------------------------------------- reverse mode

GRAD_FIELDS = ("T", "ne", "n_eff_vdW", "xi", "n_div_U", "nH_I", "nHe_I", "UH_I", "log_gf", "cntm_vals",
               "alpha_ref_cntm")


def synthesize_vjp(inp: SynthesisInputs, dflux, dcntm=None, precision="fp64", hydrogen=True, wanted=GRAD_FIELDS,
                   reuse_forward=False, ctx=None):
    """Vector-Jacobian product of :func:`synthesize_prepared` (korg_synthesize_vjp): the
    gradient of sum(dflux * flux + dcntm * cntm) with respect to the hot-path inputs, as a dict
    keyed by GRAD_FIELDS (shapes: [L], n_div_U [S, L], log_gf [n lines], cntm_vals [L, nk]).
    reuse_forward: the previous call on ``ctx`` was synthesize_prepared of the same inputs and
    precision; its opacity is reused instead of recomputed.  hydrogen: differentiate the
    hydrogen lines too (the exact derivatives of their approximation with respect to T, ne, xi,
    nH_I, nHe_I, UH_I); False holds them fixed."""
    ctx = ctx or _lib.default_context()
    if inp.hydrogen_lines:
        ctx.ensure_stark()
    keep = _lib.Keep()
    s = inp.struct(keep)
    lines = _lib.lines_struct(inp.linelist, keep)
    lines5 = _lib.lines_struct(inp.linelist5, keep)
    L, nwl = len(inp.T), len(inp.wls)
    shapes = {"n_div_U": inp.n_div_U.shape, "log_gf": (len(inp.linelist),), "cntm_vals": inp.cntm_vals.shape}
    out = {k: np.zeros(shapes.get(k, (L,))) for k in wanted}
    g = _lib.SynthGrads(*[_lib._p(out[k]) if k in out else None for k in GRAD_FIELDS])
    df = None if dflux is None else keep.f64(dflux)
    dc = None if dcntm is None else keep.f64(dcntm)
    w = keep.f64(inp.wls.all_wls)
    ctx.check(ctx.lib.korg_synthesize_vjp(ctx.h, C.byref(s), C.byref(lines), C.byref(lines5), _lib._p(w), nwl,
                                          _prec(precision), _lib._p(df), _lib._p(dc), C.byref(g),
                                          (_lib.KORG_VJP_HYDROGEN if hydrogen else 0) |
                                          (_lib.KORG_VJP_REUSE_FORWARD if reuse_forward else 0)))
    return out


def rectified_loss(flux, cntm, obs):
    """loss = sum((flux/cntm - obs)^2) and its cotangents (dL/dflux, dL/dcntm)."""
    r = flux / cntm - obs
    return float(np.sum(r * r)), 2 * r / cntm, -2 * r * flux / cntm ** 2


def loss_and_gradient(inp: SynthesisInputs, obs, precision="fp64", hydrogen=True, reuse_forward=False, ctx=None):
    """Rectified-flux least squares against ``obs`` and its gradient with respect to the
    hot-path inputs (a forward synthesis, then the reverse mode)."""
    ctx = ctx or _lib.default_context()
    res = synthesize_prepared(inp, precision=precision, ctx=ctx)
    loss, dF, dC = rectified_loss(res.flux, res.cntm, obs)
    return loss, synthesize_vjp(inp, dF, dC, precision=precision, hydrogen=hydrogen, reuse_forward=reuse_forward,
                                ctx=ctx)


def atmosphere_gradient(inp: SynthesisInputs, g, ctx=None):
    """Gradient of a synthesis loss with respect to the model atmosphere's layer temperatures and
    total number densities and the abundances A(X), through Korg's continuum absorption and chemical
    equilibrium as prepare_synthesis(chemistry="gpu", continuum="gpu") evaluated them: what
    ForwardDiff through synthesize gives for those inputs (src/Fit/fit_via_synthesis.jl:345-355).
    ``g`` is the hot-path gradient (:func:`synthesize_vjp`).  The chain: the hot path's own
    dependences (:func:`physical_gradient`), the continuum's (central differences of the device
    kernel, :func:`korg_gb300.continuum.absorption_vjp`), then the chemical equilibrium's
    (implicit-function rule on the device, korg_chemical_equilibrium_vjp); A(X) enters through the
    normalised abundances 10^(A(X) - 12) / sum.  Returns {"T", "n_tot", "A_X", "vmic", "log_gf"}."""
    from .continuum import absorption_vjp, layer_inputs, layer_inputs_vjp
    from .statmech import chemical_equilibrium_vjp, default_equilibrium_tables
    if inp.chemistry is None:
        raise ValueError('needs inputs prepared with chemistry="gpu"')
    n_tot, ne_model, ab = inp.chemistry
    pf = default_partition_funcs()
    T = inp.T
    L = len(T)
    phys = physical_gradient(inp, g)
    dT, dne, dn = phys["T"].copy(), np.array(phys["ne"], np.float64), dict(phys["n"])
    d = layer_inputs(T, inp.ne, inp.number_densities, pf)
    gk = absorption_vjp(inp.cntm_knots, d, g["cntm_vals"], ctx)
    gr = absorption_vjp(np.array([inp.ref_wl]), d, np.asarray(g["alpha_ref_cntm"])[:, None], ctx)
    cT, cne, cn = layer_inputs_vjp({k: gk[k] + gr[k] for k in gk}, T, inp.number_densities, pf)
    dT += cT
    dne += cne
    for s, v in cn.items():
        dn[s] = dn.get(s, 0.0) + v
    species = default_equilibrium_tables().species
    col = {s: k for k, s in enumerate(species) if s is not None}
    dens = np.empty((L, len(species)))
    dens[:, 0] = inp.ne
    for s, k in col.items():
        dens[:, k] = np.broadcast_to(np.asarray(inp.number_densities[s], np.float64), (L,))
    gbar = np.zeros_like(dens)
    gbar[:, 0] = dne
    for s, v in dn.items():
        if s in col:  # species outside the chemical equilibrium have no density to differentiate
            gbar[:, col[s]] += v
    chT, dnt, dab = chemical_equilibrium_vjp(T, n_tot, ne_model, ab, dens, gbar, ctx=ctx)
    dT += chT
    return {"T": dT, "n_tot": dnt, "A_X": abundance_vjp(ab, dab.sum(axis=0)), "vmic": phys["vmic"],
            "log_gf": phys["log_gf"]}


def abundance_vjp(ab, gbar_ab):
    """Reverse mode of the normalisation ab = 10^(A(X) - 12) / sum (src/synthesize.jl:204-209):
    the cotangent of the normalised abundances ``ab`` to dL/dA(X),
    ln 10 ab_Z (gbar_Z - sum_Y ab_Y gbar_Y)."""
    ab, gbar_ab = np.asarray(ab, np.float64), np.asarray(gbar_ab, np.float64)
    return np.log(10.0) * ab * (gbar_ab - np.dot(ab, gbar_ab))


def physical_gradient(inp: SynthesisInputs, g, vmic_scalar=True):
    """Chain rule from the hot-path inputs to the quantities a fit varies, holding the continuum
    opacity fixed: layer temperatures (through n/U(T) and U_HI(T) as well), electron density,
    number densities per species (through n/U, n_eff_vdW and the hydrogen-line inputs),
    microturbulence (km/s) and log gf per line."""
    pf = default_partition_funcs()
    T = inp.T
    lnT = np.log(T)
    dT = g["T"].copy()
    dn = {}
    for k, sp in enumerate(inp.linelist.species):
        U = pf[sp](lnT)
        dU = pf[sp].derivative(lnT) / T
        n = inp.n_div_U[k] * U
        dn[sp] = dn.get(sp, 0.0) + g["n_div_U"][k] / U
        dT += -g["n_div_U"][k] * n * dU / U ** 2
    H1, He1, H2 = parse_species("H I"), parse_species("He I"), parse_species("H2")
    dn[H1] = dn.get(H1, 0.0) + g["n_eff_vdW"] + g.get("nH_I", 0.0)
    dn[He1] = dn.get(He1, 0.0) + C_HE * g["n_eff_vdW"] + g.get("nHe_I", 0.0)
    dn[H2] = dn.get(H2, 0.0) + C_H2 * g["n_eff_vdW"]
    if "UH_I" in g:
        dT += g["UH_I"] * pf[H1].derivative(lnT) / T
    dvmic = g["xi"] * 1e5
    return {"T": dT, "ne": g["ne"], "n": dn, "vmic": float(np.sum(dvmic)) if vmic_scalar else dvmic,
            "log_gf": g["log_gf"]}
