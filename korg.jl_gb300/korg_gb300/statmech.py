"""Chemical equilibrium on the GPU (korg_chemical_equilibrium), with the reference's interface.

* :func:`chemical_equilibrium` -- ``chemical_equilibrium(T, n_tot, ne, absolute_abundances,
  ionization_energies, partition_fns, log_equilibrium_constants)`` (src/statmech.jl:148-206) for
  one layer (scalars) or every layer of an atmosphere (arrays), returning ``(ne, {Species: n})``;
* :func:`solve_layers` -- the batched form over many atmospheres (a layer -> atmosphere map and
  one abundance vector per atmosphere), returning the dense [layers, species] density matrix;
* :func:`saha_ion_weights`, :func:`translational_U`, :func:`get_log_nK`, :func:`Hminus_nK` --
  the reference's host helpers (src/statmech.jl:19-79).

The solve runs on the device (csrc/statmech.cuh).  The tables it needs are built from the same
dicts the reference takes: partition functions and log10 equilibrium constants must be
CubicSpline objects (or PolyatomicLogK for the polyatomics), as the package's data loaders return
them.
"""
from __future__ import annotations

import ctypes as C
import functools
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .constants import electron_mass_cgs, hplanck_cgs, kboltz_cgs, kboltz_eV
from .cubic_spline import CubicSpline
from .species import Species

MAX_ATOMIC_NUMBER = 92
HMINUS = Species([1], -1)
_STATUS = {1: "unconverged at anchor", 2: "unconverged during the log xi continuation",
           3: "solution contains non-finite values", 4: "more than 20000 Newton iterations"}


class ChemicalEquilibriumError(Exception):
    """src/statmech.jl:81-86."""


def translational_U(m, T):
    """src/statmech.jl:47-51."""
    return (2 * np.pi * m * kboltz_cgs * T / hplanck_cgs ** 2) ** 1.5


def saha_ion_weights(T, ne, atom, ionization_energies, partition_funcs):
    """(wII, wIII) = n(X II)/n(X I), n(X III)/n(X I) of element ``atom`` (src/statmech.jl:19-35)."""
    chiI, chiII, _ = ionization_energies[atom]
    lnT = np.log(T)
    UI = partition_funcs[Species([atom], 0)](lnT)
    UII = partition_funcs[Species([atom], 1)](lnT)
    transU = translational_U(electron_mass_cgs, T)
    wII = 2.0 / ne * (UII / UI) * transU * np.exp(-chiI / (kboltz_eV * T))
    if atom == 1:
        return wII, 0.0 * wII
    UIII = partition_funcs[Species([atom], 2)](lnT)
    return wII, wII * 2.0 / ne * (UIII / UII) * transU * np.exp(-chiII / (kboltz_eV * T))


def get_log_nK(mol, T, log_equilibrium_constants):
    """log10 of n(A) n(B) ... / n(mol) (src/statmech.jl:60-62)."""
    return log_equilibrium_constants[mol](np.log(T)) - (len(mol.atoms) - 1) * np.log10(kboltz_cgs * T)


def Hminus_nK(T):
    """n(H-) = nK(T) n(H I) n_e (src/statmech.jl:73-79)."""
    return np.exp(0.754204 / (kboltz_eV * T)) / (4 * translational_U(electron_mass_cgs, T))


@dataclass(eq=False)
class EquilibriumTables:
    """The arrays of korg_equilibrium_tables and the species order of the density matrix."""
    lnT: np.ndarray
    U_u: np.ndarray
    U_z: np.ndarray
    chi: np.ndarray
    molecules: list
    atoms: np.ndarray
    charge: np.ndarray
    kind: np.ndarray
    off: np.ndarray
    spl_t: np.ndarray
    spl_u: np.ndarray
    spl_z: np.ndarray
    D00: np.ndarray
    lmr: np.ndarray
    species: list = field(default_factory=list)

    @classmethod
    def from_dicts(cls, ionization_energies, partition_funcs, log_equilibrium_constants):
        from .data import PolyatomicLogK
        ref = partition_funcs[Species([1], 0)]
        lnT = np.asarray(ref.t, np.float64)
        nk = len(lnT)
        U_u, U_z = np.zeros((3 * MAX_ATOMIC_NUMBER, nk)), np.zeros((3 * MAX_ATOMIC_NUMBER, nk))
        for Z in range(1, MAX_ATOMIC_NUMBER + 1):
            for q in range(3):
                if Z == 1 and q == 2:
                    continue
                spl = partition_funcs[Species([Z], q)]
                if not isinstance(spl, CubicSpline) or not np.array_equal(spl.t, lnT):
                    raise NotImplementedError("atomic partition functions must be CubicSplines on shared knots")
                U_u[3 * (Z - 1) + q], U_z[3 * (Z - 1) + q] = spl.u, spl.z
        chi = np.array([ionization_energies[Z][:3] for Z in range(1, MAX_ATOMIC_NUMBER + 1)], np.float64)
        mols = list(log_equilibrium_constants)
        if len(mols) > _lib.KORG_CHEM_MAX_MOL:
            raise ValueError(f"at most {_lib.KORG_CHEM_MAX_MOL} molecules")
        atoms = np.zeros((len(mols), 6), np.int32)
        charge, kind = np.zeros(len(mols), np.int32), np.zeros(len(mols), np.int32)
        D00, lmr = np.zeros(len(mols)), np.zeros(len(mols))
        ts, us, zs, off = [], [], [], [0]
        for m, spec in enumerate(mols):
            f = log_equilibrium_constants[spec]
            if len(spec.atoms) > 6 or spec.charge not in (0, 1):
                raise NotImplementedError(f"{spec}: up to 6 atoms, neutral or singly ionized")
            atoms[m, :len(spec.atoms)] = sorted(spec.atoms)
            charge[m] = spec.charge
            if isinstance(f, PolyatomicLogK):
                for Z, U in zip(f.Zs, f.U_atoms):
                    if U is not partition_funcs[Species([Z], 0)]:
                        raise NotImplementedError(f"{spec}: its atoms' partition functions must be the atomic ones")
                kind[m], D00[m], lmr[m], spl = 1, f.D00, f.log_masses_ratio, f.U_mol
            elif isinstance(f, CubicSpline):
                spl = f
            else:
                raise NotImplementedError(f"{spec}: log equilibrium constants must be CubicSpline or PolyatomicLogK")
            ts.append(spl.t)
            us.append(spl.u)
            zs.append(spl.z)
            off.append(off[-1] + len(spl.t))
        species = ([None] + [Species([Z], q) for Z in range(1, MAX_ATOMIC_NUMBER + 1) for q in range(3)] +
                   [HMINUS] + mols)
        cat = lambda v: np.concatenate(v) if v else np.zeros(1)
        return cls(lnT, U_u, U_z, chi, mols, atoms, charge, kind, np.array(off, np.int64), cat(ts), cat(us), cat(zs),
                   D00, lmr, species)


@functools.lru_cache(maxsize=None)
def default_equilibrium_tables():
    from .data import default_log_equilibrium_constants, default_partition_funcs, ionization_energies
    return EquilibriumTables.from_dicts(ionization_energies(), default_partition_funcs(),
                                        default_log_equilibrium_constants())


def _tables(ionization_energies, partition_funcs, log_equilibrium_constants):
    if ionization_energies is None and partition_funcs is None and log_equilibrium_constants is None:
        return default_equilibrium_tables()
    from .data import default_log_equilibrium_constants, default_partition_funcs
    from .data import ionization_energies as default_ionization_energies
    return EquilibriumTables.from_dicts(ionization_energies or default_ionization_energies(),
                                        partition_funcs or default_partition_funcs(),
                                        log_equilibrium_constants or default_log_equilibrium_constants())


def solve_layers(T, n_tot, ne_model, abundances, atm=None, tables=None, ctx=None, raise_on_failure=True):
    """Chemical equilibrium of every layer on the device (korg_chemical_equilibrium).

    ``abundances`` is [n_atm, 92] (N_X / N_total, normalised) or [92]; ``atm`` maps each layer to
    its atmosphere.  Returns (densities [L, 278 + n_mol] in the order of ``tables.species`` -- n_e
    first --, status [L], info [L, 5]: Newton iterations, solves, log xi reached, last inf-norm,
    steps solved by the FP64 fallback)."""
    ctx = ctx or _lib.default_context()
    t = ctx.ensure_equilibrium(tables)
    keep = _lib.Keep()
    T = keep.f64(np.atleast_1d(T))
    L = len(T)
    nt = keep.f64(np.broadcast_to(np.asarray(n_tot, np.float64), (L,)))
    ne = keep.f64(np.broadcast_to(np.asarray(ne_model, np.float64), (L,)))
    ab = keep.f64(np.atleast_2d(abundances))
    if ab.shape[1] != MAX_ATOMIC_NUMBER:
        raise ValueError("abundances must have 92 entries per atmosphere")
    at = None if atm is None else keep.i32(atm)
    if at is not None and len(at) != L:
        raise ValueError("atm must have one entry per layer")
    dens = np.empty((L, _lib.KORG_CHEM_MOL0 + len(t.molecules)))
    status = np.empty(L, np.int32)
    info = np.empty((L, 5))
    y = _lib.ChemLayers(L, _lib._p(T), _lib._p(nt), _lib._p(ne), _lib._p(ab), _lib._p(at, _lib._ip))
    rc = ctx.lib.korg_chemical_equilibrium(ctx.h, C.byref(y), ab.shape[0], _lib._p(dens),
                                           _lib._p(status, _lib._ip), _lib._p(info))
    if rc == _lib.KORG_ECHEM:
        if raise_on_failure:
            l = int(np.flatnonzero(status)[0])
            raise ChemicalEquilibriumError(f"layer {l}: {_STATUS.get(int(status[l]), status[l])} "
                                           f"(log xi={info[l, 2]}, inf-norm={info[l, 3]})")
    else:
        ctx.check(rc)
    return dens, status, info


def chemical_equilibrium_vjp(T, n_tot, ne_model, abundances, densities, gbar, atm=None, tables=None, ctx=None):
    """Reverse mode of :func:`solve_layers` at its solution ``densities`` (korg_chemical_equilibrium_vjp):
    given ``gbar`` [L, 278 + n_mol], the cotangents of every density in the same layout, returns
    (dL/dT [L], dL/dn_tot [L], dL/dabundances [L, 92]) per layer -- the reference differentiates
    through its solver with ForwardDiff and the implicit-function rule (src/statmech.jl:307-355)."""
    ctx = ctx or _lib.default_context()
    t = ctx.ensure_equilibrium(tables)
    keep = _lib.Keep()
    T = keep.f64(np.atleast_1d(T))
    L = len(T)
    nt = keep.f64(np.broadcast_to(np.asarray(n_tot, np.float64), (L,)))
    ne = keep.f64(np.broadcast_to(np.asarray(ne_model, np.float64), (L,)))
    ab = keep.f64(np.atleast_2d(abundances))
    at = None if atm is None else keep.i32(atm)
    nspec = _lib.KORG_CHEM_MOL0 + len(t.molecules)
    d, g = keep.f64(densities), keep.f64(gbar)
    if d.shape != (L, nspec) or g.shape != (L, nspec):
        raise ValueError(f"densities and gbar must be [{L}, {nspec}]")
    dT, dnt, dab = np.empty(L), np.empty(L), np.empty((L, MAX_ATOMIC_NUMBER))
    y = _lib.ChemLayers(L, _lib._p(T), _lib._p(nt), _lib._p(ne), _lib._p(ab), _lib._p(at, _lib._ip))
    ctx.check(ctx.lib.korg_chemical_equilibrium_vjp(ctx.h, C.byref(y), ab.shape[0], _lib._p(d), _lib._p(g),
                                                    _lib._p(dT), _lib._p(dnt), _lib._p(dab)))
    return dT, dnt, dab


def chemical_equilibrium(T, n_tot, model_atm_ne, absolute_abundances, ionization_energies=None,
                         partition_funcs=None, log_equilibrium_constants=None,
                         electron_number_density_warn_threshold=0.1,
                         electron_number_density_warn_min_value=1e-4, ctx=None):
    """``(n_e, {Species: n})`` as src/statmech.jl:148-206: scalars for one layer, arrays over the
    layers when ``T``, ``n_tot`` and ``model_atm_ne`` are arrays."""
    scalar = np.ndim(T) == 0
    tables = _tables(ionization_energies, partition_funcs, log_equilibrium_constants)
    dens, _, _ = solve_layers(T, n_tot, model_atm_ne, np.asarray(absolute_abundances, np.float64), tables=tables,
                              ctx=ctx)
    ne = dens[:, 0]
    ne_m = np.broadcast_to(np.asarray(model_atm_ne, np.float64), ne.shape)
    nt = np.broadcast_to(np.asarray(n_tot, np.float64), ne.shape)
    off = np.flatnonzero((ne / nt > electron_number_density_warn_min_value) &
                         (np.abs((ne - ne_m) / ne_m) > electron_number_density_warn_threshold))
    if len(off):  # the reference warns per layer; one warning per call names the first layer
        l = int(off[0])
        warnings.warn(f"Electron number density differs from model atmosphere by a factor greater than "
                      f"{electron_number_density_warn_threshold}. (calculated ne = {ne[l]}, model atmosphere "
                      f"ne = {ne_m[l]}{f'; {len(off)} layers' if len(off) > 1 else ''})")
    cols = {s: k for k, s in enumerate(tables.species) if s is not None}  # n(H III) is written as 0
    if scalar:
        return float(ne[0]), {s: float(dens[0, k]) for s, k in cols.items()}
    return ne.copy(), {s: dens[:, k].copy() for s, k in cols.items()}
