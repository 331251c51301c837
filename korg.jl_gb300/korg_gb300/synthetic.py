"""Seeded synthetic workloads for the benchmark configurations.

The reference benchmarks on VALD / APOGEE line lists and MARCS atmospheres, none of which are
available here; these generators stand in for them with the shapes and value distributions the
configurations specify (line centres, log gf, E_lower, broadening parameters, species mixes,
grid ranges and steps, atmosphere parameters).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .linelist import LineList
from .species import parse_species
from . import standin

ATOMIC = ["Fe I", "Fe II", "Ca I", "Ti I", "Ni I"]


def synthetic_linelist(n, wl_lo, wl_hi, seed=0, species=ATOMIC, loggf=(-5.0, 0.0), E_lower=(0.0, 6.0),
                       molecular=False):
    """n lines with centres ~ U(wl_lo, wl_hi) A, log gf ~ U(loggf), E_lower ~ U(E_lower) eV,
    species drawn uniformly from ``species``, log10 gamma_rad ~ U(7, 9); atoms also get
    log10 gamma_stark ~ U(-7, -5) and log10 gamma_vdW ~ U(-8, -7) (stored as (10^v, -1));
    molecules get no Stark or vdW broadening (line_absorption.jl:91-94)."""
    rng = np.random.default_rng(seed)
    wl = np.sort(rng.uniform(wl_lo, wl_hi, n)) * 1e-8
    lg = rng.uniform(*loggf, n)
    El = rng.uniform(*E_lower, n)
    spec = rng.integers(0, len(species), n)
    grad = 10.0 ** rng.uniform(7, 9, n)
    if molecular:
        gstark = np.zeros(n)
        v1 = np.zeros(n)
    else:
        gstark = 10.0 ** rng.uniform(-7, -5, n)
        v1 = 10.0 ** rng.uniform(-8, -7, n)
    v2 = -np.ones(n)
    return LineList(wl, lg, spec.astype(np.int32), [parse_species(s) for s in species], El, grad, gstark, v1, v2)


@dataclass
class Workload:
    name: str
    Teff: float
    logg: float
    m_H: float
    L: int
    wavelengths: tuple
    linelist: LineList
    hydrogen_lines: bool = True
    vmic: float = 1.0


def config0(seed=0, n_lines=2000):
    """Plain FP64 parity case: 56 layers, Teff 5000, logg 4.4, 2,000 atomic lines in
    5000-5100 A, 10,001-point grid at 0.01 A, vmic 1 km/s."""
    ll = synthetic_linelist(n_lines, 5000.0, 5100.0, seed=seed)
    return Workload("cfg0: 56 layers, 2k lines, 5000-5100 A @ 0.01 A", 5000.0, 4.4, 0.0, 56, (5000, 5100), ll)


def config1(seed=0, n_lines=300_000, wl=(3000, 10000)):
    """Mixed-precision full optical: 56 layers, Teff 5800, logg 4.4, [M/H] 0, 300,000 atomic
    lines over 3000-10000 A plus hydrogen lines, 700,001-point grid at 0.01 A."""
    ll = synthetic_linelist(n_lines, float(wl[0]), float(wl[1]), seed=seed)
    return Workload(f"cfg1: 56 layers, {n_lines // 1000}k lines + H, {wl[0]}-{wl[1]} A @ 0.01 A", 5800.0, 4.4, 0.0,
                    56, wl, ll)


def config2(seed=0, n_atomic=50_000, n_mol=20_000):
    """72 layers, Teff 4500, logg 2.5, [M/H] -0.5; 50k atomic + 20k CO/OH/CN lines over
    15000-17000 A on a 0.005 A grid (400,001 points)."""
    a = synthetic_linelist(n_atomic, 15000.0, 17000.0, seed=seed)
    m = synthetic_linelist(n_mol, 15000.0, 17000.0, seed=seed + 1, species=["CO", "OH", "CN"],
                           loggf=(-8.0, -2.0), E_lower=(0.0, 3.0), molecular=True)
    ll = a.concat(m).sorted()
    return Workload("cfg2: 72 layers, 70k lines, 15000-17000 A @ 0.005 A", 4500.0, 2.5, -0.5, 72,
                    (15000, 17000, 0.005), ll)


def config3(seed=0, n_spectra=256, n_list=500_000, n_min=20_000, n_max=200_000, L=56,
            wavelengths=(15000, 17000, 0.005)):
    """Batched persistent launch: n_spectra atmospheres with Teff ~ U(3500, 7000) K,
    logg ~ U(1, 5), [M/H] ~ U(-2.5, 0.5), each with its own pruned subset of n ~ U(n_min, n_max)
    lines of one n_list-line atomic + molecular list (5:2) over the wavelength range
    (15000-17000 A on the 0.005 A grid by default).

    Each spectrum keeps a seeded random subset of n lines.  (A strength cut such as
    prune_linelist's keeps a subset whose size varies per atmosphere; keeping the n strongest
    of this synthetic list, whose log gf are uniform up to 0, would give cool dwarfs windows
    spanning most of the grid for every line, which pruned real line lists do not have.)"""
    rng = np.random.default_rng(seed)
    na = n_list * 5 // 7
    lo, hi = float(wavelengths[0]), float(wavelengths[1])
    a = synthetic_linelist(na, lo, hi, seed=seed)
    m = synthetic_linelist(n_list - na, lo, hi, seed=seed + 1, species=["CO", "OH", "CN"],
                           loggf=(-8.0, -2.0), E_lower=(0.0, 3.0), molecular=True)
    master = a.concat(m).sorted()
    out = []
    for k in range(n_spectra):
        Teff = float(rng.uniform(3500, 7000))
        logg = float(rng.uniform(1, 5))
        m_H = float(rng.uniform(-2.5, 0.5))
        n = int(rng.integers(n_min, n_max + 1))
        keep = np.sort(rng.choice(len(master), size=min(n, len(master)), replace=False))
        out.append(Workload(f"cfg3[{k}]: Teff {Teff:.0f} logg {logg:.2f} [M/H] {m_H:+.2f}, {n} lines", Teff, logg,
                            m_H, L, wavelengths, master.subset(keep)))
    return out


def config4(seed=0, n_lines=1_000_000):
    """80 layers, Teff 3500, logg 1.0; 1M lines (40% atomic, 60% TiO/CO/OH/CN) over 3000-10000 A
    on a 0.01 A grid."""
    na = int(0.4 * n_lines)
    a = synthetic_linelist(na, 3000.0, 10000.0, seed=seed)
    m = synthetic_linelist(n_lines - na, 3000.0, 10000.0, seed=seed + 1, species=["TiO", "CO", "OH", "CN"],
                           loggf=(-9.0, -1.0), E_lower=(0.0, 4.0), molecular=True)
    ll = a.concat(m).sorted()
    return Workload("cfg4: 80 layers, 1M lines, 3000-10000 A @ 0.01 A", 3500.0, 1.0, 0.0, 80, (3000, 10000), ll)


def abundance_variants(inp, n_variants=16, seed=0, spread=0.3):
    """n_variants copies of prepared inputs whose metal number densities are scaled by
    10^U(-spread, spread) dex per species (the batch of abundance variants of one atmosphere).
    Only the line-strength rows n/U change; the atmosphere, continuum and H lines are shared."""
    import copy
    from .species import parse_species
    rng = np.random.default_rng(seed)
    H = {parse_species("H I"), parse_species("H II"), parse_species("He I"), parse_species("He II"),
         parse_species("H2")}
    out = []
    for v in range(n_variants):
        c = copy.copy(inp)
        scale = np.array([1.0 if s in H else 10.0 ** rng.uniform(-spread, spread) for s in inp.linelist.species])
        c.n_div_U = np.ascontiguousarray(inp.n_div_U * scale[:, None])
        out.append(c)
    return out


def prepare(work: Workload, **kwargs):
    """Synthetic atmosphere + host precompute for a workload (keyword arguments go to
    prepare_synthesis, e.g. continuum="gpu")."""
    from .api import prepare_synthesis
    atm, A_X = standin.synthetic_atmosphere(work.Teff, work.logg, work.m_H, work.L)
    return prepare_synthesis(atm, work.linelist, A_X, work.wavelengths, vmic=work.vmic,
                             hydrogen_lines=work.hydrogen_lines, **kwargs)
