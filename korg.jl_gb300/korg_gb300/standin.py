"""Host-side stand-ins for the physics that stays off the GPU hot path.

Korg computes the model atmosphere (MARCS interpolation), chemical equilibrium and continuum
opacity on the host (src/atmosphere.jl, src/statmech.jl:148-286,
src/ContinuumAbsorption/ContinuumAbsorption.jl:39-74) and feeds the results to the line,
hydrogen-line and transfer code.  Those host steps are outside this package's scope.  To drive
the hot path with realistic inputs anyway, this module provides compact, physically reasonable
replacements:

* :func:`synthetic_atmosphere`: a grey Eddington T(tau) on log tau_5000 in [-5, 2] in
  hydrostatic equilibrium with the stand-in 5000 A opacity;
* :func:`chemical_equilibrium`: Saha ionisation (I/II/III) for all elements with Korg's
  partition functions and Barklem & Collet ionisation energies, plus dissociation equilibrium
  of the common diatomics from dissociation energies;
* :func:`continuum_opacity`: H- bound-free (John 1988 fit) and free-free (Bell & Berrington
  fit as tabulated by Gray), hydrogenic H I bound-free/free-free (Kramers), Thomson and H I
  Rayleigh scattering.

These are *inputs* of the hot path; the GPU kernels and the oracle consume the same numbers,
so kernel parity does not depend on how close these are to Korg's own host physics.
"""
from __future__ import annotations

import math

import numpy as np

from .constants import (amu_cgs, c_cgs, electron_mass_cgs, hplanck_cgs, kboltz_cgs, kboltz_eV)
from .data import default_partition_funcs, ionization_energies
from .species import Species, atomic_masses, parse_species

# Solar abundances A(X) = log(X/H) + 12, Asplund et al. 2021 (A&A 653, A141).
solar_A_X = np.array([
    12.00, 10.91, 0.96, 1.38, 2.70, 8.46, 7.83, 8.69, 4.40, 8.06, 6.22, 7.55, 6.43, 7.51, 5.41,
    7.12, 5.31, 6.38, 5.07, 6.30, 3.14, 4.97, 3.90, 5.62, 5.42, 7.46, 4.94, 6.20, 4.18, 4.56,
    3.02, 3.62, 2.30, 3.34, 2.54, 3.12, 2.32, 2.83, 2.21, 2.59, 1.47, 1.88, -5.00, 1.75, 0.78,
    1.57, 0.96, 1.71, 0.80, 2.02, 1.01, 2.18, 1.55, 2.22, 1.08, 2.27, 1.11, 1.58, 0.75, 1.42,
    -5.00, 0.95, 0.52, 1.08, 0.31, 1.10, 0.48, 0.93, 0.11, 0.85, 0.10, 0.85, -0.15, 0.79, 0.26,
    1.35, 1.32, 1.61, 0.91, 1.17, 0.92, 1.95, 0.65, -5.00, -5.00, -5.00, -5.00, -5.00, -5.00,
    0.03, -5.00, -0.54])


def format_A_X(m_H=0.0):
    """A(X) with every metal (Z >= 3) scaled by [M/H] (src/abundances.jl:45-123, no alpha
    enhancement)."""
    A = solar_A_X.copy()
    A[2:] += m_H
    return A


# Diatomics: (name, dissociation energy D0 in eV), standard spectroscopic values.
DIATOMICS = [("H2", 4.478), ("CO", 11.092), ("OH", 4.392), ("CN", 7.72), ("OTi", 6.87),
             ("OZr", 7.85), ("OV", 6.44), ("HMg", 1.34), ("HSi", 3.06), ("C2", 6.21),
             ("N2", 9.759), ("NO", 6.497), ("CH", 3.465), ("HN", 3.42), ("O2", 5.116)]


def _transU(m, T):
    return (2 * math.pi * m * kboltz_cgs * T / hplanck_cgs ** 2) ** 1.5


def chemical_equilibrium(T, n_tot, A_X, n_iter=200):
    """Stand-in chemical equilibrium for arrays of layer temperatures and total particle
    densities.  Returns (n_e, {Species: array of number densities}).

    Saha ionisation (neutral, singly and doubly ionised) of every element with ionisation
    energies, plus the diatomic dissociation equilibria of DIATOMICS, solved by fixed-point
    iteration on n_e (outer) and the neutral atom densities (inner), all elements and layers
    at once."""
    T = np.asarray(T, dtype=np.float64)
    n_tot = np.asarray(n_tot, dtype=np.float64)
    pf = default_partition_funcs()
    chi = ionization_energies()
    lnT = np.log(T)
    Zs = [z for z in range(1, 93) if z in chi]
    zi = {z: k for k, z in enumerate(Zs)}
    abund = 10.0 ** (np.asarray(A_X) - 12)
    abund = abund / abund.sum()

    def U(z, q):
        s = Species([z], q)
        return pf[s](np.clip(lnT, pf[s].t[0], pf[s].t[-1])) if s in pf else np.ones_like(T)

    U0 = np.array([U(z, 0) for z in Zs])
    U1 = np.array([U(z, 1) for z in Zs])
    U2 = np.array([U(z, 2) for z in Zs])
    chi1 = np.array([chi[z][0] for z in Zs])[:, None]
    chi2 = np.array([chi[z][1] for z in Zs])[:, None]
    third = np.array([z != 1 and chi[z][1] >= 0 for z in Zs])[:, None]
    A = np.array([abund[z - 1] for z in Zs])[:, None]
    tU = _transU(electron_mass_cgs, T)
    kT = kboltz_eV * T
    mols, ia, ib, Ks = [], [], [], []
    for name, D0 in DIATOMICS:
        sp = parse_species(name)
        a, b = sp.atoms
        mu = atomic_masses[a - 1] * atomic_masses[b - 1] / (atomic_masses[a - 1] + atomic_masses[b - 1])
        Umol = pf[sp](lnT) if sp in pf else np.ones_like(T)
        K = _transU(mu, T) * U0[zi[a]] * U0[zi[b]] / Umol * np.exp(-D0 / kT)  # n_a n_b / n_ab
        mols.append(sp)
        ia.append(zi[a])
        ib.append(zi[b])
        Ks.append(K)
    ia, ib, Ks = np.array(ia), np.array(ib), np.array(Ks)
    homo = ia == ib
    saha1 = (U1 / U0) * tU * np.exp(-chi1 / kT)
    saha2 = np.where(third, (U2 / np.where(third, U1, 1.0)) * tU * np.exp(-np.where(third, chi2, 0.0) / kT), 0.0)
    ne = 1e-4 * n_tot * np.clip(T / 5000.0, 0.5, 3) ** 4
    for it in range(n_iter):
        wII = 2.0 / ne * saha1
        wIII = wII * 2.0 / ne * saha2
        N = A * (n_tot - ne)
        base = 1 + wII + wIII
        n0 = N / base
        for _ in range(30):
            denom = base.copy()
            np.add.at(denom, ia[homo], 2 * n0[ia[homo]] / Ks[homo])
            np.add.at(denom, ia[~homo], n0[ib[~homo]] / Ks[~homo])
            np.add.at(denom, ib[~homo], n0[ia[~homo]] / Ks[~homo])
            n0 = np.sqrt(n0 * (N / denom))
        ne_new = np.maximum(np.sum(n0 * (wII + 2 * wIII), axis=0), 1e-10 * n_tot)
        if np.max(np.abs(ne_new / ne - 1)) < 1e-10:
            ne = ne_new
            break
        ne = np.sqrt(ne * ne_new)
    nd = {}
    for z in Zs:
        k = zi[z]
        nd[Species([z], 0)] = n0[k]
        nd[Species([z], 1)] = n0[k] * wII[k]
        nd[Species([z], 2)] = n0[k] * wIII[k]
    for sp, a, b, K in zip(mols, ia, ib, Ks):
        nd[sp] = n0[a] * n0[b] / K
    return ne, nd


# John (1988) H- bound-free fit coefficients, lambda in micron
_HM_BF_C = [152.519, 49.534, -118.858, 92.536, -34.194, 4.982]


def _hminus_bf_sigma(wl_um):
    lam0 = 1.6419
    x = np.clip(1.0 / wl_um - 1.0 / lam0, 0.0, None)
    f = sum(c * x ** (n / 2.0) for n, c in enumerate(_HM_BF_C))
    return np.where(wl_um < lam0, 1e-18 * wl_um ** 3 * x ** 1.5 * f, 0.0)


def _hminus_ff_k(wl_A, T):
    """Bell & Berrington (1987) fit (Gray eq. 8.13): cm^2 per H atom per dyn cm^-2 of P_e."""
    lg = np.log10(wl_A)
    f0 = -2.2763 - 1.6850 * lg + 0.76661 * lg ** 2 - 0.053346 * lg ** 3
    f1 = 15.2827 - 9.2846 * lg + 1.99381 * lg ** 2 - 0.142631 * lg ** 3
    f2 = -197.789 + 190.266 * lg - 67.9775 * lg ** 2 + 10.6913 * lg ** 3 - 0.625151 * lg ** 4
    lt = np.log10(5040.0 / T)
    return 10.0 ** (-26 + f0 + f1 * lt + f2 * lt ** 2)


def continuum_opacity(wls_cm, T, ne, n_HI, n_HII):
    """Stand-in continuum alpha (cm^-1) at wavelengths wls_cm for one layer."""
    wl = np.asarray(wls_cm, dtype=np.float64)
    nu = c_cgs / wl
    stim = 1 - np.exp(-hplanck_cgs * nu / (kboltz_cgs * T))
    # H- bound-free
    n_hm = n_HI * ne * np.exp(0.754195 / (kboltz_eV * T)) / (4 * _transU(electron_mass_cgs, T))
    a = n_hm * _hminus_bf_sigma(wl * 1e4) * stim
    # H- free-free
    a = a + _hminus_ff_k(wl * 1e8, T) * ne * kboltz_cgs * T * n_HI
    # H I bound-free, levels 1..8 (Kramers, Gaunt factor 1)
    U = 2.0
    for n in range(1, 9):
        chi_n = 13.598 * (1 - 1.0 / n ** 2)
        pop = n_HI * 2 * n * n * np.exp(-chi_n / (kboltz_eV * T)) / U
        edge = 911.75e-8 * n * n
        sig = np.where(wl <= edge, 2.815e29 / (n ** 5 * nu ** 3), 0.0)
        a = a + pop * sig * stim
    # H I free-free (Kramers)
    a = a + 3.7e8 / (np.sqrt(T) * nu ** 3) * ne * n_HII * stim
    # Thomson and Rayleigh (H I, Dalgarno)
    wA = wl * 1e8
    a = a + 6.652e-25 * ne + n_HI * (5.799e-13 / wA ** 4 + 1.422e-6 / wA ** 6 + 2.784 / wA ** 8)
    return a


def _layer_opacity_5000(T, ne, nd):
    H1, H2 = Species([1], 0), Species([1], 1)
    return np.array([continuum_opacity(np.array([5e-5]), T[l], ne[l], nd[H1][l], nd[H2][l])[0]
                     for l in range(len(T))])


class PlanarAtmosphere:
    """Plane-parallel model atmosphere (src/atmosphere.jl:36): per-layer tau_5000, z (cm), T,
    electron and total number densities, reference wavelength 5000 A."""

    def __init__(self, tau_ref, z, T, ne, n_tot, reference_wavelength=5e-5):
        self.tau_ref = np.asarray(tau_ref, np.float64)
        self.z = np.asarray(z, np.float64)
        self.T = np.asarray(T, np.float64)
        self.ne = np.asarray(ne, np.float64)
        self.n_tot = np.asarray(n_tot, np.float64)
        self.reference_wavelength = reference_wavelength

    def __len__(self):
        return len(self.T)


def synthetic_atmosphere(Teff, logg, m_H=0.0, L=56, n_hydro_iter=4):
    """Grey Eddington atmosphere on log tau_5000 uniform in [-5, 2] in hydrostatic equilibrium
    with the stand-in continuum at 5000 A: dP/dtau = g / kappa_5000."""
    A_X = format_A_X(m_H)
    logtau = np.linspace(-5, 2, L)
    tau = 10.0 ** logtau
    T = (0.75 * Teff ** 4 * (tau + 2.0 / 3.0)) ** 0.25
    g = 10.0 ** logg
    abund = 10.0 ** (A_X - 12)
    mu_amu = (abund * np.array([m / amu_cgs for m in atomic_masses])).sum() / abund.sum()
    # initial guess: P = g tau / kappa with kappa ~ 1 cm^2/g scaled
    P = g * tau / 0.5
    for _ in range(n_hydro_iter):
        n_tot = P / (kboltz_cgs * T)
        ne, nd = chemical_equilibrium(T, n_tot, A_X, n_iter=60)
        rho = (n_tot - ne) * mu_amu * amu_cgs
        kappa = _layer_opacity_5000(T, ne, nd) / rho
        # integrate dP/dlog tau = ln10 tau g / kappa (trapezoid, starting at the top)
        f = np.log(10.0) * tau * g / kappa
        Pn = np.empty(L)
        Pn[0] = g * tau[0] / kappa[0]
        for i in range(1, L):
            Pn[i] = Pn[i - 1] + 0.5 * (f[i] + f[i - 1]) * (logtau[i] - logtau[i - 1])
        P = Pn
    n_tot = P / (kboltz_cgs * T)
    ne, nd = chemical_equilibrium(T, n_tot, A_X)
    alpha5 = _layer_opacity_5000(T, ne, nd)
    # height: dz = -dtau / alpha_5000, z = 0 at tau_5000 = 1
    z = np.zeros(L)
    for i in range(1, L):
        z[i] = z[i - 1] - (tau[i] - tau[i - 1]) / (0.5 * (alpha5[i] + alpha5[i - 1]))
    z -= np.interp(0.0, logtau, z)
    return PlanarAtmosphere(tau, z, T, ne, n_tot), A_X
