"""FP64 restatement of Korg's continuum absorption (src/ContinuumAbsorption/), numpy.

TEST INFRASTRUCTURE ONLY: the checker of the device continuum kernel (tests/) -- the product
never imports it.  Each function restates the cited reference function; tables are the
reference's own, converted unchanged into korg_gb300/data/continuum_tables.npz.  Frequencies in
Hz, temperatures in K, number densities in cm^-3, results in cm^-1.

Every term follows the reference's bounds handling with error_oobounds=false: outside a term's
frequency or temperature range the term contributes nothing (bounds_checking.jl:47-73).
Metal bound-free absorption (absorption_metals_bf.jl) needs data/bf_cross-sections/
bf_cross-sections.h5, which is missing from the reference checkout: it is not restated.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = os.path.join(HERE, "..", "korg.jl_gb300", "korg_gb300", "data", "continuum_tables.npz")

# src/constants.jl
kboltz_cgs, hplanck_cgs, c_cgs = 1.380649e-16, 6.62607015e-27, 2.99792458e10
electron_mass_cgs, electron_charge_cgs = 9.1093897e-28, 4.80320425e-10
bohr_radius_cgs, eV_to_cgs = 5.29177210903e-9, 1.602e-12
kboltz_eV, hplanck_eV = 8.617333262145e-5, 4.135667696e-15
RydbergH_eV, Rydberg_eV = 13.598287264, 13.605693122994
chi_H = 13.5984  # ionization_energies[1][1] (Barklem & Collet 2016)

_T = None


def tables():
    global _T
    if _T is None:
        with np.load(TABLES) as f:
            _T = {k: f[k] for k in f.files}
    return _T


def _lerp(x, xs, ys):
    """Linear interpolation with linear extrapolation (Interpolations.jl Line())."""
    x = np.asarray(x, np.float64)
    i = np.clip(np.searchsorted(xs, x, side="right") - 1, 0, len(xs) - 2)
    t = (x - xs[i]) / (xs[i + 1] - xs[i])
    return ys[i] * (1 - t) + ys[i + 1] * t


def _bilerp(x, y, xs, ys, Z):
    """Bilinear interpolation on a grid (Interpolations.jl Gridded(Linear()); callers keep (x, y)
    inside the grid or rely on linear extrapolation)."""
    x, y = np.broadcast_arrays(np.asarray(x, np.float64), np.asarray(y, np.float64))
    i = np.clip(np.searchsorted(xs, x, side="right") - 1, 0, len(xs) - 2)
    j = np.clip(np.searchsorted(ys, y, side="right") - 1, 0, len(ys) - 2)
    tx = (x - xs[i]) / (xs[i + 1] - xs[i])
    ty = (y - ys[j]) / (ys[j + 1] - ys[j])
    return (Z[i, j] * (1 - tx) * (1 - ty) + Z[i + 1, j] * tx * (1 - ty) + Z[i, j + 1] * (1 - tx) * ty +
            Z[i + 1, j + 1] * tx * ty)


def _in(x, lo, hi):
    return (x >= lo) & (x <= hi)


def hummer_mihalas_w(n_eff, nH, nHe, ne):
    """src/statmech.jl:463-497, default branch."""
    n_eff = np.asarray(n_eff, np.float64)
    r_level = np.sqrt(5 / 2 * n_eff ** 4 + 1 / 2 * n_eff ** 2) * bohr_radius_cgs
    neutral = nH * (r_level + np.sqrt(3) * bohr_radius_cgs) ** 3 + nHe * (r_level + 1.02 * bohr_radius_cgs) ** 3
    K = np.where(n_eff > 3, 16 / 3 * (n_eff / (n_eff + 1)) ** 2 * ((n_eff + 7 / 6) / (n_eff ** 2 + n_eff + 1 / 2)), 1.0)
    chi = RydbergH_eV / n_eff ** 2 * eV_to_cgs
    charged = 16 * ((electron_charge_cgs ** 2) / (chi * np.sqrt(K))) ** 3 * ne
    return np.exp(-4 * np.pi / 3 * (neutral + charged))


def H_I_bf(nu, T, nH_I, nHe_I, ne, invU_H, n_max_MHD=6):
    """absorption_H.jl:54-125 (H_I_bf) with simple_hydrogen_bf_cross_section (:139-163)."""
    t = tables()
    nu = np.asarray(nu, np.float64)
    total = np.zeros_like(nu)
    for n in range(1, n_max_MHD + 1):
        Es, sig = t["H_bf_E"][n - 1], t["H_bf_sigma"][n - 1]
        w_lower = hummer_mihalas_w(n, nH_I, nHe_I, ne)
        occ = w_lower * np.exp(-chi_H * (1 - 1 / n ** 2) / (kboltz_eV * T))
        nu_break = chi_H / (n ** 2 * hplanck_eV)
        above = nu > nu_break
        if n == 1:
            frac = np.where(above, 1.0, 0.0)
        else:
            with np.errstate(invalid="ignore", divide="ignore"):
                n_eff = 1 / np.sqrt(1 / n ** 2 - hplanck_eV * nu / chi_H)
                frac = np.where(above, 1.0, 1 - hummer_mihalas_w(n_eff, nH_I, nHe_I, ne) / w_lower)
        sigma_break = _lerp(nu_break * hplanck_eV, Es, sig)
        scaling = sigma_break / nu_break ** -3
        with np.errstate(invalid="ignore"):
            cs = np.where(above, _lerp(hplanck_eV * nu, Es, sig), nu ** -3 * scaling)
        total += occ * cs * frac
    for n in range(n_max_MHD + 1, 41):
        w_lower = hummer_mihalas_w(n, nH_I, nHe_I, ne)
        if w_lower < 1e-5:
            break
        occ = 2 * n ** 2 * w_lower * np.exp(-chi_H * (1 - 1 / n ** 2) / (kboltz_eV * T))
        simple = np.where(hplanck_eV * nu < RydbergH_eV / n ** 2, 0.0,
                          2.815e29 * (1.0 / n) ** 5 * (1.0 / nu) ** 3 * 1e18)
        total += occ * simple
    return nH_I * invU_H * total * (1.0 - np.exp(-hplanck_eV * nu / (kboltz_eV * T))) * 1e-18


H_MINUS_ION_EV = 0.754204  # absorption_H.jl:6


def Hminus_bf_cross_section(nu):
    """absorption_H.jl:170-195 (_Hminus_bf_cross_section), cm^2."""
    t = tables()
    nus, sig = t["Hminus_bf_nu"], t["Hminus_bf_sigma"]
    nu = np.asarray(nu, np.float64)
    nu_ion = H_MINUS_ION_EV / hplanck_eV
    nu_min = nus[0]
    coef = np.interp(nu_min, nus, sig) / (nu_min - nu_ion) ** 1.5
    with np.errstate(invalid="ignore"):
        low = coef * (nu - nu_ion) ** 1.5
    return np.where(nu <= nu_ion, 0.0, np.where(nu < nu_min, low, np.interp(nu, nus, sig)))


def Hminus_bf(nu, T, n_Hminus):
    """absorption_H.jl:197-228: n(H-) sigma (1 - exp(-h nu / k T)) for nu <= 2.418e19 Hz, T > 0."""
    nu = np.asarray(nu, np.float64)
    a = n_Hminus * Hminus_bf_cross_section(nu) * (1 - np.exp(-hplanck_cgs * nu / (kboltz_cgs * T)))
    return np.where(_in(nu, 0.0, 2.417989242625068e19) & (T > 0), a, 0.0)


def Hminus_ff(nu, T, nH_I_div_U, ne):
    """absorption_H.jl:261-325: Bell & Berrington K(lambda, theta) Pe n(H I, n=1), for
    1823 A <= lambda <= 151890 A and 1400 K <= T <= 10080 K."""
    t = tables()
    nu = np.asarray(nu, np.float64)
    lam = c_cgs * 1e8 / nu
    theta = 5040.0 / T
    ok = _in(nu, c_cgs / 151890e-8, c_cgs / 1823e-8) & _in(T, 1400, 10080)
    K = 1e-26 * _bilerp(np.where(ok, lam, 5000.0), theta if ok.any() else 1.0, t["Hminus_ff_lambda"],
                        t["Hminus_ff_theta"], t["Hminus_ff_K"])
    Pe = ne * kboltz_cgs * T
    return np.where(ok, K * Pe * 2 * nH_I_div_U, 0.0)


def H2plus_bf_and_ff(nu, T, nH_I, nH_II):
    """absorption_H.jl:327-380 with Stancil1994.jl: (sigma_bf / K + sigma_ff) n(H I) n(H II)
    (1 - exp(-h nu / k T)), for 700 A <= lambda <= 200000 A and 3150 K <= T <= 25200 K."""
    t = tables()
    nu = np.asarray(nu, np.float64)
    ok = _in(nu, c_cgs / 2e-3, c_cgs / 7e-6) & _in(T, 3150, 25200)
    lam = np.where(ok, c_cgs * 1e8 / nu, 5000.0)
    Tc = T if _in(T, 3150, 25200) else 5000.0
    K = _lerp(Tc, t["H2plus_T"], t["H2plus_K"])
    sbf = _bilerp(lam, Tc, t["H2plus_bf_lambda"], t["H2plus_T"], t["H2plus_bf_sigma"] * 1e-18)
    sff = _bilerp(lam, Tc, t["H2plus_ff_lambda"], t["H2plus_T"], t["H2plus_ff_sigma"] * 1e-39)
    stim = 1 - np.exp(-hplanck_eV * nu / (kboltz_eV * T))
    return np.where(ok, (sbf / K + sff) * nH_I * nH_II * stim, 0.0)


def Heminus_ff(nu, T, nHe_I_div_U, ne):
    """absorption_He.jl:9-95: John (1994) K(lambda, theta) Pe n(He I, n=1), for
    5063 A <= lambda <= 151878 A and 1400 K <= T <= 10080 K."""
    t = tables()
    nu = np.asarray(nu, np.float64)
    ok = _in(nu, c_cgs / 1.518780e-3, c_cgs / 5.063e-5) & _in(T, 1400, 10080)
    lam = np.where(ok, c_cgs * 1e8 / nu, 10000.0)
    theta = 5040.0 / T if _in(T, 1400, 10080) else 1.0
    K = 1e-26 * _bilerp(lam, theta, t["Heminus_ff_lambda"], t["Heminus_ff_theta"], t["Heminus_ff_K"])
    Pe = ne * kboltz_cgs * T
    return np.where(ok, K * nHe_I_div_U * Pe, 0.0)  # n(He I, n=1) = g_1 exp(0) n/U, g_1 = 1


def gaunt_ff(log_u, log_g2):
    """hydrogenic_bf_ff.jl:82-114: the van Hoof et al. (2014) table, bilinear."""
    t = tables()
    return _bilerp(log_u, log_g2, t["gaunt_log_u"], t["gaunt_log_g2"], t["gaunt_ff"])


def hydrogenic_ff(nu, T, Z, ni, ne):
    """hydrogenic_bf_ff.jl:116-176 (hydrogenic_ff_absorption)."""
    nu = np.asarray(nu, np.float64)
    inv_T = 1.0 / T
    Z2 = Z * Z
    hnu_kT = (hplanck_eV / kboltz_eV) * nu * inv_T
    g = gaunt_ff(np.log10(hnu_kT), np.log10((Rydberg_eV / kboltz_eV) * Z2 * inv_T))
    F = 3.6919e8 * g * Z2 * np.sqrt(inv_T) / (nu * nu * nu)
    return ni * ne * F * (1 - np.exp(-hnu_kT))


PEACH_SPECIES = ("HeII", "CII", "SiII", "MgII")  # Peach1970.jl: the ion taking part, with its charge 1


def peach_departure(tag, T, sigma):
    """Peach1970.jl: bilinear in (T, sigma), zero outside the table (extrapolation_bc=0)."""
    t = tables()
    Ts, ss, D = t[f"peach_{tag}_T"], t[f"peach_{tag}_sigma"], t[f"peach_{tag}_D"]
    sigma = np.asarray(sigma, np.float64)
    inside = _in(T, Ts[0], Ts[-1]) & _in(sigma, ss[0], ss[-1])
    return np.where(inside, _bilerp(np.clip(T, Ts[0], Ts[-1]), np.clip(sigma, ss[0], ss[-1]), Ts, ss, D), 0.0)


def positive_ion_ff(nu, T, ne, n_Z1, n_Z2, n_peach):
    """absorption_ff_positive_ion.jl:44-84: hydrogenic free-free of every positive ion, with
    Peach (1970) departure coefficients for the ions in n_peach (dict tag -> density, charge 1);
    n_Z1 / n_Z2 are the summed densities of the other singly / doubly charged species.  Only for
    100 K <= T <= 1e6 K and 1e-6 cm < lambda < 1e-2 cm."""
    nu = np.asarray(nu, np.float64)
    out = np.zeros_like(nu)
    if not (100.0 <= T <= 1e6):
        return out
    idx = (c_cgs / 1e-2 < nu) & (nu < c_cgs / 1e-6)
    v = nu[idx]
    acc = np.zeros_like(v)
    for tag in PEACH_SPECIES:
        n = n_peach.get(tag, 0.0)
        sig = v / 1 ** 2 * (hplanck_eV / Rydberg_eV)
        acc += hydrogenic_ff(v, T, 1, n, ne) * (1 + peach_departure(tag, T, sig))
    acc += hydrogenic_ff(v, T, 1, n_Z1, ne)
    acc += hydrogenic_ff(v, T, 2, n_Z2, ne)
    out[idx] = acc
    return out


def electron_scattering(ne):
    """scattering.jl:48-56."""
    return 8 * np.pi / 3 * (electron_charge_cgs ** 2 / (electron_mass_cgs * c_cgs ** 2)) ** 2 * ne


def rayleigh(nu, nH_I, nHe_I, nH2):
    """scattering.jl:1-46 (Colgan+ 2016 for H and He, Dalgarno & Williams 1962 for H2)."""
    nu = np.asarray(nu, np.float64)
    sth = 6.65246e-25
    E2 = (hplanck_eV * nu / (2 * Rydberg_eV)) ** 2
    E4, E6, E8 = E2 ** 2, E2 * E2 ** 2, E2 ** 4
    sH = 20.24 * E4 + 239.2 * E6 + 2256 * E8
    sHe = 1.913 * E4 + 4.52 * E6 + 7.90 * E8
    i2 = (nu / (1e8 * c_cgs)) ** 2
    i4, i6, i8 = i2 ** 2, i2 * i2 ** 2, i2 ** 4
    return (nH_I * sH + nHe_I * sHe) * sth + (8.14e-13 * i4 + 1.28e-6 * i6 + 1.61 * i8) * nH2


def Hminus_nK(T):
    """src/statmech.jl:75-79: n(H-) = nK(T) n(H I) ne."""
    transU = (2 * np.pi * electron_mass_cgs * kboltz_cgs * T / hplanck_cgs ** 2) ** 1.5
    return np.exp(H_MINUS_ION_EV / (kboltz_eV * T)) / (4 * transU)


def total_continuum_absorption(nu, T, ne, d):
    """ContinuumAbsorption.jl:39-74 without metal bound-free absorption.  d: the per-layer
    quantities of korg_continuum_layers for one layer (nH_I, nH_II, nHe_I, nH2, nH_minus, invU_H_I,
    invU_He_I, n_Z1, n_Z2, n_HeII, n_CII, n_SiII, n_MgII)."""
    a = H_I_bf(nu, T, d["nH_I"], d["nHe_I"], ne, d["invU_H_I"])
    a += Hminus_bf(nu, T, d["nH_minus"])
    a += Hminus_ff(nu, T, d["nH_I"] * d["invU_H_I"], ne)
    a += H2plus_bf_and_ff(nu, T, d["nH_I"], d["nH_II"])
    a += Heminus_ff(nu, T, d["nHe_I"] * d["invU_He_I"], ne)
    a += positive_ion_ff(nu, T, ne, d["n_Z1"], d["n_Z2"],
                         {"HeII": d["n_HeII"], "CII": d["n_CII"], "SiII": d["n_SiII"], "MgII": d["n_MgII"]})
    a += electron_scattering(ne)
    a += rayleigh(nu, d["nH_I"], d["nHe_I"], d["nH2"])
    return a
