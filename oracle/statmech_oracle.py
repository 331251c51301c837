"""FP64 restatement of Korg's chemical equilibrium (src/statmech.jl, src/newton.jl), numpy.

TEST INFRASTRUCTURE ONLY: the checker of the device chemical-equilibrium solver (tests/) and the
CPU leg of the benchmark -- the product never imports it.  Every function restates the cited
reference function with the same arguments: temperatures in K, number densities in cm^-3,
``ionization_energies`` as {Z: [chi1, chi2, chi3]} (eV), ``partition_funcs`` as
{Species: U(ln T)} and ``log_equilibrium_constants`` as {Species: log10 K(ln T)} in partial
pressure form (the package's data loaders give the reference's tables in that form).

The solver is the reference's: 93 unknowns (log10 n of the 92 neutral atoms and log10 n_e),
residuals scaled by the element abundance times n_tot, a Newton iteration whose step is clipped
to at most 1 dex in any unknown, and a continuation on log xi (the log10 scale of every molecule
and H- density) when the plain solve does not converge.  Like ForwardDiff.jacobian in the
reference, the Jacobian is the exact derivative of the residual expression: here each quantity
carries its tangent (the forward-mode chain rule, written out over the molecule incidence matrix).
Linear solves use LAPACK's LU with partial pivoting, as Julia's ``J \\ F`` does.
"""
from __future__ import annotations

import warnings

import numpy as np

# src/constants.jl
kboltz_cgs, hplanck_cgs = 1.380649e-16, 6.62607015e-27
electron_mass_cgs, kboltz_eV = 9.1093897e-28, 8.617333262145e-5
MAX_ATOMIC_NUMBER = 92
LN10 = np.log(10.0)


class ChemicalEquilibriumError(Exception):
    """statmech.jl:81-86."""


def translational_U(m, T):
    """statmech.jl:47-51."""
    return (2 * np.pi * m * kboltz_cgs * T / hplanck_cgs ** 2) ** 1.5


def saha_ion_weights(T, ne, Z, ionization_energies, partition_funcs):
    """(wII, wIII) = n(X II)/n(X I), n(X III)/n(X I) (statmech.jl:19-35)."""
    from_species = _species_ctor(partition_funcs)
    chiI, chiII, _ = ionization_energies[Z]
    UI = partition_funcs[from_species(Z, 0)](np.log(T))
    UII = partition_funcs[from_species(Z, 1)](np.log(T))
    k = kboltz_eV
    transU = translational_U(electron_mass_cgs, T)
    wII = 2.0 / ne * (UII / UI) * transU * np.exp(-chiI / (k * T))
    if Z == 1:
        wIII = 0.0
    else:
        UIII = partition_funcs[from_species(Z, 2)](np.log(T))
        wIII = wII * 2.0 / ne * (UIII / UII) * transU * np.exp(-chiII / (k * T))
    return wII, wIII


def _species_ctor(partition_funcs):
    """The Species type of the dict's keys (the package's Species(atoms, charge))."""
    spec = next(iter(partition_funcs))
    return lambda Z, q: type(spec)([Z], q)


def get_log_nK(mol, T, log_equilibrium_constants):
    """log10 of n(A)n(B).../n(mol) (statmech.jl:60-62)."""
    return log_equilibrium_constants[mol](np.log(T)) - (len(mol.atoms) - 1) * np.log10(kboltz_cgs * T)


def Hminus_nK(T):
    """n(H-) = nK n(H I) n_e (statmech.jl:73-79)."""
    return np.exp(0.754204 / (kboltz_eV * T)) / (4 * translational_U(electron_mass_cgs, T))


class Residuals:
    """``setup_chemical_equilibrium_residuals`` (statmech.jl:360-439): the scaled residuals of
    nuclei conservation for every element and of charge balance, with their Jacobian."""

    def __init__(self, T, n_tot, absolute_abundances, ionization_energies, partition_funcs,
                 log_equilibrium_constants, logxi):
        self.molecules = list(log_equilibrium_constants)
        self.n_tot, self.logxi = n_tot, logxi
        self.ab = np.asarray(absolute_abundances, np.float64)
        log_nKs = np.array([get_log_nK(m, T, log_equilibrium_constants) for m in self.molecules])
        self.log_nK_Hminus = np.log10(Hminus_nK(T))
        pairs = [saha_ion_weights(T, 1.0, Z, ionization_energies, partition_funcs)
                 for Z in range(1, MAX_ATOMIC_NUMBER + 1)]
        with np.errstate(divide="ignore"):
            self.log_wII_ne = np.log10([p[0] for p in pairs])
            self.log_wIII_ne2 = np.log10([p[1] for p in pairs])
        n = MAX_ATOMIC_NUMBER + 1
        # log10 n(mol) = C @ x + offset: C counts each constituent's neutral density; a singly
        # ionized diatomic takes its first (lower-Z) atom as the ion, adding log wII_ne - log n_e
        C = np.zeros((len(self.molecules), n))
        offset = -log_nKs + logxi
        for i, m in enumerate(self.molecules):
            for Z in m.atoms:
                C[i, Z - 1] += 1
            if m.charge == 1:
                C[i, -1] -= 1
                offset[i] += self.log_wII_ne[m.atoms[0] - 1]
        self.C, self.offset = C, offset
        self.charge = np.array([m.charge for m in self.molecules], np.float64)
        self.extra = np.array([len(m.atoms) - 1 for m in self.molecules], np.float64)

    def __call__(self, x):
        """(F, J) at x: value and exact derivative of statmech.jl:378-438."""
        n = MAX_ATOMIC_NUMBER + 1
        log_ne = x[-1]
        ne = 10.0 ** log_ne
        d_ne = np.zeros(n)
        d_ne[-1] = LN10 * ne
        xa = x[:MAX_ATOMIC_NUMBER]
        # molecules (:385-409)
        n_mol = 10.0 ** (self.C @ x + self.offset)
        d_mol = LN10 * n_mol[:, None] * self.C
        Fa = self.C[:, :MAX_ATOMIC_NUMBER].T @ n_mol
        Ja = self.C[:, :MAX_ATOMIC_NUMBER].T @ d_mol
        n_nuclei = self.n_tot - ne + self.extra @ n_mol
        d_nuclei = -d_ne + self.extra @ d_mol
        Fe = self.charge @ n_mol
        Je = self.charge @ d_mol
        # H- (:411-416)
        n_Hm = 10.0 ** (self.log_nK_Hminus + xa[0] + log_ne + self.logxi)
        Fa[0] += n_Hm
        Ja[0, 0] += LN10 * n_Hm
        Ja[0, -1] += LN10 * n_Hm
        Fe -= n_Hm
        Je[0] -= LN10 * n_Hm
        Je[-1] -= LN10 * n_Hm
        # atoms and their ions (:418-430)
        n_I = 10.0 ** xa
        n_II = 10.0 ** (xa + self.log_wII_ne - log_ne)
        n_III = 10.0 ** (xa + self.log_wIII_ne2 - 2 * log_ne)
        idx = np.arange(MAX_ATOMIC_NUMBER)
        Fa += n_I + n_II + n_III - self.ab * n_nuclei
        Ja[idx, idx] += LN10 * (n_I + n_II + n_III)
        Ja[:, -1] += -LN10 * (n_II + 2 * n_III)
        Ja -= self.ab[:, None] * d_nuclei[None, :]
        Fe += np.sum(n_II + 2 * n_III)
        Je[idx] += LN10 * (n_II + 2 * n_III)
        Je[-1] += -LN10 * np.sum(n_II + 4 * n_III)
        # charge balance LHS and scaling (:432-437)
        Fe -= ne
        Je -= d_ne
        scale = self.ab * self.n_tot
        F = np.concatenate([Fa / scale, [Fe / self.n_tot]])
        J = np.vstack([Ja / scale[:, None], Je[None, :] / self.n_tot])
        return F, J


def clipped_newton(residuals, x0, tol=1e-8, max_iter=200, max_step=1.0):
    """Newton's method with the step clipped to ``max_step`` in every unknown (newton.jl:2-35).
    Returns (x, converged, inf-norm of the last residuals)."""
    x = np.array(x0, np.float64)
    inf_norm = np.inf
    for _ in range(max_iter):
        F, J = residuals(x)
        inf_norm = np.max(np.abs(F))
        if not np.isfinite(inf_norm):
            return x, False, inf_norm
        if inf_norm < tol:
            return x, True, inf_norm
        if not np.all(np.isfinite(J)):
            return x, False, inf_norm
        try:
            step = -np.linalg.solve(J, F)
        except np.linalg.LinAlgError:
            return x, False, inf_norm
        if not np.all(np.isfinite(step)):
            return x, False, inf_norm
        smax = np.max(np.abs(step))
        alpha = max_step / smax if smax > max_step else 1.0
        x = x + alpha * step
    return x, False, inf_norm


def solve_chemical_equilibrium(T, n_tot, absolute_abundances, neutral_fraction_guess, ne_guess,
                               ionization_energies, partition_funcs, log_equilibrium_constants,
                               ftol=1e-8, minimum_annealing_dlogxi=0.0625, trace=None):
    """``_solve_chemical_equilibrium`` (statmech.jl:240-305): the plain solve, else the log xi
    continuation (anchor at -5, -20 or -50, steps of at most 2 that halve on failure down to
    ``minimum_annealing_dlogxi`` and double after a success).  ``trace``, a list, receives
    (log xi, converged, iterations-free inf-norm) per attempted solve."""
    ab = np.asarray(absolute_abundances, np.float64)
    x0 = np.concatenate([np.log10((n_tot - ne_guess) * ab * np.asarray(neutral_fraction_guess)),
                         [np.log10(ne_guess)]])

    def solve_at(logxi, xstart, max_iter):
        r = Residuals(T, n_tot, ab, ionization_energies, partition_funcs, log_equilibrium_constants, logxi)
        out = clipped_newton(r, xstart, tol=ftol, max_iter=max_iter, max_step=1.0)
        if trace is not None:
            trace.append((logxi, out[1], out[2]))
        return out

    x, converged, last_inf = solve_at(0.0, x0, 50)
    if not converged:
        anchor_converged = False
        for lam in (-5.0, -20.0, -50.0):
            x_anchor, anchor_converged, last_inf = solve_at(lam, x0, 100)
            if anchor_converged:
                logxi = lam
                break
        if not anchor_converged:
            raise ChemicalEquilibriumError(f"unconverged at anchor (inf-norm={last_inf})")
        x = x_anchor
        dlogxi_init = 2.0
        dlogxi = dlogxi_init
        while logxi < -1e-12:
            step = min(dlogxi, 0 - logxi)
            x_try, conv, last_inf = solve_at(logxi + step, x, 100)
            if not conv:
                step /= 2
                while not conv and step >= minimum_annealing_dlogxi:
                    x_try, conv, last_inf = solve_at(logxi + step, x, 100)
                    if not conv:
                        step /= 2
                if not conv:
                    raise ChemicalEquilibriumError(f"unconverged at logxi={logxi + 2 * step} (inf-norm={last_inf})")
                dlogxi = step
            else:
                dlogxi = min(dlogxi_init, 2 * step)
            x = x_try
            logxi += step
    if not np.all(np.isfinite(x)):
        raise ChemicalEquilibriumError("solution contains non-finite values")
    return x


_T_FACTORS = {}


def _t_factors(T, ionization_energies, partition_funcs, log_equilibrium_constants):
    """Saha weights at n_e = 1 and log nK of every molecule at T (cached by T)."""
    key = (float(T), id(partition_funcs), id(log_equilibrium_constants))
    if key not in _T_FACTORS:
        w = np.array([saha_ion_weights(T, 1.0, Z, ionization_energies, partition_funcs)
                      for Z in range(1, MAX_ATOMIC_NUMBER + 1)])
        lk = np.array([get_log_nK(m, T, log_equilibrium_constants) for m in log_equilibrium_constants])
        if len(_T_FACTORS) > 64:
            _T_FACTORS.clear()
        _T_FACTORS[key] = (w[:, 0], w[:, 1], lk)
    return _T_FACTORS[key]


def densities_from_x(x, T, ionization_energies, partition_funcs, log_equilibrium_constants):
    """The number densities chemical_equilibrium returns for the solver's unknowns x
    (statmech.jl:160-205, the Saha weights scaled from n_e = 1): {"ne": n_e, Species: n}."""
    species = _species_ctor(partition_funcs)
    w2, w3, lk = _t_factors(T, ionization_energies, partition_funcs, log_equilibrium_constants)
    ne = 10.0 ** x[-1]
    nI = 10.0 ** np.asarray(x[:MAX_ATOMIC_NUMBER])
    nII = w2 / ne * nI
    nIII = w3 / ne ** 2 * nI
    nd = {"ne": ne}
    for Z in range(1, MAX_ATOMIC_NUMBER + 1):
        nd[species(Z, 0)] = nI[Z - 1]
        nd[species(Z, 1)] = nII[Z - 1]
        nd[species(Z, 2)] = nIII[Z - 1]
    nd[type(next(iter(partition_funcs)))([1], -1)] = Hminus_nK(T) * nI[0] * ne
    for mol, log_nK in zip(log_equilibrium_constants, lk):
        if mol.charge == 0:
            s = sum(np.log10(nI[Z - 1]) for Z in mol.atoms)
        else:
            Z1, Z2 = mol.atoms
            s = np.log10(nII[Z1 - 1]) + np.log10(nI[Z2 - 1])
        nd[mol] = 10.0 ** (s - log_nK)
    return nd


def chemical_equilibrium_vjp(T, n_tot, absolute_abundances, x, gbar, ionization_energies, partition_funcs,
                             log_equilibrium_constants, elements=(), rel=1e-6):
    """Gradient of L = sum_s gbar[s] n_s(x*(p), p) with respect to p = T, n_tot and the abundances
    of ``elements`` at the solution x* (the implicit-function rule of the reference's ForwardDiff
    method, statmech.jl:307-355): lambda = J^-T (dn/dx)^T gbar with the restated residuals'
    Jacobian, then dL/dp = gbar (dn/dp)|x - lambda (dF/dp)|x, the explicit derivatives at fixed x
    by central differences (smooth functions; no solver in them).  ``gbar``: {"ne" or Species: g}."""
    ab = np.asarray(absolute_abundances, np.float64)
    args = (ionization_energies, partition_funcs, log_equilibrium_constants)
    keys = list(gbar)
    gv = np.array([gbar[k] for k in keys])
    def dens(xx, TT):
        d = densities_from_x(xx, TT, *args)
        return np.array([d[k] for k in keys])
    n = len(x)
    dndx = np.empty((len(keys), n))
    h = 1e-7
    for j in range(n):
        e = np.zeros(n)
        e[j] = h
        dndx[:, j] = (dens(x + e, T) - dens(x - e, T)) / (2 * h)
    F, J = Residuals(T, n_tot, ab, *args, 0.0)(x)
    lam = np.linalg.solve(J.T, dndx.T @ gv)
    hT = rel * T
    dFdT = (Residuals(T + hT, n_tot, ab, *args, 0.0)(x)[0] - Residuals(T - hT, n_tot, ab, *args, 0.0)(x)[0]) / (2 * hT)
    dndT = (dens(x, T + hT) - dens(x, T - hT)) / (2 * hT)
    hn = rel * n_tot
    dFdn = (Residuals(T, n_tot + hn, ab, *args, 0.0)(x)[0] - Residuals(T, n_tot - hn, ab, *args, 0.0)(x)[0]) / (2 * hn)
    dab = {}
    for Z in elements:
        ha = rel * ab[Z - 1]
        ap, am = ab.copy(), ab.copy()
        ap[Z - 1] += ha
        am[Z - 1] -= ha
        dFda = (Residuals(T, n_tot, ap, *args, 0.0)(x)[0] - Residuals(T, n_tot, am, *args, 0.0)(x)[0]) / (2 * ha)
        dab[Z] = -lam @ dFda
    return gv @ dndT - lam @ dFdT, -lam @ dFdn, dab


def chemical_equilibrium(T, n_tot, model_atm_ne, absolute_abundances, ionization_energies,
                         partition_funcs, log_equilibrium_constants,
                         electron_number_density_warn_threshold=0.1,
                         electron_number_density_warn_min_value=1e-4):
    """(n_e, {Species: n}) for one layer (statmech.jl:148-206)."""
    species = _species_ctor(partition_funcs)
    guess = []
    for Z in range(1, MAX_ATOMIC_NUMBER + 1):
        wII, wIII = saha_ion_weights(T, model_atm_ne, Z, ionization_energies, partition_funcs)
        guess.append(1 / (1 + wII + wIII))
    x = solve_chemical_equilibrium(T, n_tot, absolute_abundances, np.array(guess), model_atm_ne,
                                   ionization_energies, partition_funcs, log_equilibrium_constants)
    ne = 10.0 ** x[-1]
    if (ne / n_tot > electron_number_density_warn_min_value and
            abs((ne - model_atm_ne) / model_atm_ne) > electron_number_density_warn_threshold):
        warnings.warn(f"Electron number density differs from model atmosphere by a factor greater than "
                      f"{electron_number_density_warn_threshold}. (calculated ne = {ne}, model atmosphere "
                      f"ne = {model_atm_ne})")
    nd = {}
    for Z in range(1, MAX_ATOMIC_NUMBER + 1):
        nd[species(Z, 0)] = 10.0 ** x[Z - 1]
    for Z in range(1, MAX_ATOMIC_NUMBER + 1):
        wII, wIII = saha_ion_weights(T, ne, Z, ionization_energies, partition_funcs)
        nd[species(Z, 1)] = wII * nd[species(Z, 0)]
        nd[species(Z, 2)] = wIII * nd[species(Z, 0)]
    Hminus = type(next(iter(partition_funcs)))([1], -1)
    nd[Hminus] = Hminus_nK(T) * nd[species(1, 0)] * ne
    for mol in log_equilibrium_constants:
        log_nK = get_log_nK(mol, T, log_equilibrium_constants)
        if mol.charge == 0:
            s = sum(np.log10(nd[species(Z, 0)]) for Z in mol.atoms)
        else:
            Z1, Z2 = mol.atoms
            s = np.log10(nd[species(Z1, 1)]) + np.log10(nd[species(Z2, 0)])
        nd[mol] = 10.0 ** (s - log_nK)
    return ne, nd
