"""Shared checks of the chemical-equilibrium tests: the reference's property test
(test/statmech.jl:103-150, ``check_solution``) restated, its representative stars
(test/statmech.jl:145-154) and C/O sweep (:170-197)."""
import numpy as np

from korg_gb300.species import Species, parse_species

# (Teff, logg, [M/H], [alpha/M], [C/M], label), test/statmech.jl:145-154
REPRESENTATIVE = [(5777.0, 4.44, 0.0, 0.0, 0.0, "solar"), (4500.0, 2.5, -0.5, 0.2, 0.0, "K giant"),
                  (3500.0, 4.8, 0.0, 0.0, 0.0, "M dwarf"), (2800.0, 0.5, -2.5, -1.0, -1.5, "extreme cool C-poor giant"),
                  (2800.0, 4.5, -2.5, 0.0, 0.0, "cool metal-poor dwarf"), (4000.0, 0.5, 0.5, 0.0, 0.0, "cool metal-rich giant"),
                  (3000.0, 5.0, -4.0, 0.4, 0.0, "low-Z cool dwarf"), (2500.0, 5.0, -5.0, 0.4, 0.0, "low-Z extreme cool dense dwarf")]
ALPHA = (8, 10, 12, 14, 16, 18, 20, 22)  # O Ne Mg Si S Ar Ca Ti (src/abundances.jl)
CO_LOG_RATIOS = [-0.5, -0.2, -0.1, -0.02, 0.0, 0.02, 0.1, 0.2, 0.5]


def format_A_X(M_H=0.0, alpha_M=0.0, C_M=0.0):
    """A(X) with metals scaled by [M/H], alpha elements by [alpha/M] + [M/H] and C by [C/M] + [M/H]
    (format_A_X(M_H, alpha_H, Dict("C" => ...)) as the reference test calls it)."""
    from korg_gb300.standin import solar_A_X
    A = solar_A_X.copy()
    A[2:] += M_H
    for Z in ALPHA:
        A[Z - 1] += alpha_M
    A[5] += C_M
    return A


def absolute_abundances(A_X):
    ab = 10.0 ** (np.asarray(A_X, np.float64) - 12)
    return ab / ab.sum()


def representative_atmospheres():
    """(label, T, n_tot, ne, absolute abundances) of the representative stars: grey synthetic
    atmospheres with the stars' Teff, log g and abundances (the MARCS grid is not distributed)."""
    from korg_gb300 import standin
    out = []
    for Teff, logg, M_H, a_M, C_M, label in REPRESENTATIVE:
        A_X = format_A_X(M_H, a_M, C_M)
        atm, _ = standin.synthetic_atmosphere(Teff, logg, M_H)
        out.append((label, atm.T, atm.n_tot, atm.ne, absolute_abundances(A_X)))
    return out


def marcs_atmospheres():
    """The reference's three MARCS test atmospheres (tests/golden/marcs_layers.npz), with their
    own abundance tables (absent elements at A = -5)."""
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "marcs_layers.npz"))
    out = []
    for k in ("sun", "s5000", "s6000"):
        A = np.where(d[k + "_A_X"] < -5, -5.0, d[k + "_A_X"])
        out.append((k, d[k + "_T"], d[k + "_n_tot"], d[k + "_ne"], absolute_abundances(A)))
    return out


def _isapprox(a, b, rtol):
    """Julia's isapprox for arrays: norm(a - b) <= rtol * max(norm(a), norm(b))."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def check_solution(T, ne, nd, nt, ab, Hminus_nK, rtol=1e-8):
    """The failed properties of one layer's solution (empty list: all hold)."""
    bad = []
    if not (np.isfinite(ne) and ne > 0):
        bad.append("ne")
    if not all(np.isfinite(v) and v >= 0 for v in nd.values()):
        bad.append("densities finite and >= 0")
    pos = sum(n * s.charge for s, n in nd.items())
    if not abs(ne - pos) <= rtol * max(abs(ne), abs(pos)):
        bad.append(f"charge balance {ne} vs {pos}")
    Hm, HI = nd[Species([1], -1)], nd[parse_species("H I")]
    if not (abs(Hm - Hminus_nK(T) * HI * ne) <= 1e-5 * max(Hm, Hminus_nK(T) * HI * ne) and Hm > 0):
        bad.append("H-")
    tot = ne + sum(nd.values())
    if not abs(tot - nt) <= rtol * max(tot, nt):
        bad.append(f"total density {tot} vs {nt}")
    nuc = np.zeros(92)
    for s, n in nd.items():
        for Z in s.atoms:
            nuc[Z - 1] += n
    if not _isapprox(nuc / nuc.sum(), ab, rtol):
        bad.append("abundances")
    if not nd[parse_species("C I")] < HI:
        bad.append("n(C I) < n(H I)")
    if T <= 6000 and not (nd[parse_species("C III")] < nd[parse_species("C II")] < nd[parse_species("C I")]):
        bad.append("C III < C II < C I")
    return bad


def co_bound_ok(nd):
    """CO cannot exceed the smaller of the total C and O nuclear densities (test/statmech.jl:189-195)."""
    nC = sum(n * s.atoms.count(6) for s, n in nd.items())
    nO = sum(n * s.atoms.count(8) for s, n in nd.items())
    return nd[parse_species("CO")] <= min(nC, nO)
