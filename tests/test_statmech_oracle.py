"""The FP64 chemical-equilibrium restatement (oracle/statmech_oracle.py) and the converted data
against the reference's own statmech tests (test/statmech.jl), restated.  CPU only.

The reference pins chemical equilibrium by properties (charge, particle-number and nuclei
conservation, the H- relation, ion ordering, insensitivity to the n_e guess, determinism) rather
than golden values; the same properties pin the restatement here, on the reference's three MARCS
test atmospheres and on synthetic atmospheres of its representative stars."""
import numpy as np
import pytest

import chem_checks as cc


@pytest.fixture(scope="module")
def so():
    import statmech_oracle
    return statmech_oracle


@pytest.fixture(scope="module")
def tabs():
    from korg_gb300 import data
    return data.ionization_energies(), data.default_partition_funcs(), data.default_log_equilibrium_constants()


def _run(so, tabs, T, nt, ne, ab):
    chi, pf, K = tabs
    return so.chemical_equilibrium(T, nt, ne, ab, chi, pf, K, electron_number_density_warn_threshold=np.inf)


def test_ionization_energies_and_tables(tabs):
    """test/statmech.jl:231-236, and the molecule set: 282 Barklem & Collet molecules plus 24
    polyatomics with atomization energies (src/read_statmech_quantities.jl:53-98)."""
    chi, pf, K = tabs
    assert len(chi) == 92
    assert chi[1] == [13.5984, -1.0, -1.0]
    assert chi[44] == [7.3605, 16.760, 28.470]
    assert chi[92] == [6.1940, 11.590, 19.800]
    assert len(K) == 306
    from korg_gb300.data import PolyatomicLogK
    from korg_gb300.species import parse_species
    assert sum(isinstance(f, PolyatomicLogK) for f in K.values()) == 24
    assert isinstance(K[parse_species("H2O")], PolyatomicLogK) and parse_species("CO") in K


def test_C2_correction():
    """The C2 constant is shifted by log10(e) (D_Visser - D_BC) / kT (src/read_statmech_quantities.jl:109-118)."""
    from korg_gb300 import data
    e = data._npz("equilibrium_constants.npz")
    k = list(e["bc_mols"]).index("CC")
    from korg_gb300.species import parse_species
    spec, lnT, logK = next(x for x in data.barklem_collet_log_K_tables() if x[0] == parse_species("C2"))
    raw = e["bc_logKs"][k][np.isfinite(e["bc_lnTs"][k])]
    corr = np.log10(np.e) / (8.617333262145e-5 * np.exp(lnT)) * (6.24 - 6.371)
    assert np.allclose(logK - raw, corr, rtol=1e-12, atol=0)


def test_polyatomic_partition_functions_astrophysical_convention():
    """ExoMol partition functions divided by the nuclear-spin degeneracy of the most abundant
    isotopologue (src/read_statmech_quantities.jl:211-224): H2O 4, HCN 6, CO2 1."""
    from korg_gb300 import data
    e = data._npz("equilibrium_constants.npz")
    g = dict(zip(e["poly_names"], e["poly_g_ns"]))
    assert (g["HHO"], g["HCN"], g["COO"]) == (4.0, 6.0, 1.0)


def test_partition_functions_nearly_monotonic(tabs):
    """test/statmech.jl:238-245."""
    from korg_gb300.species import parse_species
    _, pf, _ = tabs
    lnTs = np.arange(0, np.log(100_000.0), 0.1)
    for s in ("O I", "O II", "O III", "CN"):
        assert np.all(np.diff(pf[parse_species(s)](lnTs)) > -1e-4), s


def test_saha_pure_hydrogen(so):
    """test/statmech.jl:2-34: the Saha equation of a pure-H plasma, rtol 1e-14 (1e-9 at 1.5e5 K)."""
    from korg_gb300.species import Species
    nH = 1e15
    chis = {1: [13.598287264, -1.0, -1.0]}

    class Const:
        def __init__(self, v):
            self.v = v

        def __call__(self, lnT):
            return self.v

    Us = {Species([1], 0): Const(2.0), Species([1], 1): Const(1.0)}
    for T in [3e3, 4e3, 5e3, 6e3, 7e3, 8e3, 9e3, 1e4, 1.1e4, 1.2e4, 1.3e4, 1.4e4, 1.5e5]:
        coef = 2.0 * (2.0 * np.pi * so.electron_mass_cgs * so.kboltz_cgs / so.hplanck_cgs ** 2) ** 1.5
        rhs = coef * T ** 1.5 * np.exp(-13.598287264 / (so.kboltz_eV * T)) / 2.0
        ne = (-rhs + np.sqrt(rhs * rhs + 4 * rhs * nH)) / 2
        wII, wIII = so.saha_ion_weights(T, ne, 1, chis, Us)
        assert wIII == 0.0
        rtol = 1e-9 if T == 1.5e5 else 1e-14
        assert abs(wII / (1 + wII + wIII) - ne / nH) <= rtol * (ne / nH)


def test_monotonic_N_ions(so, tabs):
    """test/statmech.jl:36-44."""
    chi, pf, _ = tabs
    w = [so.saha_ion_weights(float(T), 1.0, 7, chi, pf) for T in range(1, 10000, 100)]
    assert np.all(np.diff([a + b for a, b in w]) >= 0)
    assert np.all(np.diff([b for _, b in w]) >= 0)


def test_jacobian_is_the_derivative(so, tabs):
    """The forward-mode Jacobian of the restated residuals against central differences, at a
    solution (where the residual terms balance, so differences are not swamped by round-off)."""
    chi, pf, K = tabs
    ab = cc.absolute_abundances(cc.format_A_X())
    guess = np.array([1 / (1 + sum(so.saha_ion_weights(3000.0, 1e10, Z, chi, pf))) for Z in range(1, 93)])
    x = so.solve_chemical_equilibrium(3000.0, 1e16, ab, guess, 1e10, chi, pf, K)
    r = so.Residuals(3000.0, 1e16, ab, chi, pf, K, 0.0)
    F, J = r(x)
    for c in (0, 5, 7, 8, 25, 92):
        h = 1e-5
        e = np.zeros(93)
        e[c] = h
        fd = (r(x + e)[0] - r(x - e)[0]) / (2 * h)
        assert np.allclose(J[:, c], fd, rtol=1e-6, atol=1e-9 * np.max(np.abs(J[:, c]))), c


@pytest.mark.parametrize("atm", ["sun", "s5000", "s6000"])
def test_marcs_layers(so, tabs, atm):
    """check_solution (test/statmech.jl:103-150) on every 7th layer of the MARCS test atmospheres."""
    label, T, nt, ne, ab = next(a for a in cc.marcs_atmospheres() if a[0] == atm)
    for l in range(0, len(T), 7):
        ne_l, nd = _run(so, tabs, T[l], nt[l], ne[l], ab)
        assert cc.check_solution(T[l], ne_l, nd, nt[l], ab, so.Hminus_nK) == [], (label, l)


@pytest.mark.parametrize("k", [0, 2, 4, 7])
def test_representative_stars(so, tabs, k):
    """check_solution on the top, middle and bottom layers of representative stars, including
    cool dense dwarfs that need the log xi continuation."""
    label, T, nt, ne, ab = cc.representative_atmospheres()[k]
    for l in (0, len(T) // 3, len(T) // 2, len(T) - 1):
        ne_l, nd = _run(so, tabs, T[l], nt[l], ne[l], ab)
        assert cc.check_solution(T[l], ne_l, nd, nt[l], ab, so.Hminus_nK) == [], (label, l)


def test_insensitive_to_ne_guess(so, tabs):
    """test/statmech.jl:61-74: rtol 1e-8 on n_e, 1e-7 on every density."""
    ab = cc.absolute_abundances(cc.format_A_X())
    res = [_run(so, tabs, 3500.0, 1e16, g, ab) for g in (1e6, 1e9, 1e11, 1e13, 1e15)]
    ne0, nd0 = res[0]
    for ne, nd in res[1:]:
        assert abs(ne - ne0) <= 1e-8 * ne0
        a = np.array([nd0[s] for s in nd0])
        b = np.array([nd[s] for s in nd0])
        assert np.all(np.abs(a - b) <= 1e-7 * np.maximum(np.abs(a), np.abs(b)))


def test_deterministic(so, tabs):
    """test/statmech.jl:76-86: bitwise-identical reruns."""
    ab = cc.absolute_abundances(cc.format_A_X())
    a, b = _run(so, tabs, 3000.0, 1e16, 1e10, ab), _run(so, tabs, 3000.0, 1e16, 1e10, ab)
    assert a[0] == b[0] and all(a[1][s] == b[1][s] for s in a[1])


@pytest.mark.parametrize("d", [-0.5, 0.0, 0.02, 0.5])
def test_CO_ratio_sweep(so, tabs, d):
    """test/statmech.jl:170-197 at T = 1500 K, n_tot = 1e17 (the continuation regime)."""
    A_X = cc.format_A_X()
    A_X[5] = A_X[7] + d
    ab = cc.absolute_abundances(A_X)
    ne, nd = _run(so, tabs, 1500.0, 1e17, 1e9, ab)
    assert cc.check_solution(1500.0, ne, nd, 1e17, ab, so.Hminus_nK) == []
    assert cc.co_bound_ok(nd)


def _cotangent(nd, nt, seed):
    """Random cotangent g_s = r_s / n_s on the species above 1e-30 n_tot (every species weighs O(1))."""
    rng = np.random.default_rng(seed)
    return {k: (rng.normal() / v if v > 1e-30 * nt else 0.0) for k, v in nd.items()}


def test_vjp_matches_solver_differences(so, tabs):
    """The implicit-function gradient of L = sum g n against central differences of the whole
    solve (what ForwardDiff through chemical_equilibrium gives in the reference,
    test/statmech.jl:199-212), at a solar photospheric layer."""
    chi, pf, K = tabs
    ab = cc.absolute_abundances(cc.format_A_X())
    T, nt, ne0 = 5000.0, 1e16, 1e12

    def solve(TT, ntt, abb):  # the solve, then two plain Newton steps: x to rounding level
        guess = np.array([1 / (1 + sum(so.saha_ion_weights(TT, ne0, Z, chi, pf))) for Z in range(1, 93)])
        x = so.solve_chemical_equilibrium(TT, ntt, abb, guess, ne0, chi, pf, K)
        r = so.Residuals(TT, ntt, abb, chi, pf, K, 0.0)
        for _ in range(2):
            F, J = r(x)
            x = x - np.linalg.solve(J, F)
        return x, so.densities_from_x(x, TT, chi, pf, K)

    x, nd = solve(T, nt, ab)
    g = _cotangent(nd, nt, 0)
    loss = lambda d: sum(g[k] * d[k] for k in g)
    dT, dnt, dab = so.chemical_equilibrium_vjp(T, nt, ab, x, g, chi, pf, K, elements=(6, 26))
    h = 1e-5  # relative step: the Boltzmann factors' (chi / kT)^2 ~ 900 make h^2 terms ~1e-5 at 1e-4
    fT = (loss(solve(T * (1 + h), nt, ab)[1]) - loss(solve(T * (1 - h), nt, ab)[1])) / (2 * h * T)
    fn = (loss(solve(T, nt * (1 + h), ab)[1]) - loss(solve(T, nt * (1 - h), ab)[1])) / (2 * h * nt)
    assert abs(dT - fT) <= 1e-5 * abs(fT), (dT, fT)
    assert abs(dnt - fn) <= 1e-5 * abs(fn), (dnt, fn)
    for Z in (6, 26):
        ap, am = ab.copy(), ab.copy()
        ap[Z - 1] *= 1 + h
        am[Z - 1] *= 1 - h
        fa = (loss(solve(T, nt, ap)[1]) - loss(solve(T, nt, am)[1])) / (2 * h * ab[Z - 1])
        assert abs(dab[Z] - fa) <= 1e-5 * abs(fa), (Z, dab[Z], fa)


def test_product_host_helpers_match_the_restatement(so, tabs):
    """The package's host helpers mirroring src/statmech.jl:19-79 (saha_ion_weights,
    translational_U, get_log_nK, Hminus_nK) equal the restatement's over temperatures, electron
    densities, elements and molecules."""
    from korg_gb300 import statmech as sm
    from korg_gb300.constants import electron_mass_cgs
    chi, pf, K = tabs
    Ts = np.array([2500.0, 3500.0, 5777.0, 9000.0, 15000.0])
    for T in Ts:
        assert sm.translational_U(electron_mass_cgs, T) == pytest.approx(so.translational_U(electron_mass_cgs, T),
                                                                         rel=1e-15)
        assert sm.Hminus_nK(T) == pytest.approx(so.Hminus_nK(T), rel=1e-15)
        for ne in (1e8, 1e12, 1e15):
            for Z in (1, 2, 6, 8, 12, 14, 20, 26, 56, 92):
                a, b = sm.saha_ion_weights(T, ne, Z, chi, pf), so.saha_ion_weights(T, ne, Z, chi, pf)
                np.testing.assert_allclose(a, b, rtol=1e-15, atol=0)
        for mol in list(K)[::17]:
            assert sm.get_log_nK(mol, T, K) == pytest.approx(so.get_log_nK(mol, T, K), rel=1e-14, abs=1e-12)


def test_equilibrium_tables_layout():
    """The host table builder (korg_set_equilibrium_tables' input) on the package's data: 306
    molecules, the densities layout n_e, (Z, charge 0..2) for Z = 1..92, H-, then the molecules."""
    from korg_gb300 import _lib
    from korg_gb300.species import Species, parse_species
    from korg_gb300.statmech import default_equilibrium_tables
    t = default_equilibrium_tables()
    assert len(t.molecules) == 306
    sp = t.species
    assert len(sp) == _lib.KORG_CHEM_MOL0 + 306 and _lib.KORG_CHEM_MOL0 == 278
    assert sp[0] is None
    assert sp[1] == parse_species("H I") and sp[2] == parse_species("H II")
    assert sp[1 + 3 * 25] == parse_species("Fe I") and sp[3 + 3 * 25] == parse_species("Fe III")
    assert sp[277] == Species([1], -1)
    assert list(sp[278:]) == list(t.molecules)
    assert parse_species("CO") in t.molecules and parse_species("H2O") in t.molecules
