"""The FP64 continuum-absorption restatement (oracle/continuum_oracle.py) against the reference's
own continuum tests (test/continuum_absorption.jl): the same comparison functions and tolerances,
restated.  CPU only."""
import numpy as np
import pytest

c_cgs, kboltz_cgs = 2.99792458e10, 1.380649e-16


@pytest.fixture(scope="module")
def co():
    import continuum_oracle
    return continuum_oracle


def _rel(a, b):
    return np.max(np.abs(a - b) / np.abs(b))


def test_Hminus_ff_against_gray_polynomial(co):
    """test/continuum_absorption.jl:87-104 (Gray 2005 eq. 8.13), rtol 0.0225."""
    lam = np.array([9113, 7595, 6510, 5696, 5063, 4557, 3645, 3038, 2604.0])
    theta = np.array([0.5, 0.6, 0.8, 1.0, 1.2, 1.4, 1.6, 1.8])
    ll, lt = np.log10(lam)[:, None], np.log10(theta)[None, :]
    f0 = -2.2763 - 1.6850 * ll + 0.76661 * ll ** 2 - 0.053346 * ll ** 3
    f1 = 15.2827 - 9.2846 * ll + 1.99381 * ll ** 2 - 0.142631 * ll ** 3
    f2 = -197.789 + 190.266 * ll - 67.9775 * ll ** 2 + 10.6913 * ll ** 3 - 0.625151 * ll ** 4
    ref = 1e-26 * (kboltz_cgs * (5040 / 10 ** lt) * 1.0) * 10.0 ** (f0 + f1 * lt + f2 * lt * lt)
    got = np.array([[co.Hminus_ff(np.array([c_cgs / (l * 1e-8)]), 5040.0 / t, 0.5, 1.0)[0] for t in theta] for l in lam])
    assert _rel(got, ref) <= 0.0225


def test_Hminus_bf_against_gray_and_extremes(co):
    """test/continuum_absorption.jl:118-175: Gray (2005) eq. 8.11 over 2250-15000 A (rtol 0.02),
    zero below the electron affinity, increasing from threshold into the table."""
    lam = np.arange(2250.0, 15000.0 + 1, 1.0)
    gray = 1e-18 * (1.99654 - 1.18267e-5 * lam + 2.64243e-6 * lam ** 2 - 4.40524e-10 * lam ** 3 +
                    3.23992e-14 * lam ** 4 - 1.39568e-18 * lam ** 5 + 2.78701e-23 * lam ** 6)
    assert _rel(co.Hminus_bf_cross_section(c_cgs / (lam * 1e-8)), gray) <= 0.02
    assert co.Hminus_bf_cross_section(np.array([c_cgs / (20_000e-8)]))[0] == 0
    nu_ion = co.H_MINUS_ION_EV / co.hplanck_eV
    nus = np.arange(nu_ion, co.tables()["Hminus_bf_nu"][0] + 2e13, 1e12)
    assert np.all(np.diff(co.Hminus_bf_cross_section(nus)) > 0)


def test_Heminus_ff_against_gray_polynomial(co):
    """test/continuum_absorption.jl:196-236 (Gray 2005 eq. 8.16), rtol 0.05."""
    T = np.arange(2520.0, 10080 + 1, 100.0)
    lam = np.arange(5063.0, 150_000, 1000.0)
    th = (5040.0 / T)[None, :]
    c0 = 9.66736 - 71.76242 * th + 105.29576 * th ** 2 - 56.49259 * th ** 3 + 10.69206 * th ** 4
    c1 = -10.50614 + 48.28802 * th - 70.43363 * th ** 2 + 37.80099 * th ** 3 - 7.15445 * th ** 4
    c2 = 2.74020 - 10.62144 * th + 15.50518 * th ** 2 - 8.33845 * th ** 3 + 1.57960 * th ** 4
    c3 = -0.19923 + 0.77485 * th - 1.13200 * th ** 2 + 0.60994 * th ** 3 - 0.11564 * th ** 4
    ll = np.log10(lam)[:, None]
    ref = 1e-26 * 10.0 ** (c0 + c1 * ll + c2 * ll ** 2 + c3 * ll ** 3) * kboltz_cgs * (5040.0 / th)
    nu = c_cgs / (lam * 1e-8)
    got = np.stack([co.Heminus_ff(nu, t, 1.0, 1.0) for t in T], axis=1)
    assert _rel(got, ref) <= 0.05


def test_H2plus_against_bates_1952(co):
    """test/continuum_absorption.jl:244-296 (Bates 1952 table II), rtol 0.2."""
    table = np.array([[1.77, 1.35, 1.09, 0.92, 0.79, 0.62, 0.51], [1.96, 1.47, 1.17, 0.98, 0.84, 0.66, 0.54],
                      [2.15, 1.57, 1.25, 1.04, 0.89, 0.69, 0.57], [2.33, 1.67, 1.31, 1.08, 0.92, 0.71, 0.58],
                      [2.53, 1.77, 1.37, 1.12, 0.95, 0.73, 0.59], [2.74, 1.87, 1.43, 1.16, 0.97, 0.74, 0.60],
                      [2.95, 1.97, 1.48, 1.19, 0.99, 0.75, 0.61], [3.4, 2.18, 1.58, 1.25, 1.03, 0.77, 0.62],
                      [4.0, 2.40, 1.69, 1.30, 1.06, 0.78, 0.62], [4.7, 2.64, 1.80, 1.36, 1.09, 0.78, 0.62],
                      [5.4, 2.91, 1.91, 1.41, 1.11, 0.79, 0.61], [6.3, 3.2, 2.03, 1.46, 1.14, 0.79, 0.61],
                      [7.3, 3.5, 2.16, 1.52, 1.16, 0.79, 0.60], [8.4, 3.8, 2.29, 1.57, 1.18, 0.79, 0.59],
                      [9.6, 4.2, 2.42, 1.63, 1.21, 0.79, 0.58]])
    T = np.array([4.0e3, 5.0e3, 6.0e3, 7.0e3, 8.0e3, 1.0e4, 1.2e4])
    k = np.array([4000, 5000, 6000, 7000, 8000, 9000, 10000, 12000, 14000, 16000, 18000, 20000, 22000, 24000, 26000.0])
    nH_I, nH_II = 1e15, 1e13
    got = np.stack([1e39 / (nH_I * nH_II) * co.H2plus_bf_and_ff(c_cgs * k, t, nH_I, nH_II) for t in T], axis=1)
    assert _rel(got, table) <= 0.2


def test_gaunt_ff_against_kurucz_1970(co):
    """test/continuum_absorption.jl:306-342 (Karsas & Latter values tabulated by Kurucz), rtol 0.15,
    where both tables have data."""
    g2 = np.array([-3.0, -2.5, -2.0, -1.5, -1.0, -0.5, 0.0, 0.5, 1.0, 1.5, 2.0])
    u = np.array([-4.0, -3.5, -3.0, -2.5, -2.0, -1.5, -1.0, -0.5, 0.0, 0.5, 1.0, 1.5])
    ref = np.array([[5.53, 5.49, 5.46, 5.43, 5.40, 5.25, 5.00, 4.69, 4.48, 4.16, 3.85],
                    [4.91, 4.87, 4.84, 4.80, 4.77, 4.63, 4.40, 4.13, 3.87, 3.52, 3.27],
                    [4.29, 4.25, 4.22, 4.18, 4.15, 4.02, 3.80, 3.57, 3.27, 2.98, 2.70],
                    [3.64, 3.61, 3.59, 3.56, 3.54, 3.41, 3.22, 2.97, 2.70, 2.45, 2.20],
                    [3.00, 2.98, 2.97, 2.95, 2.94, 2.81, 2.65, 2.44, 2.21, 2.01, 1.81],
                    [2.41, 2.41, 2.41, 2.41, 2.41, 2.32, 2.19, 2.02, 1.84, 1.67, 1.50],
                    [1.87, 1.89, 1.91, 1.93, 1.95, 1.90, 1.80, 1.68, 1.52, 1.41, 1.30],
                    [1.33, 1.39, 1.44, 1.49, 1.55, 1.56, 1.51, 1.42, 1.33, 1.25, 1.17],
                    [0.90, 0.95, 1.00, 1.08, 1.17, 1.30, 1.32, 1.30, 1.20, 1.15, 1.11],
                    [0.45, 0.48, 0.52, 0.60, 0.75, 0.91, 1.15, 1.18, 1.15, 1.11, 1.08],
                    [0.33, 0.36, 0.39, 0.46, 0.59, 0.76, 0.97, 1.09, 1.13, 1.10, 1.08],
                    [0.19, 0.21, 0.24, 0.28, 0.38, 0.53, 0.76, 0.96, 1.08, 1.09, 1.09]])
    t = co.tables()
    ui = (u >= t["gaunt_log_u"][0]) & (u <= t["gaunt_log_u"][-1])
    gi = (g2 >= t["gaunt_log_g2"][0]) & (g2 <= t["gaunt_log_g2"][-1])
    assert ui.any() and gi.any()
    got = co.gaunt_ff(u[ui][:, None], g2[gi][None, :])
    assert _rel(got, ref[np.ix_(ui, gi)]) <= 0.15


def test_H_I_ff_against_gray(co):
    """test/continuum_absorption.jl:357-432 (Gray 2005 eq. 8.10 with eq. 8.6 Gaunt factor), rtol 0.034."""
    lam = 3e3 + 250.0 * np.arange(69)
    nu = c_cgs * 1e8 / lam
    R = 1.0968e5
    I = co.hplanck_eV * c_cgs * R
    loge = np.log10(np.e)
    for logPe, T in [(1.08, 5143.0), (1.77, 6429.0), (2.50, 7715.0), (2.76, 11572.0)]:
        theta = 5040 / T
        chi_lam = 1.2398e4 / lam
        gff = 1.0 + 0.3456 * (0.5 + loge / (theta * chi_lam)) / np.cbrt(lam * R / 1e8)
        ref = 1.0449e-26 * lam ** 3 * gff * loge * 10.0 ** (-theta * I) / (2 * theta * I) * (1 - 10.0 ** (-chi_lam * theta))
        ne = 10.0 ** logPe / (kboltz_cgs * T)
        nH = ne * 100.0
        transU = (2 * np.pi * co.electron_mass_cgs * kboltz_cgs * T / co.hplanck_cgs ** 2) ** 1.5
        wII = 2.0 / ne * (1.0 / 2.0) * transU * np.exp(-co.RydbergH_eV / (co.kboltz_eV * T))
        nH_I, nH_II = nH / (1 + wII), nH * wII / (1 + wII)
        got = co.positive_ion_ff(nu, T, ne, nH_II, 0.0, {})
        assert np.all(got >= 0) and _rel(got / nH_I, ref) <= 0.034


def test_H_I_bf_against_gray(co):
    """test/continuum_absorption.jl:434-534 (Gray 2005 eq. 8.8), rtol 0.09."""
    lam = 3e3 + 250.0 * np.arange(69)
    nu = c_cgs * 1e8 / lam
    chi = co.chi_H
    for T in [5143.0, 6429.0, 7715.0, 11572.0]:
        theta = 5040 / T
        ref = np.empty_like(lam)
        for k, l in enumerate(lam):
            e_ph = co.hplanck_eV * c_cgs * 1e8 / l
            n0 = int(np.ceil(np.sqrt(chi / e_ph)))
            s = 0.0
            for n in range(n0, n0 + 4):
                x = chi * (1.0 - 1.0 / (n * n))
                gbf = 1.0 - 0.3456 * (l * 1.0968e-3 / (n * n) - 0.5) / np.cbrt(l * 1.0968e-3)
                s += 10.0 ** (-theta * x) * gbf / n ** 3
            x3 = chi * (1 - 1 / (n0 + 3) ** 2)
            integ = (10 ** (-x3 * theta) - 10 ** (-chi * theta)) * 0.5 * 0.43429 / (theta * chi)
            ref[k] = 1.0449e-26 * l ** 3 * (s + integ) * (1 - 10.0 ** (-1.2398e4 / l * theta))
        got = co.H_I_bf(nu, T, 1.0, 0.0, 0.0, 0.5)
        assert np.all(got >= 0) and _rel(got, ref) <= 0.09


def test_Hminus_opacity_minimum_at_1_6_micron(co):
    """test/continuum_absorption.jl:570-589: at the tau ~ 1 layer of a solar atmosphere the total
    continuum opacity is lower at 1.6 um than at 0.5 um (chemical equilibrium: the stand-in)."""
    from korg_gb300 import standin
    from korg_gb300.continuum import layer_inputs
    T, n_total = 6400.0, 1.5e17
    ne, nd = standin.chemical_equilibrium(np.array([T]), np.array([n_total]), standin.format_A_X(0.0))
    d = {k: v[0] for k, v in layer_inputs(np.array([T]), ne, nd).items()}
    a = co.total_continuum_absorption(c_cgs / np.array([1.6e-4, 5e-5]), T, d["ne"], d)
    assert a[0] < a[1]
