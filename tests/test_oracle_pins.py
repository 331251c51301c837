"""The FP64 oracle against the reference's own known answers and golden vectors (CPU)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_voigt_normalisation_and_monotonicity(oracle_lib):
    """test/line_absorption.jl:4-17: 0.98 < sum(phi dl)/amp < 1 and monotone within 1e-3 max."""
    from korg_gb300.wavelengths import Wavelengths
    wls = Wavelengths((4750, 5250)).all_wls
    d = 0.01e-8
    amp = 7.0
    for sigma in [1e-7, 1e-8, 1e-9]:
        for gamma in [3e-8, 3e-9, 3e-10]:
            phi = oracle_lib.line_profile(5e-5, sigma, gamma, amp, wls)
            half = int(np.ceil(len(phi) / 2))
            assert np.all(np.diff(phi[:half]) > -1e-3 * phi.max())
            assert np.all(np.diff(phi[half - 1:]) < 1e-3 * phi.max())
            assert 0.98 < (phi * d).sum() / amp < 1


def test_expint2_against_scipy(oracle_lib):
    """test/transfer.jl:4-7: E2 approximation within rtol 1e-3 of expint(2, x) on 2:0.01:8."""
    from scipy.special import expn
    x = np.arange(2, 8.0000001, 0.01)
    np.testing.assert_allclose(oracle_lib.exponential_integral_2(x), expn(2, x), rtol=1e-3)


def test_expint2_branches_continuous(oracle_lib):
    """The piecewise E2 (RadiativeTransfer.jl:408-497) is accurate to ~1% everywhere."""
    from scipy.special import expn
    x = np.concatenate([np.geomspace(1e-8, 1, 200), np.linspace(1, 30, 400)])
    np.testing.assert_allclose(oracle_lib.exponential_integral_2(x), expn(2, x), rtol=1.5e-2)
    assert oracle_lib.exponential_integral_2(np.array([0.0]))[0] == 1.0


def test_lyman_golden(oracle_lib):
    """test/line_absorption.jl:19-39: hydrogen_line_absorption! vs the reference golden vector,
    atol 5e-9 (T = 9000 K, xi = 0, window 150 A, use_MHD = false)."""
    from korg_gb300.data import stark_profiles
    from korg_gb300.wavelengths import Wavelengths
    g = np.load(os.path.join(HERE, "golden", "lyman_absorption.npz"))
    w = Wavelengths([(float(g["start_wl"]), float(g["stop_wl"]), float(g["wl_step"]))])
    assert len(w) == len(g["profile"])
    a = np.zeros(len(w))
    oracle_lib.hydrogen_line_absorption(a, w.all_wls, 9000.0, float(g["ne"]), float(g["nH_I"]), 0.0,
                                        float(g["UH_I_9000"]), 0.0, 15e-7, False, stark_profiles())
    np.testing.assert_allclose(a, g["profile"], rtol=0, atol=5e-9)


def test_hydrogen_no_nan(oracle_lib):
    """test/line_absorption.jl:41-47: no NaNs for ne = 1.1e16 over 3800-4200 A (MHD on)."""
    from korg_gb300.data import stark_profiles, default_partition_funcs
    from korg_gb300.species import parse_species
    from korg_gb300.wavelengths import Wavelengths
    w = Wavelengths((3800, 4200))
    a = np.zeros(len(w))
    U = default_partition_funcs()[parse_species("H I")](np.log(9000.0))
    oracle_lib.hydrogen_line_absorption(a, w.all_wls, 9000.0, 1.1e16, 1.0, 0.0, U, 0.0, 15e-7, True,
                                        stark_profiles())
    assert np.all(np.isfinite(a)) and a.max() > 0


def test_brackett_peak_centred(oracle_lib):
    """test/line_absorption.jl:50-73: the Brackett-gamma profile peaks within window/500 of its
    centre."""
    import ctypes as C
    n_upper, n_lower = 7, 4
    E = 13.598287264 * (1 / n_lower ** 2 - 1 / n_upper ** 2)
    wl0 = 4.135667696e-15 * 2.99792458e10 / E
    grid = np.zeros(201)
    vals = np.zeros(201)
    win = oracle_lib.lib().ko_brackett_profile(7, wl0, 8000.0, 1e14, 1e5, 0.0, np.inf,
                                               grid.ctypes.data_as(C.POINTER(C.c_double)),
                                               vals.ctypes.data_as(C.POINTER(C.c_double)))
    test = np.linspace(wl0 - win / 10, wl0 + win / 10, 10001)
    itp = np.interp(test, grid, vals)
    assert abs(test[np.argmax(itp)] - wl0) < win / 500


def test_rt_scheme_agreement(oracle_lib):
    """RadiativeTransfer: the exponential-integral flux and the mu-quadrature linear schemes
    agree (the reference compares schemes at rtol 0.16, test/transfer.jl:83-113)."""
    from korg_gb300 import synthetic
    inp = synthetic.prepare(synthetic.config0(n_lines=50))
    L = len(inp.T)
    wl = inp.wls.all_wls[::500]
    alpha = np.ascontiguousarray(np.interp(wl, inp.cntm_knots, inp.cntm_vals[0])[:, None] *
                                 (inp.cntm_vals[:, 0] / inp.cntm_vals[0, 0])[None, :])
    S = np.array([[oracle_lib.blackbody(T, w) for T in inp.T] for w in wl])
    F = oracle_lib.rt_flux_expint(alpha, S, inp.tau_ref, inp.alpha_ref_cntm)
    mu, wts = np.polynomial.legendre.leggauss(20)
    mu, wts = mu / 2 + 0.5, wts / 2
    z = np.linspace(0, -1e8, L)
    for I_scheme in (0, 1):
        F2 = oracle_lib.rt_general(alpha, S, z, False, inp.tau_ref, inp.alpha_ref_cntm, mu, wts, False, 0, I_scheme)
        np.testing.assert_allclose(F2, F, rtol=0.16)


def test_mu_grid_weights():
    """test/transfer.jl:115-141: trapezoid weights of an explicit mu grid sum to 1."""
    for mus in ([0, 0.2, 1.0], np.arange(0, 1.0001, 0.5)):
        mus = np.asarray(mus, float)
        d = np.diff(mus)
        w = 0.5 * np.concatenate([[d[0]], d[:-1] + d[1:], [d[-1]]])
        assert abs(w.sum() - 1) < 1e-12


def test_line_absorption_threads_agree(oracle_lib):
    """The chunked-threads mode (line_absorption.jl:62-127) only reorders additions."""
    from korg_gb300 import synthetic
    inp = synthetic.prepare(synthetic.config0(n_lines=200))
    L, nwl = len(inp.T), len(inp.wls)
    outs = []
    for nt in (1, 4):
        a = np.zeros((nwl, L))
        oracle_lib.line_absorption(a, inp.linelist, inp.wls.all_wls, inp.T, inp.ne, inp.n_eff_vdW, inp.xi,
                                   inp.n_div_U, inp.cntm_knots, inp.cntm_vals, nthreads=nt)
        outs.append(a)
    np.testing.assert_allclose(outs[0], outs[1], rtol=1e-13, atol=0)


def test_rt_spherical_limits(oracle_lib):
    """A shell atmosphere of very large radius transfers like the plane-parallel one, and seeding
    the outward rays from inward rays changes the flux only slightly (RadiativeTransfer.jl:196:
    'the effect is immeasurable')."""
    from korg_gb300 import synthetic
    inp = synthetic.prepare(synthetic.config0(n_lines=20))
    L = len(inp.T)
    wl = inp.wls.all_wls[::2000]
    alpha = np.ascontiguousarray(np.interp(wl, inp.cntm_knots, inp.cntm_vals[0])[:, None] *
                                 (inp.cntm_vals[:, 0] / inp.cntm_vals[0, 0])[None, :])
    S = np.array([[oracle_lib.blackbody(T, w) for T in inp.T] for w in wl])
    mu, wts = np.polynomial.legendre.leggauss(10)
    mu, wts = mu / 2 + 0.5, wts / 2
    z = np.linspace(0, -1e8, L)
    Fp = oracle_lib.rt_general(alpha, S, z, False, inp.tau_ref, inp.alpha_ref_cntm, mu, wts, False, 0, 0)
    Fs = oracle_lib.rt_general(alpha, S, 1e16 + z, True, inp.tau_ref, inp.alpha_ref_cntm, mu, wts, False, 0, 0)
    np.testing.assert_allclose(Fs, Fp, rtol=1e-6)
    F1 = oracle_lib.rt_general(alpha, S, 7e10 + z, True, inp.tau_ref, inp.alpha_ref_cntm, mu, wts, False, 0, 0)
    F2 = oracle_lib.rt_general(alpha, S, 7e10 + z, True, inp.tau_ref, inp.alpha_ref_cntm, mu, wts, True, 0, 0)
    np.testing.assert_allclose(F2, F1, rtol=1e-3)
