"""Every radiative-transfer scheme (RadiativeTransfer.jl:62-371) on the GPU against the FP64
oracle: planar and spherical rays, inward rays, anchored and Bezier optical depth, linear,
linear-flux-only, Bezier and exponential-integral formal solutions."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def column(oracle_lib):
    from korg_gb300 import synthetic
    inp = synthetic.prepare(synthetic.config0(n_lines=50))
    L = len(inp.T)
    wl = inp.wls.all_wls[::97]
    rng = np.random.default_rng(2)
    base = np.interp(wl, inp.cntm_knots, inp.cntm_vals[0])[:, None] * (inp.cntm_vals[:, 0] / inp.cntm_vals[0, 0])[None, :]
    alpha = np.ascontiguousarray(base * (1 + rng.uniform(0, 3, base.shape)))  # lines of random strength
    S = np.array([[oracle_lib.blackbody(T, w) for T in inp.T] for w in wl])
    return inp, alpha, S


CASES = ([(False, t, i, False) for t in (0, 1) for i in (0, 1, 2)] + [(False, 0, 3, False)] +
         [(True, t, i, inw) for t in (0, 1) for i in (0, 1, 2) for inw in (False, True)])


@pytest.mark.parametrize("spherical,tau_scheme,I_scheme,inward", CASES)
def test_rt_general_matches_oracle(gpu_lib, oracle_lib, column, spherical, tau_scheme, I_scheme, inward):
    inp, alpha, S = column
    L = len(inp.T)
    nwl = alpha.shape[0]
    z = np.linspace(0, -1e8, L)
    spatial = 7e10 + z if spherical else z
    mu, w = np.polynomial.legendre.leggauss(12)
    mu, w = mu / 2 + 0.5, w / 2
    ref = oracle_lib.rt_general(alpha, S, spatial, spherical, inp.tau_ref, inp.alpha_ref_cntm, mu, w, inward,
                                tau_scheme, I_scheme)
    ctx = gpu_lib.default_context()
    F = np.empty(nwl)
    Isurf = np.empty((len(mu), nwl))
    dp = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(C.POINTER(C.c_double))
    keep = [alpha, S, spatial, inp.tau_ref, inp.alpha_ref_cntm, mu, w]
    ctx.check(ctx.lib.korg_radiative_transfer_general(ctx.h, dp(alpha), dp(S), L, nwl, dp(spatial), int(spherical),
                                                      dp(inp.tau_ref), dp(inp.alpha_ref_cntm), dp(mu), dp(w), len(mu),
                                                      int(inward), tau_scheme, I_scheme, dp(F), dp(Isurf)))
    # The Bezier coefficients (2 + d^2 - 2d - 2e^-d)/d^2 ... cancel to a few digits for small
    # optical-depth steps, and spherical Bezier tau differences nearly equal path lengths near
    # the tangent point: there, one-ulp differences between CUDA's and the C library's exp or
    # the compilers' FMA contraction show up at 1e-8..1e-5 (the reference, with Julia's exp,
    # sits as far from either).  The other schemes are well conditioned and match to 1e-9.
    ill = I_scheme == 2 or (spherical and tau_scheme == 1)
    np.testing.assert_allclose(F, ref, rtol=2e-5 if ill else 1e-9, atol=0)
    np.testing.assert_allclose(F, 2 * np.pi * (Isurf.T @ (w * mu)), rtol=1e-12)
    del keep


def test_rt_general_rejects_bad_schemes(gpu_lib, column):
    inp, alpha, S = column
    L = len(inp.T)
    ctx = gpu_lib.default_context()
    dp = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(C.POINTER(C.c_double))
    F = np.empty(alpha.shape[0])
    mu, w = np.array([1.0]), np.array([1.0])
    z = np.linspace(0, -1e8, L)
    for tau_s, I_s, sph in ((2, 0, 0), (0, 4, 0), (1, 3, 0), (0, 3, 1)):
        rc = ctx.lib.korg_radiative_transfer_general(ctx.h, dp(alpha), dp(S), L, alpha.shape[0], dp(z), sph,
                                                     dp(inp.tau_ref), dp(inp.alpha_ref_cntm), dp(mu), dp(w), 1, 0,
                                                     tau_s, I_s, dp(F), None)
        assert rc == 1  # KORG_EINVAL


def test_python_radiative_transfer_dispatch(gpu_lib, column):
    """radiative_transfer(atm, ...) picks the exponential-integral path for the planar default
    and the general kernel otherwise; with anchored tau every formal solution lands within the
    reference's 16% of it (Bezier tau integrates over the geometric heights, which this
    synthetic column does not have consistently with tau_ref, so it is only run)."""
    from korg_gb300.api import radiative_transfer

    inp, alpha, S = column

    class Atm:
        tau_ref = inp.tau_ref
        z = np.linspace(0, -1e8, len(inp.T))

    F0, I0, mu0, w0 = radiative_transfer(Atm, alpha.T.copy(order="F"), S.T.copy(order="F"), 20,
                                         alpha_ref=inp.alpha_ref_cntm)
    assert len(mu0) == 1
    for tau_scheme in ("anchored", "bezier"):
        for I_scheme in ("linear", "linear_flux_only", "bezier"):
            F, I, mu, w = radiative_transfer(Atm, alpha.T.copy(order="F"), S.T.copy(order="F"), 20,
                                             alpha_ref=inp.alpha_ref_cntm, tau_scheme=tau_scheme, I_scheme=I_scheme)
            n_mu = 1 if (tau_scheme, I_scheme) == ("anchored", "linear_flux_only") else 20  # :81-84
            assert I.shape == (n_mu, alpha.shape[0])
            assert np.all(np.isfinite(F)) and np.all(F > 0)
            if tau_scheme == "anchored":
                np.testing.assert_allclose(F, F0, rtol=0.16)
