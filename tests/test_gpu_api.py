"""The reference-signature Python entry points and the full-size optical workload against the
FP64 oracle (needs a GB300).

* ``korg_gb300.synthesize(atm, linelist, A_X, wavelengths)`` -- src/synthesize.jl:138-158 -- and
  ``korg_gb300.line_absorption_(alpha, linelist, wls, temps, ne, n_densities, partition_fns, xi,
  alpha_cntm)`` -- src/line_absorption.jl:33-34 -- called the way a user of the reference calls
  them, checked against the oracle at 1e-9 relative (plain FP64) and within the 1e-4 flux
  budget (mixed).
* The 300,000-line, 700,001-point optical synthesis computed on the GPU over its whole grid and
  compared with the oracle at every 50th point (the 0.5 A grid over the same range has exactly
  those wavelengths), so the window arithmetic, candidate tiers and tile bookkeeping at full size
  are checked, not only a small case.
"""
import os

import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def test_synthesize_reference_signature(ctx, oracle_lib):
    import korg_gb300
    from korg_gb300 import standin, synthetic
    from korg_gb300.data import stark_profiles
    w = synthetic.config0()
    atm, A_X = standin.synthetic_atmosphere(w.Teff, w.logg, w.m_H, w.L)
    res = korg_gb300.synthesize(atm, w.linelist, A_X, (5000, 5100), precision="fp64", ctx=ctx)
    with warnings.catch_warnings():  # synthesize's default: Korg's chemical equilibrium on the device
        warnings.simplefilter("ignore")
        inp = korg_gb300.prepare_synthesis(atm, w.linelist, A_X, (5000, 5100), continuum="gpu", chemistry="gpu",
                                           ctx=ctx)
    flux, cntm, _, _, ev = oracle_lib.synthesize(inp, inp.linelist, inp.linelist5, stark_profiles(),
                                                 inp.wls.all_wls, nthreads=NT)
    assert len(res.flux) == 10001 and np.array_equal(res.wavelengths, inp.wls.all_wls_angstrom)
    np.testing.assert_allclose(res.flux, flux, rtol=1e-9)
    np.testing.assert_allclose(res.cntm, cntm, rtol=1e-9)
    assert res.line_evals == ev
    mixed = korg_gb300.synthesize(atm, w.linelist, A_X, (5000, 5100), ctx=ctx)  # default: mixed precision
    assert np.max(np.abs(mixed.flux / flux - 1)) <= 1e-4


def test_line_absorption_reference_signature(ctx, oracle_lib):
    import korg_gb300
    from korg_gb300 import synthetic
    from korg_gb300.data import default_partition_funcs
    inp = synthetic.prepare(synthetic.config0())
    w = inp.wls.all_wls
    a0 = np.stack([np.interp(w, inp.cntm_knots, v) for v in inp.cntm_vals])  # (L, nwl), as Korg's alpha
    cntm = korg_gb300.ContinuumInterpolant(inp.cntm_knots, inp.cntm_vals)
    ref = np.ascontiguousarray(a0.T)
    ev_ref = oracle_lib.line_absorption(ref, inp.linelist, w, inp.T, inp.ne, inp.n_eff_vdW, inp.xi, inp.n_div_U,
                                        inp.cntm_knots, inp.cntm_vals, cutoff=inp.cutoff_threshold, nthreads=NT)
    for order in ("C", "F"):  # a Julia (column-major) matrix and a row-major numpy array
        alpha = np.array(a0, order=order)
        ev = korg_gb300.line_absorption_(alpha, inp.linelist, inp.wls, inp.T, inp.ne, inp.number_densities,
                                         default_partition_funcs(), inp.xi, cntm, precision="fp64", ctx=ctx)
        assert ev == ev_ref
        np.testing.assert_allclose(alpha, ref.T, rtol=1e-9, atol=0)
    # an empty line list returns without touching alpha (line_absorption.jl:35-37)
    alpha = a0.copy()
    assert korg_gb300.line_absorption_(alpha, inp.linelist.subset(np.zeros(0, np.int64)), inp.wls, inp.T, inp.ne,
                                       inp.number_densities, default_partition_funcs(), inp.xi, cntm, ctx=ctx) == 0
    assert np.array_equal(alpha, a0)
    # a species with no number density is a KeyError, as the reference's Dict lookup
    nd = dict(inp.number_densities)
    del nd[inp.linelist.species[0]]
    with pytest.raises(KeyError):
        korg_gb300.line_absorption_(a0.copy(), inp.linelist, inp.wls, inp.T, inp.ne, nd, default_partition_funcs(),
                                    inp.xi, cntm, ctx=ctx)


def test_precision_must_be_fp64_or_mixed(ctx):
    """Any precision other than KORG_FP64 / KORG_MIXED is KORG_EINVAL, not the FP64 form."""
    import ctypes as C
    from korg_gb300 import _lib, synthetic
    inp = synthetic.prepare(synthetic.config0(n_lines=50))
    keep = _lib.Keep()
    s = inp.struct(keep)
    l1, l5 = _lib.lines_struct(inp.linelist, keep), _lib.lines_struct(inp.linelist5, keep)
    nwl = len(inp.wls)
    flux, cntm = np.empty(nwl), np.empty(nwl)
    for prec in (2, -1):
        rc = ctx.lib.korg_synthesize(ctx.h, C.byref(s), C.byref(l1), C.byref(l5), _lib._p(keep.f64(inp.wls.all_wls)),
                                     nwl, prec, _lib._p(flux), _lib._p(cntm), None, None)
        assert rc == 1 and b"precision" in ctx.lib.korg_last_error(ctx.h)
        rc = ctx.lib.korg_line_absorption(ctx.h, _lib._p(np.zeros((nwl, len(inp.T)))),
                                          _lib._p(keep.f64(inp.wls.all_wls)), nwl, C.byref(l1), C.byref(s.layers),
                                          C.byref(s.cntm), 3e-4, prec, None)
        assert rc == 1
    tw, stage = C.c_int32(), C.c_int32()
    assert ctx.lib.korg_get_tile_config(ctx.h, 56, 2, C.byref(tw), C.byref(stage), None, None) == 1


def test_full_optical_fp64_against_oracle(ctx, oracle_lib):
    """300k lines + hydrogen lines, 56 layers, 700,001 points: the GPU's plain FP64 synthesis
    over the whole grid matches the oracle to 1e-9 at every 50th point; the mixed form stays
    within the 1e-4 flux budget there."""
    import copy
    from korg_gb300 import synthetic
    from korg_gb300.api import synthesize_prepared
    from korg_gb300.data import stark_profiles
    from korg_gb300.wavelengths import Wavelengths
    inp = synthetic.prepare(synthetic.config1())
    assert len(inp.wls) == 700_001 and len(inp.linelist) == 300_000
    r64 = synthesize_prepared(inp, precision="fp64", ctx=ctx)
    r32 = synthesize_prepared(inp, precision="mixed", ctx=ctx)
    sub = copy.copy(inp)
    sub.wls = Wavelengths((3000, 10000, 0.5))
    assert np.array_equal(sub.wls.all_wls, inp.wls.all_wls[::50])
    flux, cntm, _, _, _ = oracle_lib.synthesize(sub, sub.linelist, sub.linelist5, stark_profiles(), sub.wls.all_wls,
                                                nthreads=NT)
    np.testing.assert_allclose(r64.flux[::50], flux, rtol=1e-9)
    np.testing.assert_allclose(r64.cntm[::50], cntm, rtol=1e-9)
    err = np.max(np.abs(r32.flux[::50] / flux - 1))
    rms = np.sqrt(np.mean((r32.flux[::50] / r32.cntm[::50] - flux / cntm) ** 2))
    print(f"full optical, mixed vs oracle at 14,001 points: max rel flux err {err:.3e}, rectified RMS {rms:.3e}")
    assert err <= 1e-4
