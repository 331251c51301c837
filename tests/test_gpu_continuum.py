"""Continuum absorption on the GPU (korg_continuum_absorption) against the FP64 restatement of
Korg's continuum module (oracle/continuum_oracle.py), through the C ABI (needs a GB300).

The restatement is pinned to the reference's continuum tests on the CPU
(tests/test_continuum_oracle.py); here the device kernel must equal it to 1e-12 relative, term by
term summed, over stellar layers from 3500 K to 12000 K and wavelengths from 1300 A to 20 um
(every term's range edge included)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def _layers(Teff, logg, m_H):
    from korg_gb300 import standin
    from korg_gb300.continuum import layer_inputs
    atm, A_X = standin.synthetic_atmosphere(Teff, logg, m_H, 56)
    ne, nd = standin.chemical_equilibrium(atm.T, atm.n_tot, A_X)
    return layer_inputs(atm.T, ne, nd), (atm.T, ne, nd)


@pytest.mark.parametrize("star", [(3500.0, 1.0, 0.0), (5800.0, 4.4, 0.0), (12000.0, 4.0, -1.0)])
def test_continuum_matches_restatement(ctx, star):
    import continuum_oracle as co
    from korg_gb300.continuum import continuum_absorption
    from korg_gb300.wavelengths import Wavelengths
    d, (T, ne, nd) = _layers(*star)
    edges = np.array([1823.0, 5063.0, 7000.0, 9113.0, 14588.0, 151878.0, 151890.0]) * 1e-8
    wls = np.unique(np.concatenate([Wavelengths((1300, 200_000, 7.0)).all_wls, edges, edges * (1 + 1e-12),
                                    edges * (1 - 1e-12)]))
    got = continuum_absorption(wls, T, ne, nd, ctx=ctx)
    nu = 2.99792458e10 / wls
    for l in range(len(T)):
        ref = co.total_continuum_absorption(nu, T[l], d["ne"][l], {k: v[l] for k, v in d.items()})
        np.testing.assert_allclose(got[l], ref, rtol=1e-12, atol=0, err_msg=f"layer {l}")
    assert np.all(got > 0)


def test_total_continuum_absorption_reference_signature(ctx):
    """total_continuum_absorption(nus, T, ne, number_densities, partition_funcs) for one layer:
    sorted frequencies in, alpha at those frequencies out; unsorted frequencies are an error."""
    import continuum_oracle as co
    from korg_gb300.continuum import total_continuum_absorption
    d, (T, ne, nd) = _layers(5800.0, 4.4, 0.0)
    l = 40
    nus = np.sort(2.99792458e10 / np.linspace(3000e-8, 20000e-8, 501))
    got = total_continuum_absorption(nus, T[l], ne[l], {k: v[l] for k, v in nd.items()}, ctx=ctx)
    ref = co.total_continuum_absorption(nus, T[l], d["ne"][l], {k: v[l] for k, v in d.items()})
    np.testing.assert_allclose(got, ref, rtol=1e-12)
    with pytest.raises(ValueError):
        total_continuum_absorption(nus[::-1], T[l], ne[l], {k: v[l] for k, v in nd.items()}, ctx=ctx)


def test_synthesis_with_device_continuum(ctx, oracle_lib):
    """synthesize with the device continuum: the plain FP64 hot path still matches the oracle fed
    with the same continuum interpolants."""
    import os
    from korg_gb300 import synthetic
    from korg_gb300.api import synthesize_prepared
    from korg_gb300.data import stark_profiles
    inp = synthetic.prepare(synthetic.config0(n_lines=500), continuum="gpu", ctx=ctx)
    flux, cntm, _, _, _ = oracle_lib.synthesize(inp, inp.linelist, inp.linelist5, stark_profiles(),
                                                inp.wls.all_wls, nthreads=os.cpu_count() or 1)
    res = synthesize_prepared(inp, precision="fp64", ctx=ctx)
    np.testing.assert_allclose(res.flux, flux, rtol=1e-9)
    np.testing.assert_allclose(res.cntm, cntm, rtol=1e-9)
