"""Molecular cross-sections (src/molecular_cross_sections.jl) on the GPU against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _co_lines(n=300, lo=15000.0, hi=15020.0):
    from korg_gb300 import synthetic
    return synthetic.synthetic_linelist(n, lo, hi, seed=4, species=["CO"], loggf=(-8.0, -2.0), E_lower=(0.0, 3.0),
                                        molecular=True)


def test_cross_section_table_matches_oracle(gpu_lib, oracle_lib):
    from korg_gb300.molecular import MolecularCrossSection
    from korg_gb300.data import default_partition_funcs
    from korg_gb300.wavelengths import Wavelengths
    ll = _co_lines()
    wls = Wavelengths((15000.0, 15020.0, 0.01))
    vm = np.array([0.0, 1.0, 2.5])
    lt = np.arange(3.0, 4.0 + 1e-9, 0.1)
    xs = MolecularCrossSection(ll, wls, vmic_vals=vm, log_temp_vals=lt, precision="fp64")
    tab = xs.table_numpy()  # (vmic, wl, T)
    T = 10.0 ** lt
    U = default_partition_funcs()[xs.species](np.log(T))
    L, nwl = len(T), len(wls)
    cut = 1e-32
    for v, vmic in enumerate(vm):
        a = np.zeros((nwl, L))
        ll0 = ll.subset(np.arange(len(ll)))
        ll0.species_idx = np.zeros(len(ll), np.int32)
        oracle_lib.line_absorption(a, ll0, wls.all_wls, T, np.zeros(L), np.full(L, np.nan), np.full(L, vmic * 1e5),
                                   (1 / cut / U)[None, :], np.zeros(1), np.ones((L, 1)), cutoff=1.0)
        np.testing.assert_allclose(tab[v], a * cut, rtol=1e-9, atol=0)
    assert np.all(tab >= 0) and tab.max() > 0


def test_cross_section_interpolation(gpu_lib):
    torch = pytest.importorskip("torch")
    from scipy.interpolate import RegularGridInterpolator
    from korg_gb300.molecular import MolecularCrossSection
    from korg_gb300.wavelengths import Wavelengths
    ll = _co_lines(200)
    xs = MolecularCrossSection(ll, Wavelengths((15000.0, 15020.0, 0.01)), vmic_vals=np.array([0.0, 1.0, 2.0, 3.0]),
                               log_temp_vals=np.arange(3.3, 4.0 + 1e-9, 0.05), precision="fp64")
    tab = xs.table_numpy()
    rgi = RegularGridInterpolator((xs.vmic_vals, xs.wls.all_wls, xs.log_temp_vals), tab, bounds_error=False,
                                  fill_value=0.0)
    rng = np.random.default_rng(0)
    L = 40
    T = 10 ** rng.uniform(3.25, 4.05, L)  # some layers outside the table: zero
    vmic = rng.uniform(0.0, 3.2, L)
    n = 10 ** rng.uniform(8, 12, L)
    wls = np.linspace(14999.0, 15021.0, 3001) * 1e-8  # some wavelengths outside: zero
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float64), device=dev)
    alpha = t(np.full((len(wls), L), 1e-9))
    xs.interpolate_into(alpha, t(wls), t(T), t(vmic), t(n))
    got = alpha.cpu().numpy()
    pts = np.stack(np.broadcast_arrays(vmic[None, :], wls[:, None], np.log10(T)[None, :]), axis=-1)
    want = 1e-9 + rgi(pts.reshape(-1, 3)).reshape(len(wls), L) * n[None, :]
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-20)
