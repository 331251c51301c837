"""Host-side pieces on CPU: wavelength grids, splines, HDF5 reader, line conversion rules, the
C ABI's exported symbols."""
import os
import re
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_wavelengths_correctly_rounded():
    from korg_gb300.wavelengths import Wavelengths
    w = Wavelengths((5000, 5100))
    assert len(w) == 10001
    c = Fraction(1e-8)
    for k in range(0, 10001, 97):
        assert float(Fraction(500000 + k, 100) * c) == w[k]
    w2 = Wavelengths([(3000, 3001), (4000, 4001, 0.5)])
    assert len(w2) == 101 + 3
    assert w2.searchsortedfirst(3000.5) == 50
    assert w2.searchsortedlast(3500) == 100  # in the gap: last point of the first range
    assert w2.searchsortedfirst(3500) == 101
    with pytest.raises(ValueError):
        Wavelengths([(5000, 5100), (4000, 4100)])


def test_cubic_spline_natural():
    from korg_gb300.cubic_spline import CubicSpline
    x = np.linspace(0, 3, 13)
    s = CubicSpline(x, np.sin(x))
    xs = np.linspace(0, 3, 101)
    assert np.max(np.abs(s(xs) - np.sin(xs))) < 2e-3
    assert s(x[5]) == pytest.approx(np.sin(x[5]), abs=1e-15)
    with pytest.raises(ValueError):
        s(3.5)
    assert CubicSpline(x, np.sin(x), extrapolate=True)(3.5) == pytest.approx(np.sin(3.0))


def test_hdf5_reader_golden_attributes():
    from korg_gb300 import hdf5lite
    # the reference checkout, if present: KORG_REFERENCE, else a sibling of this repository
    root = os.environ.get("KORG_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
    path = os.path.join(root, "test", "data", "lyman_absorption.h5")
    if not os.path.exists(path):
        pytest.skip("reference data not present (set KORG_REFERENCE to a Korg.jl checkout)")
    f = hdf5lite.File(path)
    g = np.load(os.path.join(ROOT, "tests", "golden", "lyman_absorption.npz"))
    np.testing.assert_array_equal(f.read("profile"), g["profile"])
    assert f["profile"].attrs["T"] == 9000.0


def test_line_conversion_rules():
    """Korg's Line constructor rules (src/linelist.jl:56-100)."""
    from korg_gb300.linelist import make_line, approximate_radiative_gamma
    l = make_line(5000.0, -1.0, "Fe I", 2.0, 1e8, 1e-6, -7.5)
    assert l[0] == 5000.0 * 1e-8 and l[6] == pytest.approx(10 ** -7.5) and l[7] == -1
    l = make_line(5000.0, -1.0, "Fe I", 2.0, 1e8, 1e-6, 0.0)
    assert l[6] == 0.0 and l[7] == -1
    l = make_line(5000.0, -1.0, "Fe I", 2.0, 1e8, 1e-6, 300.25)  # packed ABO
    assert l[6] == pytest.approx(300 * 5.29177210903e-9 ** 2) and l[7] == pytest.approx(0.25)
    l = make_line(5e-5, -1.0, "Fe I", 2.0, None, 1e-6, (1e-14, 0.3))
    assert l[4] == pytest.approx(approximate_radiative_gamma(5e-5, -1.0))
    l = make_line(5e-5, -1.0, "CO", 1.0, 1e8)  # molecules: no Stark / vdW
    assert l[5] == 0.0 and l[6] == 0.0


def test_alpha5000_linelist():
    from korg_gb300.linelist import alpha_5000_linelist
    ll = alpha_5000_linelist()
    assert len(ll) == 409 and ll.is_sorted()
    assert np.all(ll.wl > 4.97e-5) and np.all(ll.wl < 5.03e-5)


def test_filter_linelist():
    """src/synthesize.jl:331-350 against a naive filter (test/synthesize.jl:89-110)."""
    from korg_gb300 import synthetic
    from korg_gb300.linelist import filter_linelist
    from korg_gb300.wavelengths import Wavelengths
    ll = synthetic.synthetic_linelist(5000, 4000, 7000, seed=3)
    w = Wavelengths([(4500, 4600), (5000, 5050), (6000, 6100)])
    f = filter_linelist(ll, w, 10e-8)
    naive = np.zeros(len(ll), bool)
    for a, b in w.eachwindow():
        naive |= (ll.wl >= a - 10e-8) & (ll.wl <= b + 10e-8)
    np.testing.assert_array_equal(f.wl, ll.wl[naive])


def test_header_symbols_exported():
    """Every KORG_API function declared in include/korg_gb300.h is exported by the library."""
    import subprocess
    from korg_gb300 import _lib
    import build as korg_build
    hdr = open(os.path.join(ROOT, "include", "korg_gb300.h")).read()
    declared = set(re.findall(r"KORG_API\s+[\w\s\*]+?\b(korg_\w+)\s*\(", hdr))
    assert declared == set(_lib.exported_symbols())
    korg_build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r"\bT\s+(korg_\w+)", out.stdout))
    assert declared <= exported, declared - exported
    import ctypes
    ctypes.CDLL(_lib.LIB_PATH)  # loads without a GPU


def test_julia_binding_symbols_declared():
    """Every entry point the Julia binding ccalls is declared in include/korg_gb300.h (Julia is
    not in this image, so the binding is checked by its text)."""
    hdr = open(os.path.join(ROOT, "include", "korg_gb300.h")).read()
    declared = set(re.findall(r"KORG_API\s+[\w\s\*]+?\b(korg_\w+)\s*\(", hdr))
    jl = open(os.path.join(ROOT, "korg.jl_gb300", "julia", "KorgGPU.jl")).read()
    called = set(re.findall(r"ccall\(\(:(korg_\w+)\s*,", jl))
    assert {"korg_chemical_equilibrium", "korg_chemical_equilibrium_vjp", "korg_synthesize_vjp"} <= called
    assert called <= declared, called - declared


def test_no_oracle_in_product():
    """The product package never imports or links the oracle."""
    pkg = os.path.join(ROOT, "korg.jl_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h", ".jl")):
                src = open(os.path.join(dirpath, fn)).read()
                assert "korg_oracle" not in src and "import oracle" not in src, fn


def test_reference_signature_entry_points_are_functions():
    """korg_gb300.synthesize is the function synthesize(atm, linelist, A_X, wavelengths; ...) of
    src/synthesize.jl:138, not a module; the other mirrors of the reference API likewise."""
    import inspect
    import korg_gb300
    for name in ("synthesize", "line_absorption_", "hydrogen_line_absorption_", "radiative_transfer",
                 "prepare_synthesis", "synthesize_prepared", "synthesize_vjp"):
        f = getattr(korg_gb300, name)
        assert callable(f) and inspect.isfunction(f), name
    params = list(inspect.signature(korg_gb300.synthesize).parameters)
    assert params[:4] == ["atm", "linelist", "A_X", "wavelengths"]
    params = list(inspect.signature(korg_gb300.line_absorption_).parameters)
    assert params[:9] == ["alpha", "linelist", "wls", "temps", "ne", "n_densities", "partition_fns", "xi",
                          "alpha_cntm"]


def test_continuum_layer_inputs_vjp_is_the_chain_rule():
    """continuum.layer_inputs_vjp (the host chain rule behind the continuum's reverse mode) against
    central differences of sum(gbar * layer_inputs(T, ne, densities)): the temperatures through
    1/U(H I), 1/U(He I) and T itself, n_e, and each species' density, including the Peach ions,
    the other ions' charge sums and a neutral species that does not enter."""
    from korg_gb300 import continuum
    from korg_gb300.data import default_partition_funcs
    from korg_gb300.species import Species, parse_species
    rng = np.random.default_rng(2)
    L = 4
    T, ne = rng.uniform(4000, 7000, L), 10 ** rng.uniform(12, 14, L)
    names = ["H I", "H II", "He I", "H2", "He II", "C II", "Si II", "Mg II", "Fe II", "Fe III", "Ca II", "O I"]
    nd = {parse_species(n): 10 ** rng.uniform(8, 16, L) for n in names}
    nd[Species([1], -1)] = 10 ** rng.uniform(6, 9, L)
    pf = default_partition_funcs()
    gbar = {k: rng.normal(size=L) for k in continuum.INPUTS}

    def diff(Tp, Tm, nep, nem, ndp, ndm):
        dp, dm = continuum.layer_inputs(Tp, nep, ndp, pf), continuum.layer_inputs(Tm, nem, ndm, pf)
        return sum(float(np.sum(gbar[k] * (dp[k] - dm[k]))) for k in continuum.INPUTS)

    dT, dne, dn = continuum.layer_inputs_vjp(gbar, T, nd, pf)
    for l in range(L):
        h = 1e-5 * T[l]
        Tp, Tm = T.copy(), T.copy()
        Tp[l] += h
        Tm[l] -= h
        fd = diff(Tp, Tm, ne, ne, nd, nd) / (2 * h)
        assert abs(dT[l] - fd) <= 1e-6 * abs(fd), (l, dT[l], fd)
        h = 1e-6 * ne[l]
        nep, nem = ne.copy(), ne.copy()
        nep[l] += h
        nem[l] -= h
        fd = diff(T, T, nep, nem, nd, nd) / (2 * h)
        assert abs(dne[l] - fd) <= 1e-6 * abs(fd), (l, dne[l], fd)
        for s in nd:
            h = 0.5 * nd[s][l]  # the inputs are linear in the densities: any step is exact
            ndp, ndm = dict(nd), dict(nd)
            ndp[s], ndm[s] = nd[s].copy(), nd[s].copy()
            ndp[s][l] += h
            ndm[s][l] -= h
            fd = diff(T, T, ne, ne, ndp, ndm) / (2 * h)
            ad = np.asarray(dn.get(s, np.zeros(L)))[l]
            assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-12 * abs(gbar["n_Z1"][l]), (str(s), l, ad, fd)
    assert np.all(np.asarray(dn.get(parse_species("O I"), np.zeros(L))) == 0)


def test_abundance_vjp_is_the_chain_rule():
    """api.abundance_vjp, the last link of atmosphere_gradient: d/dA(X) of
    sum(gbar * 10^(A - 12) / sum(10^(A - 12))) against central differences."""
    from korg_gb300.api import abundance_vjp
    rng = np.random.default_rng(4)
    A = 12 + rng.uniform(-9, 0, 92)
    A[0] = 12.0
    gbar = rng.normal(size=92)
    f = lambda A: float(np.dot(gbar, 10.0 ** (A - 12) / np.sum(10.0 ** (A - 12))))
    ab = 10.0 ** (A - 12) / np.sum(10.0 ** (A - 12))
    dA = abundance_vjp(ab, gbar)
    def central(Z, h):
        Ap, Am = A.copy(), A.copy()
        Ap[Z - 1] += h
        Am[Z - 1] -= h
        return (f(Ap) - f(Am)) / (2 * h)

    for Z in (1, 2, 6, 26, 92):
        fd = (4 * central(Z, 5e-4) - central(Z, 1e-3)) / 3  # Richardson: truncation O(h^4)
        assert abs(dA[Z - 1] - fd) <= 1e-6 * abs(fd) + 1e-13, (Z, dA[Z - 1], fd)
