"""Chemical equilibrium on the GPU (korg_chemical_equilibrium) against the FP64 restatement of
Korg's statmech.jl (oracle/statmech_oracle.py) and against the reference's property tests
(test/statmech.jl), through the C ABI (needs a GB300).

Parity bar: the device and the restatement run the same Newton iteration from the same start, so
they reach the same root; densities agree to 1e-9 relative (1e-6 for species below 1e-30 of
n_tot, whose logarithms carry the same absolute error)."""
import warnings

import numpy as np
import pytest

import chem_checks as cc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def tabs():
    from korg_gb300 import data
    return data.ionization_energies(), data.default_partition_funcs(), data.default_log_equilibrium_constants()


def _device(ctx, T, nt, ne, ab):
    from korg_gb300.statmech import default_equilibrium_tables, solve_layers
    dens, status, info = solve_layers(T, nt, ne, ab, ctx=ctx)
    return dens, status, info, default_equilibrium_tables().species


def _as_dict(dens_row, species):
    return {s: float(dens_row[k]) for k, s in enumerate(species) if s is not None}


def _oracle(tabs, T, nt, ne, ab):
    import statmech_oracle as so
    chi, pf, K = tabs
    return so.chemical_equilibrium(T, nt, ne, ab, chi, pf, K, electron_number_density_warn_threshold=np.inf)


def _compare(dev_ne, dev_nd, ora_ne, ora_nd, nt):
    worst = abs(dev_ne / ora_ne - 1)
    for s, v in ora_nd.items():
        d = dev_nd[s]
        if v == 0 and d == 0:
            continue
        tol = 1e-9 if v > 1e-30 * nt else 1e-6
        err = abs(d - v) / max(abs(v), abs(d))
        worst = max(worst, err / tol * 1e-9)
        assert err <= tol, (str(s), d, v)
    return worst


@pytest.mark.parametrize("which", ["sun", "s5000", "s6000", "solar", "M dwarf", "cool metal-poor dwarf",
                                   "low-Z extreme cool dense dwarf"])
def test_device_matches_oracle(ctx, tabs, which):
    atms = {a[0]: a for a in cc.marcs_atmospheres() + cc.representative_atmospheres()}
    _, T, nt, ne, ab = atms[which]
    dens, status, info, species = _device(ctx, T, nt, ne, ab)
    assert np.all(status == 0)
    worst = 0.0
    for l in range(0, len(T), 5):
        o_ne, o_nd = _oracle(tabs, T[l], nt[l], ne[l], ab)
        worst = max(worst, _compare(dens[l, 0], _as_dict(dens[l], species), o_ne, o_nd, nt[l]))
    print(f"{which}: worst scaled rel err {worst:.2e}; Newton iterations per layer "
          f"{info[:, 0].min():.0f}-{info[:, 0].max():.0f}, solves up to {info[:, 1].max():.0f}")


def test_properties_every_layer(ctx):
    """check_solution (test/statmech.jl:103-168) on every layer of the eight representative stars
    and the three MARCS atmospheres, all solved in one batched call."""
    from korg_gb300.statmech import Hminus_nK, default_equilibrium_tables, solve_layers
    atms = cc.representative_atmospheres() + cc.marcs_atmospheres()
    T = np.concatenate([a[1] for a in atms])
    nt = np.concatenate([a[2] for a in atms])
    ne = np.concatenate([a[3] for a in atms])
    ab = np.stack([a[4] for a in atms])
    atm = np.concatenate([np.full(len(a[1]), k, np.int32) for k, a in enumerate(atms)])
    dens, status, _ = solve_layers(T, nt, ne, ab, atm=atm, ctx=ctx)
    assert np.all(status == 0)
    species = default_equilibrium_tables().species
    for l in range(len(T)):
        bad = cc.check_solution(T[l], dens[l, 0], _as_dict(dens[l], species), nt[l], ab[atm[l]], Hminus_nK)
        assert bad == [], (atms[atm[l]][0], l, bad)


def test_batched_equals_separate(ctx):
    from korg_gb300.statmech import solve_layers
    atms = cc.marcs_atmospheres()
    sep = [solve_layers(a[1], a[2], a[3], a[4], ctx=ctx)[0] for a in atms]
    T = np.concatenate([a[1] for a in atms])
    atm = np.concatenate([np.full(len(a[1]), k, np.int32) for k, a in enumerate(atms)])
    bat = solve_layers(T, np.concatenate([a[2] for a in atms]), np.concatenate([a[3] for a in atms]),
                       np.stack([a[4] for a in atms]), atm=atm, ctx=ctx)[0]
    assert np.array_equal(bat, np.concatenate(sep))


def test_deterministic(ctx):
    """test/statmech.jl:76-86: bitwise-identical reruns."""
    ab = cc.absolute_abundances(cc.format_A_X())
    a = _device(ctx, np.full(8, 3000.0), 1e16, 1e10, ab)[0]
    b = _device(ctx, np.full(8, 3000.0), 1e16, 1e10, ab)[0]
    assert np.array_equal(a, b)
    assert np.all(a == a[0])


def test_insensitive_to_ne_guess(ctx):
    """test/statmech.jl:61-74: rtol 1e-8 on n_e, 1e-7 on every density."""
    ab = cc.absolute_abundances(cc.format_A_X())
    dens = _device(ctx, np.full(5, 3500.0), 1e16, np.array([1e6, 1e9, 1e11, 1e13, 1e15]), ab)[0]
    assert np.all(np.abs(dens[1:, 0] - dens[0, 0]) <= 1e-8 * dens[0, 0])
    assert np.all(np.abs(dens[1:] - dens[0]) <= 1e-7 * np.maximum(np.abs(dens[1:]), np.abs(dens[0])))


def test_CO_ratio_sweep(ctx, tabs):
    """test/statmech.jl:170-197 (T = 1500 K, n_tot = 1e17, the continuation regime), each ratio
    also against the restatement."""
    from korg_gb300.statmech import Hminus_nK, solve_layers
    A0 = cc.format_A_X()
    abs_ = []
    for d in cc.CO_LOG_RATIOS:
        A = A0.copy()
        A[5] = A[7] + d
        abs_.append(cc.absolute_abundances(A))
    n = len(abs_)
    dens, status, info = solve_layers(np.full(n, 1500.0), 1e17, 1e9, np.stack(abs_), atm=np.arange(n, dtype=np.int32),
                                      ctx=ctx)
    assert np.all(status == 0)
    from korg_gb300.statmech import default_equilibrium_tables
    species = default_equilibrium_tables().species
    for k in range(n):
        nd = _as_dict(dens[k], species)
        assert cc.check_solution(1500.0, dens[k, 0], nd, 1e17, abs_[k], Hminus_nK) == []
        assert cc.co_bound_ok(nd)
        o_ne, o_nd = _oracle(tabs, 1500.0, 1e17, 1e9, abs_[k])
        _compare(dens[k, 0], nd, o_ne, o_nd, 1e17)
    print("C/O sweep solves per ratio:", info[:, 1].astype(int).tolist())


def test_reference_interface(ctx, tabs):
    """chemical_equilibrium(T, n_tot, ne, abundances, ...) with the reference's signature: scalar
    call returns (ne, {Species: n}) equal to the batched solve."""
    from korg_gb300.statmech import chemical_equilibrium
    from korg_gb300.species import parse_species
    chi, pf, K = tabs
    ab = cc.absolute_abundances(cc.format_A_X())
    ne, nd = chemical_equilibrium(5000.0, 1e16, 1e12, ab, chi, pf, K, electron_number_density_warn_threshold=np.inf,
                                  ctx=ctx)
    o_ne, o_nd = _oracle(tabs, 5000.0, 1e16, 1e12, ab)
    _compare(ne, nd, o_ne, o_nd, 1e16)
    assert nd[parse_species("H III")] == 0.0
    with pytest.warns(UserWarning, match="Electron number density differs"):
        chemical_equilibrium(5700.0, 1e15, 1.2e12, ab, ctx=ctx)


def test_bad_inputs(ctx):
    from korg_gb300._lib import KorgError
    from korg_gb300.statmech import solve_layers
    ab = cc.absolute_abundances(cc.format_A_X())
    with pytest.raises(KorgError):
        solve_layers([2e5], 1e16, 1e10, ab, ctx=ctx)  # above the partition functions' range
    with pytest.raises(KorgError):
        solve_layers([5000.0], 1e10, 1e12, ab, ctx=ctx)  # n_e > n_tot
    bad = ab.copy()
    bad[40] = 0.0
    with pytest.raises(KorgError):
        solve_layers([5000.0], 1e16, 1e12, bad, ctx=ctx)
    with pytest.raises(KorgError):
        solve_layers([5000.0, 5000.0], 1e16, 1e12, ab, atm=np.array([0, 1], np.int32), ctx=ctx)


def test_synthesize_with_device_chemistry(ctx, tabs):
    """prepare_synthesis(chemistry="gpu") takes every layer's number densities from the device
    solve, starting from the atmosphere's n_e, as src/synthesize.jl:207-219 does."""
    from korg_gb300 import standin, synthetic
    from korg_gb300.api import prepare_synthesis, synthesize_prepared
    from korg_gb300.species import parse_species
    atm, A_X = standin.synthetic_atmosphere(5777.0, 4.44, 0.0)
    ll = synthetic.synthetic_linelist(300, 5000.0, 5020.0, seed=3)
    with warnings.catch_warnings():  # the grey atmosphere's n_e is not Korg's: the n_e warning may fire
        warnings.simplefilter("ignore")
        inp = prepare_synthesis(atm, ll, A_X, (5000, 5020), chemistry="gpu", continuum="gpu", ctx=ctx)
    ab = cc.absolute_abundances(A_X)
    for l in (0, 20, 55):
        o_ne, o_nd = _oracle(tabs, atm.T[l], atm.n_tot[l], atm.ne[l], ab)
        assert abs(inp.ne[l] / o_ne - 1) <= 1e-9
        for s in ("H I", "Fe I", "Fe II", "CO", "H2O", "H-"):
            sp = parse_species(s)
            assert abs(inp.number_densities[sp][l] / o_nd[sp] - 1) <= 1e-9, s
    res = synthesize_prepared(inp, precision="fp64", ctx=ctx)
    assert np.all(np.isfinite(res.flux)) and np.all(res.flux > 0)


def _cotangent(dens_row, nt, seed):
    """Random cotangent r_s / n_s on the species above 1e-30 n_tot (each weighs O(1))."""
    rng = np.random.default_rng(seed)
    r = rng.normal(size=dens_row.shape)
    return np.where(dens_row > 1e-30 * nt, r / np.maximum(dens_row, 1e-300), 0.0)


@pytest.mark.parametrize("which,layers", [("sun", (0, 20, 40, 55)), ("M dwarf", (10,)),
                                          ("cool metal-poor dwarf", (25,))])
def test_vjp_matches_restatement(ctx, tabs, which, layers):
    """Reverse mode (korg_chemical_equilibrium_vjp) against the restatement's implicit-function
    gradient at the device's solution (tests/test_statmech_oracle.py pins that gradient against
    differences of the whole solve): dL/dT, dL/dn_tot and dL/d(abundance) of H, C, O and Fe."""
    import statmech_oracle as so
    from korg_gb300.statmech import chemical_equilibrium_vjp, default_equilibrium_tables, solve_layers
    chi, pf, K = tabs
    atms = {a[0]: a for a in cc.marcs_atmospheres() + cc.representative_atmospheres()}
    _, T, nt, ne, ab = atms[which]
    dens, status, _ = solve_layers(T, nt, ne, ab, ctx=ctx)
    g = np.stack([_cotangent(dens[l], nt[l], l) for l in range(len(T))])
    dT, dnt, dab = chemical_equilibrium_vjp(T, nt, ne, ab, dens, g, ctx=ctx)
    species = default_equilibrium_tables().species
    worst = 0.0
    for l in layers:
        x = np.log10(np.concatenate([dens[l, 1:277:3], [dens[l, 0]]]))
        gd = {("ne" if sp is None else sp): g[l, k] for k, sp in enumerate(species)}
        oT, on, oab = so.chemical_equilibrium_vjp(T[l], nt[l], ab, x, gd, chi, pf, K, elements=(1, 6, 8, 26))
        pairs = [(dT[l], oT), (dnt[l], on)] + [(dab[l, Z - 1], oab[Z]) for Z in (1, 6, 8, 26)]
        scale = max(abs(v) for _, v in pairs)
        for got, want in pairs:
            err = abs(got - want) / max(abs(want), 1e-6 * scale)
            worst = max(worst, err)
            assert err <= 1e-6, (which, l, got, want)
    print(f"{which}: worst rel err of the reverse mode vs the restatement {worst:.1e}")


def test_vjp_matches_device_differences(ctx):
    """Reverse mode against central differences of the device solve itself (every layer at once:
    layers are independent), on the solar MARCS atmosphere."""
    from korg_gb300.statmech import chemical_equilibrium_vjp, solve_layers
    _, T, nt, ne, ab = cc.marcs_atmospheres()[0]
    dens, _, _ = solve_layers(T, nt, ne, ab, ctx=ctx)
    g = np.stack([_cotangent(dens[l], nt[l], 100 + l) for l in range(len(T))])
    dT, dnt, _ = chemical_equilibrium_vjp(T, nt, ne, ab, dens, g, ctx=ctx)
    loss = lambda d: np.sum(g * d, axis=1)
    h = 1e-5
    fT = (loss(solve_layers(T * (1 + h), nt, ne, ab, ctx=ctx)[0]) -
          loss(solve_layers(T * (1 - h), nt, ne, ab, ctx=ctx)[0])) / (2 * h * T)
    fn = (loss(solve_layers(T, nt * (1 + h), ne, ab, ctx=ctx)[0]) -
          loss(solve_layers(T, nt * (1 - h), ne, ab, ctx=ctx)[0])) / (2 * h * nt)
    eT = np.abs(dT - fT) / np.abs(fT)
    en = np.abs(dnt - fn) / np.abs(fn)
    print(f"device differences: median rel err T {np.median(eT):.1e} (max {eT.max():.1e}), "
          f"n_tot {np.median(en):.1e} (max {en.max():.1e})")
    assert np.median(eT) <= 1e-5 and np.median(en) <= 1e-5
    assert eT.max() <= 1e-3 and en.max() <= 1e-3  # the solve stops at |F| < 1e-8, not at rounding
