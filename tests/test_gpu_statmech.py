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


def test_atmosphere_gradient_matches_differences(ctx):
    """The loss gradient with respect to A(X), layer T and n_tot through the hot path, the device
    continuum and the device chemical equilibrium (atmosphere_gradient) against central
    differences of the whole pipeline: prepare_synthesis(chemistry="gpu", continuum="gpu"), the
    FP64 synthesis and the rectified-flux loss."""
    import copy
    from korg_gb300 import standin, synthetic
    from korg_gb300.api import atmosphere_gradient, prepare_synthesis, synthesize_prepared, synthesize_vjp
    ctx.ensure_stark()
    atm, A_X = standin.synthetic_atmosphere(5000.0, 4.0, 0.0)
    ll = synthetic.synthetic_linelist(400, 5001.0, 5029.0, seed=11)

    import statmech_oracle as so
    from korg_gb300 import data
    from korg_gb300.statmech import chemical_equilibrium as device_chemistry
    tabs = data.ionization_energies(), data.default_partition_funcs(), data.default_log_equilibrium_constants()

    def polished(T, n_tot, ne_model, ab):
        """The device solve, then two Newton steps of the restatement per layer: the differences of
        the pipeline then see the root to rounding, not the solver's 1e-8 residual tolerance."""
        ne, nd = device_chemistry(T, n_tot, ne_model, ab, ctx=ctx)
        keys = [k for k in nd if k.charge == 0 and len(k.atoms) == 1]
        out = {k: np.empty(len(T)) for k in nd}
        out_ne = np.empty(len(T))
        for l in range(len(T)):
            x = np.log10(np.array([nd[so._species_ctor(tabs[1])(Z, 0)][l] for Z in range(1, 93)] + [ne[l]]))
            r = so.Residuals(T[l], n_tot[l], ab, *tabs, 0.0)
            for _ in range(2):
                F, J = r(x)
                x = x - np.linalg.solve(J, F)
            d = so.densities_from_x(x, T[l], *tabs)
            out_ne[l] = d["ne"]
            for k in out:
                out[k][l] = d[k]
        assert keys
        return out_ne, out

    def prep(a, A, chemistry="gpu"):
        # cutoff 1e-12 and 1000 A hydrogen windows: every line window spans the grid, so no window
        # edge (a step in the loss, not part of its derivative) moves under the perturbations;
        # the hydrogen lines' centres shift with n_e, and H beta's 150 A window ends at 5011 A
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            return prepare_synthesis(a, ll, A, (5000, 5030), chemistry=chemistry, continuum="gpu",
                                     line_cutoff_threshold=1e-12, hydrogen_line_window_size=1000, ctx=ctx)

    inp = prep(atm, A_X)
    base = synthesize_prepared(inp, precision="fp64", ctx=ctx)
    obs = base.flux / base.cntm * (1 + np.random.default_rng(3).normal(0, 0.01, len(base.flux)))

    def terms_at(a, A):
        """The loss's per-wavelength terms (flux/cntm - obs)^2."""
        r = synthesize_prepared(prep(a, A, polished), precision="fp64", ctx=ctx)
        return (r.flux / r.cntm - obs) ** 2

    def differences(at):
        """Per-wavelength central differences of the loss terms at steps h and h/2 (``at(s)`` gives
        the terms at s steps of h)."""
        tp, tm, hp, hm = at(1.0), at(-1.0), at(0.5), at(-0.5)
        return (tp - tm) / 2, hp - hm

    perturbations = []
    for Z in (1, 2, 6, 26):  # H, He, C, Fe
        def at(s, Z=Z, h=1e-4):
            A = A_X.copy()
            A[Z - 1] += s * h
            return terms_at(atm, A)
        perturbations.append((f"A({Z})", ("A_X", Z - 1), 1e-4, differences(at)))
    for field, l in (("T", 15), ("T", 35), ("n_tot", 30)):
        h = 1e-5 * getattr(atm, field)[l]
        def at(s, field=field, l=l, h=h):
            a = copy.deepcopy(atm)
            getattr(a, field)[l] += s * h
            return terms_at(a, A_X)
        perturbations.append((f"{field}[{l}]", (field, l), h, differences(at)))

    # Korg's E2(x) (RadiativeTransfer.jl:408-497) is piecewise and jumps at its segment ends (by 1%
    # at x = 1.1), so the flux steps where a layer's optical depth crosses one: a step inside the
    # difference interval shows as disagreement between the h and h/2 differences of that
    # wavelength's term (a smooth term's differ by O(h^2)).  Those wavelengths get weight 0 in the
    # loss and in its gradient.
    keep = np.ones(len(obs), bool)
    for _, _, _, (d1, d2) in perturbations:
        keep &= np.abs(d1 - d2) <= 1e-3 * np.abs(d2) + 1e-9 * np.max(np.abs(d2))
    print(f"{np.count_nonzero(~keep)} of {len(keep)} wavelengths step within a difference interval")
    assert np.count_nonzero(keep) >= 0.95 * len(keep)
    w = keep * 2 * (base.flux / base.cntm - obs)
    dF, dC = w / base.cntm, -w * base.flux / base.cntm ** 2
    ag = atmosphere_gradient(inp, synthesize_vjp(inp, dF, dC, precision="fp64", ctx=ctx), ctx=ctx)

    checks = [(name, ag[key][i], np.sum(keep * d1) / h) for name, (key, i), h, (d1, _) in perturbations]
    scale = max(abs(fd) for _, _, fd in checks)
    for name, ad, fd in checks:
        print(f"{name}: adjoint {ad:.6e}, differences {fd:.6e}")
    for name, ad, fd in checks:
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-7 * scale, (name, ad, fd)
