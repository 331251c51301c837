"""Reverse mode (korg_synthesize_vjp) against central finite differences.

Loss: sum of squared rectified-flux residuals against a perturbed synthetic "observation".
The plain FP64 gradient is checked against central differences of the GPU FP64 forward (many
parameters) and of the FP64 oracle (a few, pinning the reference restatement); the mixed-precision
gradient against the FP64 gradient.
"""
import copy
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = gpu_lib.Context(0)
    c.ensure_stark()
    yield c
    c.close()


def _case(n_lines=600, wl=(5000.0, 5030.0), seed=7):
    from korg_gb300 import synthetic
    w = synthetic.config0(seed=seed, n_lines=n_lines)
    w.wavelengths = wl
    w.linelist = synthetic.synthetic_linelist(n_lines, wl[0] + 1, wl[1] - 1, seed=seed)
    return synthetic.prepare(w)


def _obs(inp, ctx):
    """A seeded perturbed synthetic observation: log gf shifted by N(0, 0.1) dex."""
    from korg_gb300.api import synthesize_prepared
    rng = np.random.default_rng(1)
    o = copy.copy(inp)
    o.linelist = copy.copy(inp.linelist)
    o.linelist.log_gf = inp.linelist.log_gf + rng.normal(0, 0.1, len(inp.linelist))
    r = synthesize_prepared(o, precision="fp64", ctx=ctx)
    return r.flux / r.cntm


def _loss(inp, obs, ctx, precision="fp64"):
    from korg_gb300.api import rectified_loss, synthesize_prepared
    r = synthesize_prepared(inp, precision=precision, ctx=ctx)
    return rectified_loss(r.flux, r.cntm, obs)[0]


def _perturbed(inp, field, idx, delta):
    c = copy.copy(inp)
    if field == "log_gf":
        c.linelist = copy.copy(inp.linelist)
        a = inp.linelist.log_gf.copy()
        a[idx] += delta
        c.linelist.log_gf = a
    else:
        a = getattr(inp, field).copy()
        a[idx] += delta
        setattr(c, field, a)
    return c


def _fd(inp, obs, ctx, field, idx, rel=1e-5, loss=None, noise=False):
    """Central difference; with noise=True also returns the rounding floor of the estimate
    (a few ulps of the loss over the step).  The relative step 1e-5 balances truncation (below
    3e-5 of the derivative for T, the most curved parameter) against the loss's round-off, which
    at a step of 1e-6 already reaches ~1e-4 of the n_e derivatives."""
    loss = loss or (lambda x: _loss(x, obs, ctx))
    v = (inp.linelist.log_gf if field == "log_gf" else getattr(inp, field))[idx]
    h = rel * max(abs(v), 1e-300) if field != "log_gf" else 1e-6
    lp, lm = loss(_perturbed(inp, field, idx, h)), loss(_perturbed(inp, field, idx, -h))
    d = (lp - lm) / (2 * h)
    return (d, 8e-16 * max(abs(lp), abs(lm)) / h) if noise else d


def _strong_lines(inp, k=4):
    return list(np.argsort(-(inp.linelist.log_gf - 0.5 * inp.linelist.E_lower))[:k])


PARAMS = [("T", 5), ("T", 25), ("T", 40), ("ne", 20), ("ne", 45), ("n_eff_vdW", 30), ("xi", 10), ("xi", 35),
          ("n_div_U", (0, 30)), ("n_div_U", (1, 12)), ("nH_I", 38), ("UH_I", 38), ("alpha_ref_cntm", 30),
          ("cntm_vals", (20, 3))]


def test_vjp_fp64_matches_central_differences(ctx):
    from korg_gb300.api import loss_and_gradient
    inp = _case()
    obs = _obs(inp, ctx)
    loss, g = loss_and_gradient(inp, obs, precision="fp64", ctx=ctx)
    assert loss > 0
    checks = PARAMS + [("log_gf", i) for i in _strong_lines(inp)]
    for field, idx in checks:
        fd, floor = _fd(inp, obs, ctx, field, idx, noise=True)
        ad = g[field][idx]
        assert abs(ad - fd) <= 1e-4 * abs(fd) + 1e-7 * np.max(np.abs(g[field])) + floor, (field, idx, ad, fd, floor)


def test_vjp_mixed_close_to_fp64(ctx):
    from korg_gb300.api import loss_and_gradient
    inp = _case(n_lines=1500, wl=(5000.0, 5060.0), seed=11)
    obs = _obs(inp, ctx)
    _, g64 = loss_and_gradient(inp, obs, precision="fp64", ctx=ctx)
    _, g32 = loss_and_gradient(inp, obs, precision="mixed", ctx=ctx)
    for k in ("T", "ne", "n_eff_vdW", "xi", "n_div_U", "log_gf", "cntm_vals", "alpha_ref_cntm", "nH_I", "nHe_I",
              "UH_I"):
        a, b = g32[k], g64[k]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err <= 2e-3, (k, err)


def test_vjp_mixed_close_to_fp64_brackett(ctx):
    """The mixed form's hydrogen-line reverse mode in the H band, where the Griem Brackett lines
    take its FP32 branch (FP32 profiles and profile derivatives on the 201-point grid)."""
    from korg_gb300.api import loss_and_gradient
    inp = _case(n_lines=200, wl=(16790.0, 16830.0), seed=5)
    obs = _obs(inp, ctx)
    _, g64 = loss_and_gradient(inp, obs, precision="fp64", ctx=ctx)
    _, g32 = loss_and_gradient(inp, obs, precision="mixed", ctx=ctx)
    for k in ("T", "ne", "xi", "nH_I", "UH_I"):
        err = np.max(np.abs(g32[k] - g64[k])) / np.max(np.abs(g64[k]))
        assert err <= 2e-3, (k, err)
    assert np.max(np.abs(g64["nH_I"])) > 0  # the Brackett lines are in reach


# (wavelength range, MHD, checks (input, layer, relative step)): the inputs and layers whose loss
# derivative stands well above the FP64 synthesis's rounding.  Deep layers, n(He I) (it only
# enters the MHD occupation probabilities) and, in the H band, n(H I) and U(H I) change the loss
# by less than its rounding lets a difference resolve at 1e-6.  n(H I) and U(H I) enter alpha_H
# linearly or as 1/U, so they take larger steps.
_HCHECKS = [("T", 8, 1e-4), ("T", 30, 1e-4), ("ne", 30, 1e-4), ("xi", 8, 1e-4), ("xi", 30, 1e-4),
            ("nH_I", 30, 1e-3), ("UH_I", 30, 1e-3)]
HYDROGEN_CASES = {"Balmer with MHD": ((4840.0, 4885.0), True, _HCHECKS),
                  "Balmer": ((4840.0, 4885.0), False, _HCHECKS),
                  "Brackett": ((16790.0, 16830.0), False, _HCHECKS[1:5])}


@pytest.mark.parametrize("case", list(HYDROGEN_CASES))
def test_hydrogen_gradient_exact(ctx, case):
    """The hydrogen-line reverse mode is exact: the gradient with respect to the hydrogen-line
    inputs of single layers (H beta with its ABO profile and the Stehle Balmer lines, with and
    without the MHD occupation probabilities; Griem Brackett lines in the H band) against
    Richardson-extrapolated central differences of the FP64 forward, to 1e-6.  Each difference
    also states its own uncertainty, the change of the extrapolation from steps (h, h/2) to
    (2h, h), which must itself be below 1e-6.  A wavelength whose loss term steps inside a
    difference interval has weight 0 in that check's loss and gradient: Korg's E2 is piecewise
    with jumps at its segment ends, and the hydrogen windows' edges follow the interpolated line
    centre."""
    from korg_gb300.api import synthesize_prepared, synthesize_vjp
    wl, mhd, checks = HYDROGEN_CASES[case]
    inp = _case(n_lines=30, wl=wl, seed=3)
    inp.use_MHD = mhd
    obs = _obs(inp, ctx)
    base = synthesize_prepared(inp, precision="fp64", ctx=ctx)
    r0 = base.flux / base.cntm - obs

    def terms(x):
        r = synthesize_prepared(x, precision="fp64", ctx=ctx)
        return (r.flux / r.cntm - obs) ** 2

    rows = []
    for field, l, rel in checks:
        h = rel * abs(getattr(inp, field)[l])
        t = {s: terms(_perturbed(inp, field, l, s * h)) for s in (2.0, 1.0, 0.5, -0.5, -1.0, -2.0)}
        d = {s: (t[s] - t[-s]) / (2 * s * h) for s in (2.0, 1.0, 0.5)}
        S = np.sum(np.abs(d[0.5]))
        # a smooth term's differences at h and h/2 differ by O(h^2) of itself; a step by far more
        keep = ((np.abs(d[1.0] - d[0.5]) <= 1e-3 * np.abs(d[0.5]) + 1e-7 * S) &
                (np.abs(d[2.0] - d[1.0]) <= 4e-3 * np.abs(d[1.0]) + 4e-7 * S))
        assert np.count_nonzero(keep) >= 0.95 * len(keep), (field, l)
        fd = np.sum(keep * (4 * d[0.5] - d[1.0]) / 3)  # Richardson: truncation O(h^4)
        unc = abs(fd - np.sum(keep * (4 * d[1.0] - d[2.0]) / 3))
        w = keep * 2 * r0
        g = synthesize_vjp(inp, w / base.cntm, -w * base.flux / base.cntm ** 2, precision="fp64", hydrogen=True,
                           ctx=ctx)
        rows.append((field, l, g[field][l], fd, unc, np.count_nonzero(~keep)))
        print(f"{case} {field}[{l}]: adjoint {g[field][l]:.10e}, differences {fd:.10e} +- {unc:.1e} "
              f"({np.count_nonzero(~keep)} wavelengths stepped)")
    for field, l, ad, fd, unc, _ in rows:
        assert np.isfinite(ad) and unc <= 1e-6 * abs(fd), (field, l, ad, fd, unc)
        assert abs(ad - fd) <= 1e-6 * abs(fd) + unc, (field, l, ad, fd, unc)


def test_vjp_without_hydrogen_holds_hydrogen_fixed(ctx):
    from korg_gb300.api import rectified_loss, synthesize_prepared, synthesize_vjp
    inp = _case()
    obs = _obs(inp, ctx)
    r = synthesize_prepared(inp, precision="fp64", ctx=ctx)
    _, dF, dC = rectified_loss(r.flux, r.cntm, obs)
    g = synthesize_vjp(inp, dF, dC, precision="fp64", hydrogen=False, ctx=ctx)
    assert np.all(g["nH_I"] == 0) and np.all(g["UH_I"] == 0)
    gh = synthesize_vjp(inp, dF, dC, precision="fp64", hydrogen=True, ctx=ctx)
    np.testing.assert_array_equal(g["log_gf"], gh["log_gf"])  # lines do not see the hydrogen part


def test_vjp_pinned_to_oracle_differences(ctx, oracle_lib):
    """Central differences of the FP64 oracle (the CPU restatement of the reference) agree with
    the GPU reverse mode."""
    from korg_gb300.data import stark_profiles
    from korg_gb300.api import loss_and_gradient, rectified_loss
    inp = _case(n_lines=250, wl=(5000.0, 5010.0), seed=3)
    obs = _obs(inp, ctx)
    _, g = loss_and_gradient(inp, obs, precision="fp64", ctx=ctx)
    st = stark_profiles()

    def oracle_loss(x):
        f, c, _, _, _ = oracle_lib.synthesize(x, x.linelist, x.linelist5, st, x.wls.all_wls, nthreads=NT)
        return rectified_loss(f, c, obs)[0]

    for field, idx in [("T", 30), ("ne", 30), ("xi", 30), ("log_gf", _strong_lines(inp, 1)[0])]:
        fd = _fd(inp, obs, ctx, field, idx, loss=oracle_loss)
        assert abs(g[field][idx] - fd) <= 1e-4 * abs(fd) + 1e-8 * np.max(np.abs(g[field])), (field, g[field][idx], fd)


def test_torch_autograd_matches_vjp(ctx):
    torch = pytest.importorskip("torch")
    from korg_gb300.autograd import Synthesis
    from korg_gb300.api import loss_and_gradient
    inp = _case(n_lines=400, wl=(5000.0, 5020.0), seed=5)
    obs = _obs(inp, ctx)
    _, g = loss_and_gradient(inp, obs, precision="fp64", ctx=ctx)
    synth = Synthesis(inp, precision="fp64", ctx=ctx)
    x = {k: v.clone().requires_grad_(True) for k, v in synth.initial().items()}
    flux, cntm = synth(**x)
    o = torch.as_tensor(obs, device=flux.device)
    loss = torch.sum((flux / cntm - o) ** 2)
    loss.backward()
    for k in ("T", "ne", "n_eff_vdW", "xi", "n_div_U", "log_gf", "cntm_vals", "alpha_ref_cntm"):
        np.testing.assert_allclose(x[k].grad.cpu().numpy(), g[k], rtol=1e-9, atol=1e-12 * np.max(np.abs(g[k])))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vjp_reusing_the_forward_opacity(ctx, precision):
    from korg_gb300.api import loss_and_gradient
    inp = _case(n_lines=500, wl=(5000.0, 5025.0), seed=9)
    obs = _obs(inp, ctx)
    _, g0 = loss_and_gradient(inp, obs, precision=precision, ctx=ctx)
    _, g1 = loss_and_gradient(inp, obs, precision=precision, reuse_forward=True, ctx=ctx)
    for k in g0:
        np.testing.assert_allclose(g1[k], g0[k], rtol=1e-9, atol=1e-14 * np.max(np.abs(g0[k])) + 1e-300)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vjp_many_layers(ctx, precision):
    """128 layers, the most the reverse mode takes: the staged-G ring of the FP64 line adjoint
    shrinks its stages to fit shared memory (rows of 1 kB)."""
    from korg_gb300 import synthetic
    from korg_gb300.api import loss_and_gradient
    w = synthetic.config0(seed=4, n_lines=300)
    w.L = 128
    w.wavelengths = (5000.0, 5015.0)
    w.linelist = synthetic.synthetic_linelist(300, 5001.0, 5014.0, seed=4)
    inp = synthetic.prepare(w)
    obs = _obs(inp, ctx)
    _, g = loss_and_gradient(inp, obs, precision=precision, ctx=ctx)
    if precision == "fp64":
        for field, idx in [("T", 100), ("log_gf", _strong_lines(inp, 1)[0])]:
            fd, floor = _fd(inp, obs, ctx, field, idx, noise=True)
            assert abs(g[field][idx] - fd) <= 1e-4 * abs(fd) + 1e-7 * np.max(np.abs(g[field])) + floor, (field, fd)
    else:
        _, g64 = loss_and_gradient(inp, obs, precision="fp64", ctx=ctx)
        for k in ("T", "ne", "log_gf"):
            assert np.max(np.abs(g[k] - g64[k])) <= 2e-3 * np.max(np.abs(g64[k])), k
