"""Batched synthesis (korg_synthesize_batch_dev): persistent (spectrum, tile) queue, chunking,
CUDA-graph replay and the tile-shape autotuner, checked against one-spectrum synthesis."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(specs):
    from korg_gb300 import synthetic
    out = []
    for Teff, logg, n, seed in specs:
        w = synthetic.config0(seed=seed, n_lines=n)
        w.Teff, w.logg = Teff, logg
        out.append(synthetic.prepare(w))
    return out


def _single(inp, precision, ctx):
    from korg_gb300.api import synthesize_prepared
    r = synthesize_prepared(inp, precision=precision, ctx=ctx)
    return r.flux, r.cntm


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single_spectrum_synthesis(gpu_lib, precision):
    from korg_gb300.batch import BatchSynthesis
    inps = _inputs([(5000.0, 4.4, 2000, 0), (4200.0, 2.0, 700, 1), (6500.0, 4.0, 1, 2)])
    b = BatchSynthesis(inps, precision=precision, use_graph=False)
    b.run()
    flux, cntm = b.results()
    for k, inp in enumerate(inps):
        f1, c1 = _single(inp, precision, b.ctx)
        # same kernels, same tile shape, same order of accumulation: identical
        assert np.array_equal(flux[k], f1), k
        assert np.array_equal(cntm[k], c1), k


def test_batch_chunks_graph_replay_and_new_inputs(gpu_lib):
    from korg_gb300.batch import BatchSynthesis
    inps = _inputs([(5200.0, 4.4, 1500, 3), (4800.0, 3.0, 1200, 4), (5900.0, 4.2, 900, 5), (4000.0, 1.5, 600, 6)])
    # a one-byte budget puts every spectrum in a chunk of its own
    b = BatchSynthesis(inps, precision="mixed", use_graph=True, max_scratch_bytes=1)
    ref = [_single(inp, "mixed", b.ctx) for inp in inps]
    for call in range(3):  # eager, captured, replayed
        b.run()
        flux, cntm = b.results()
        for k in range(len(inps)):
            assert np.array_equal(flux[k], ref[k][0]), (call, k)
            assert np.array_equal(cntm[k], ref[k][1]), (call, k)
    # new temperatures in the same buffers: the replayed graph reads them
    T = b.host_array(1, "T")
    T *= 1.02
    b.upload()
    b.run()
    flux, _ = b.results()
    import copy
    mod = copy.copy(inps[1])
    mod.T = inps[1].T * 1.02
    f1, _ = _single(mod, "mixed", b.ctx)
    assert np.array_equal(flux[1], f1)
    assert not np.array_equal(f1, ref[1][0])
    assert np.array_equal(flux[0], ref[0][0])


def test_batch_autotuner_picks_a_shape_and_keeps_results(gpu_lib):
    from korg_gb300 import synthetic
    from korg_gb300.batch import BatchSynthesis
    works = synthetic.config3(n_spectra=2, n_list=40_000, n_min=12_000, n_max=25_000,
                              wavelengths=(15000, 15500, 0.005))
    inps = [synthetic.prepare(w) for w in works]
    plain = BatchSynthesis(inps, precision="mixed", use_graph=False)
    plain.run()
    f0, c0 = plain.results()
    assert not plain.tile_config()["tuned"]
    tuned = BatchSynthesis(inps, precision="mixed", use_graph=True, autotune=True)
    for _ in range(3):
        tuned.run()
    f1, c1 = tuned.results()
    cfg = tuned.tile_config()
    # mixed shapes: 64-256 wavelengths x one layer group, 32- or 64-line batches
    assert cfg["tuned"] and cfg["tw"] in (64, 128, 256) and cfg["stage"] in (32, 64) and cfg["split"]
    # another tile shape changes the FP32 rounding of the offsets and the Kahan batches only
    np.testing.assert_allclose(f1, f0, rtol=2e-6, atol=0)
    np.testing.assert_allclose(c1, c0, rtol=2e-6, atol=0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tile_shapes_give_identical_opacity(gpu_lib, precision):
    """FP64: splitting the layer groups over CTAs keeps every thread's accumulation order, so the
    opacity is bitwise unchanged; other tile widths move only the batch boundaries.  Mixed (always
    one layer group per CTA; a shape with all groups per CTA is KORG_EINVAL): other widths and
    batch sizes move the tile origins (the FP32 offsets, and which lines take the wing cubics) and
    the Kahan batch boundaries only."""
    import ctypes as C
    from korg_gb300 import synthetic
    from korg_gb300.api import synthesize_prepared
    inp = synthetic.prepare(synthetic.config0(n_lines=3000))
    prec = gpu_lib.KORG_MIXED if precision == "mixed" else gpu_lib.KORG_FP64
    L = len(inp.T)
    shapes = ((64, 0, 0), (64, 0, 1), (32, 16, 1), (128, 0, 0)) if precision == "fp64" else \
        ((128, 0, 1), (64, 32, 1), (256, 64, 1), (32, 16, 1))
    out = {}
    for cfg in shapes:
        ctx = gpu_lib.Context(0)
        ctx.check(ctx.lib.korg_set_tile_config(ctx.h, L, prec, *cfg))
        r = synthesize_prepared(inp, precision=precision, return_alpha=True, ctx=ctx)
        out[cfg] = r
        ctx.close()
    base = out[shapes[0]]
    if precision == "fp64":
        assert np.array_equal(out[(64, 0, 1)].alpha, base.alpha)
        for cfg in ((32, 16, 1), (128, 0, 0)):
            np.testing.assert_allclose(out[cfg].alpha, base.alpha, rtol=1e-13)
    else:
        for cfg in shapes[1:]:
            np.testing.assert_allclose(out[cfg].alpha, base.alpha, rtol=1e-5)
        ctx = gpu_lib.Context(0)
        assert ctx.lib.korg_set_tile_config(ctx.h, L, prec, 64, 0, 0) == 1  # all groups per CTA: mixed has none
        ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_vjp_equals_per_spectrum_vjp(gpu_lib, precision):
    """korg_synthesize_batch_vjp_dev, reusing the batched forward's opacity and recomputing it,
    gives every spectrum the gradients of korg_synthesize_vjp (the same kernels: equal up to the
    order of the line adjoint's FP64 atomic additions)."""
    from korg_gb300.api import GRAD_FIELDS, synthesize_vjp
    from korg_gb300.batch import BatchSynthesis
    inps = _inputs([(5000.0, 4.4, 800, 7), (4200.0, 2.0, 500, 8), (6500.0, 4.0, 300, 9)])
    b = BatchSynthesis(inps, precision=precision, use_graph=False)
    torch = b.torch
    rng = np.random.default_rng(3)
    dF = torch.as_tensor(rng.normal(size=(len(inps), b.nwl)), device=b.dev)
    dC = torch.as_tensor(rng.normal(size=(len(inps), b.nwl)), device=b.dev)
    b.run()
    g_reuse = b.vjp(dF, dC, reuse_forward=True)
    g_recomp = b.vjp(dF, dC, reuse_forward=False)
    torch.cuda.synchronize()
    tol = 1e-12 if precision == "fp64" else 1e-9
    for k, inp in enumerate(inps):
        ref = synthesize_vjp(inp, dF[k].cpu().numpy(), dC[k].cpu().numpy(), precision=precision, ctx=b.ctx)
        for f in GRAD_FIELDS:
            scale = max(float(np.max(np.abs(ref[f]))), 1e-300)
            for name, g in (("reuse", g_reuse), ("recompute", g_recomp)):
                got = g[k][f].cpu().numpy().reshape(ref[f].shape)
                assert np.max(np.abs(got - ref[f])) <= tol * scale, (k, f, name)
    # reuse needs the batch forward of the same items just before
    other = BatchSynthesis(inps[:2], precision=precision, use_graph=False, ctx=b.ctx)
    other.run()
    with pytest.raises(gpu_lib.KorgError):
        b.vjp(dF, dC, reuse_forward=True)
