"""Spectral post-processing: Gaussian LSF and rotational broadening (src/utils.jl:45-240).

CPU: the FP64 restatement (oracle/postprocess_oracle.py) against the assertions of the
reference's own test/utils.jl testsets.  GPU (marked): the kernels behind korg_apply_lsf_dev /
korg_lsf_matrix_dev / korg_apply_rotation_dev and their reverse modes against the restatement.
"""
import math

import numpy as np
import pytest

import postprocess_oracle as po


def _grid(*ranges_A):
    """Korg-style ranges (start, stop, step) in Angstrom -> (all wavelengths cm, ranges cm)."""
    from korg_gb300.wavelengths import Wavelengths
    w = Wavelengths(list(ranges_A) if len(ranges_A) > 1 else ranges_A[0])
    return w.all_wls, w.ranges


# ---------------------------------------------------------------- oracle pins (CPU)
def test_lsf_oracle_pins():
    wls, _ = _grid((5900, 6100, 0.35))
    R = 1800.0
    flux = np.zeros(len(wls))
    spike = 285
    flux[spike] = 5.0
    split, _ = _grid((5900, 5935, 0.35), (5935.35, 6100, 0.35))
    np.testing.assert_allclose(po.lsf_matrix(split, wls, R), po.lsf_matrix(wls, wls, R), rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(po.lsf_matrix(wls, wls, lambda wl: R), po.lsf_matrix(wls, wls, R), rtol=1e-12)
    conv = po.apply_lsf(flux, wls, R)
    conv5 = po.apply_lsf(flux, wls, R, window_size=5)
    mat = po.lsf_matrix(wls, wls, R) @ flux
    mat5 = po.lsf_matrix(wls, wls, R, window_size=5) @ flux
    changing = po.apply_lsf(flux, wls, lambda wl: wl / 6000 * R)
    mat_changing = po.lsf_matrix(wls, wls, lambda wl: wl / 6000 * R) @ flux
    np.testing.assert_allclose(mat_changing, changing, rtol=1e-10, atol=1e-300)
    down, _ = _grid((5950, 6050, 0.4))
    mat_down = po.lsf_matrix(wls, down, R, window_size=5) @ flux
    for c in (conv, conv5, mat, mat5, changing, mat_changing):
        assert np.sum(c) == pytest.approx(np.sum(flux), rel=1e-3)  # normalised
        assert int(np.argmax(c)) == spike                            # centre preserved
    assert np.sum(mat_down) * 0.4 == pytest.approx(np.sum(flux) * 0.35, rel=1e-3)
    np.testing.assert_allclose(conv, mat5, atol=1e-4)
    np.testing.assert_allclose(conv5, mat5, rtol=1e-11)
    assert not np.allclose(conv, conv5, rtol=1e-12, atol=0)


@pytest.mark.parametrize("vsini", [0.0, 1e-10, 1.0, 5.0, 10.0, 20.0])
@pytest.mark.parametrize("eps", [0.1, 0.6, 0.9])
def test_rotation_oracle_pins(vsini, eps):
    # the reference's grid is 4090-5010 A with the block at points 990-1010; a 4990-5010 A grid
    # with the same block keeps every property the test checks (normalisation, the naive form)
    for ranges_A in (((4990, 5010, 0.01),), ((4990, 5007, 0.01), (5007.01, 5010, 0.01))):
        wls, ranges = _grid(*ranges_A)
        flux = np.zeros(len(wls))
        flux[989:1010] = 1
        rot = po.apply_rotation(flux, wls, ranges, vsini, eps)
        assert np.sum(rot) == pytest.approx(np.sum(flux), rel=1e-2)
        if vsini > 1.0 and len(ranges) == 1:
            np.testing.assert_allclose(rot, po.naive_rotation(flux, wls, ranges[0][1], vsini, eps), atol=1e-2)


# ---------------------------------------------------------------- GPU kernels vs the restatement
@pytest.fixture(scope="module")
def gctx(gpu_lib):
    c = gpu_lib.Context(0)
    yield c
    c.close()


def _spike_flux(n, idx, value=5.0):
    f = np.zeros(n)
    f[idx] = value
    return f


@pytest.mark.gpu
@pytest.mark.parametrize("R", [1800.0, "changing"])
@pytest.mark.parametrize("window", [4, 5])
def test_gpu_lsf_matches_restatement(gctx, R, window):
    from korg_gb300.postprocess import apply_LSF, compute_LSF_matrix
    Rv = (lambda wl: wl / 6000 * 1800.0) if R == "changing" else R
    wls, _ = _grid((5900, 6100, 0.35))
    rng = np.random.default_rng(3)
    flux = _spike_flux(len(wls), 285) + rng.random(len(wls))
    got = apply_LSF(flux, (5900, 6100, 0.35), Rv, window_size=window, ctx=gctx)
    np.testing.assert_allclose(got, po.apply_lsf(flux, wls, Rv, window), rtol=1e-12, atol=1e-15)
    down, _ = _grid((5950, 6050, 0.4))  # cm: the same output wavelengths for both sides
    M = compute_LSF_matrix((5900, 6100, 0.35), down, Rv, window_size=window, ctx=gctx)
    np.testing.assert_allclose(M.toarray(), po.lsf_matrix(wls, down, Rv, window), rtol=1e-12, atol=1e-15)
    obs = apply_LSF(flux, (5900, 6100, 0.35), Rv, window_size=window, obs_wls=down, ctx=gctx)
    np.testing.assert_allclose(obs, M @ flux, rtol=1e-11, atol=1e-14)


@pytest.mark.gpu
def test_gpu_lsf_stack_and_split_grid(gctx):
    from korg_gb300.postprocess import apply_LSF
    ranges = ((5900, 5935, 0.35), (5935.35, 6100, 0.35))
    wls, _ = _grid(*ranges)
    rng = np.random.default_rng(5)
    stack = rng.random((11, len(wls)))  # two blocks of the kernel's spectrum loop
    got = apply_LSF(stack, list(ranges), 1800.0, ctx=gctx)
    for k in range(11):
        np.testing.assert_allclose(got[k], po.apply_lsf(stack[k], wls, 1800.0), rtol=1e-12, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("vsini", [0.0, 1e-10, 1.0, 5.0, 10.0, 20.0])
@pytest.mark.parametrize("eps", [0.1, 0.6, 0.9])
def test_gpu_rotation_matches_restatement(gctx, vsini, eps):
    from korg_gb300.postprocess import apply_rotation
    from korg_gb300.wavelengths import Wavelengths
    rng = np.random.default_rng(7)
    for spec in ([(4990, 5010, 0.01)], [(4990, 5007, 0.01), (5007.01, 5010, 0.01)]):
        g = Wavelengths(spec if len(spec) > 1 else spec[0])
        flux = np.zeros(len(g))
        flux[989:1010] = 1
        stack = np.stack([flux, rng.random(len(g))])
        got = apply_rotation(stack, g, vsini, eps, ctx=gctx)
        for k in range(2):
            ref = po.apply_rotation(stack[k], g.all_wls, g.ranges, vsini, eps)
            np.testing.assert_allclose(got[k], ref, rtol=1e-11, atol=1e-13)


@pytest.mark.gpu
def test_gpu_postprocess_reverse_modes_are_transposes(gctx):
    """<L f, g> = <f, L^T g> for the LSF (grid to a coarser output grid) and the rotation, through
    the torch autograd functions."""
    torch = pytest.importorskip("torch")
    from korg_gb300.postprocess import LSF, Rotation
    from korg_gb300.wavelengths import Wavelengths
    dev = torch.device("cuda", 0)
    g = Wavelengths([(5000, 5010, 0.01), (5010.01, 5020, 0.01)])
    w = torch.as_tensor(g.all_wls, device=dev)
    out = torch.as_tensor(np.arange(5001, 5019, 0.05) * 1e-8, device=dev)
    R = torch.tensor([22500.0], dtype=torch.float64, device=dev)
    rng = np.random.default_rng(11)
    f = torch.as_tensor(rng.random((3, len(g))), device=dev).requires_grad_(True)
    y = LSF.apply(f, w, out, R, 4.0, gctx)
    gy = torch.as_tensor(rng.random(tuple(y.shape)), device=dev)
    (y * gy).sum().backward()
    assert torch.sum(y * gy).item() == pytest.approx(torch.sum(f * f.grad).item(), rel=1e-12)
    f2 = torch.as_tensor(rng.random((2, len(g))), device=dev).requires_grad_(True)
    z = Rotation.apply(f2, w, g, 15.0, 0.6, gctx)
    gz = torch.as_tensor(rng.random(tuple(z.shape)), device=dev)
    (z * gz).sum().backward()
    assert torch.sum(z * gz).item() == pytest.approx(torch.sum(f2 * f2.grad).item(), rel=1e-12)
