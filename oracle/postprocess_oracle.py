"""FP64 CPU restatement of Korg's spectral post-processing: the Gaussian line-spread function and
rotational broadening (src/utils.jl).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU kernels.  The product
path never imports this module.

Pinned in tests/test_postprocess.py against the assertions of the reference's own
test/utils.jl ("LSF" and "rotation" testsets: normalisation, preserved line centre, window-size
behaviour, split grids, R as a function, and the naive rotation comparison).
"""
from __future__ import annotations

import math

import numpy as np

C_CGS = 2.99792458e10


def _as_cm(w):
    w = np.asarray(w, dtype=np.float64)
    return w * 1e-8 if w.size and w[0] >= 1 else w


def lsf_bounds_and_kernel(synth_wls, wl0, R, window_size):
    """_lsf_bounds_and_kernel (src/utils.jl:45-58): FWHM wl0/R as sigma, window +- window_size
    sigma (searchsortedfirst / searchsortedlast, 0-based inclusive bounds here), normalised
    Gaussian weights."""
    R_val = R(wl0 * 1e8) if callable(R) else R
    sigma = wl0 / R_val / (2 * math.sqrt(2 * math.log(2)))
    lb = int(np.searchsorted(synth_wls, wl0 - window_size * sigma, side="left"))
    ub = int(np.searchsorted(synth_wls, wl0 + window_size * sigma, side="right")) - 1
    d = synth_wls[lb:ub + 1] - wl0
    phi = np.exp(-0.5 * d * d / sigma ** 2) / math.sqrt(2 * math.pi) / sigma  # normal_pdf, :5
    return lb, ub, phi / np.sum(phi)


def apply_lsf(flux, wls, R, window_size=4):
    """apply_LSF (src/utils.jl:94-106)."""
    flux = np.asarray(flux, dtype=np.float64)
    if R == math.inf:
        return flux.copy()
    w = _as_cm(wls)
    out = np.zeros_like(flux)
    for i in range(len(w)):
        lb, ub, phi = lsf_bounds_and_kernel(w, w[i], R, window_size)
        out[i] = np.sum(flux[lb:ub + 1] * phi)
    return out


def lsf_matrix(synth_wls, obs_wls, R, window_size=4):
    """compute_LSF_matrix (src/utils.jl:132-155) as a dense (n_obs, n_synth) array."""
    s = _as_cm(synth_wls)
    o = _as_cm(obs_wls)
    M = np.zeros((len(o), len(s)))
    for i in range(len(o)):
        lb, ub, phi = lsf_bounds_and_kernel(s, o[i], R, window_size)
        M[i, lb:ub + 1] += phi
    return M


def _rotation_kernel_integral(c1, c2, c3, detuning, dl_rot):
    """_rotation_kernel_integral_kernel (src/utils.jl:233-240)."""
    if abs(detuning) == dl_rot:
        return math.copysign(0.5, detuning)
    return (0.5 * c1 * detuning * math.sqrt(1 - detuning ** 2 / dl_rot ** 2)
            + 0.5 * c1 * dl_rot * math.asin(detuning / dl_rot)
            + c2 * (detuning - detuning ** 3 / (3 * dl_rot ** 2))) / c3


def _rotation_kernel_integrals(c1, c2, c3, det, dl_rot):
    """_rotation_kernel_integral over an array of detunings."""
    edge = np.abs(det) == dl_rot
    d = np.where(edge, 0.0, det)
    k = (0.5 * c1 * d * np.sqrt(1 - d ** 2 / dl_rot ** 2) + 0.5 * c1 * dl_rot * np.arcsin(d / dl_rot)
         + c2 * (d - d ** 3 / (3 * dl_rot ** 2))) / c3
    return np.where(edge, np.copysign(0.5, det), k)


def _rotation_core(flux, w, step, vsini, eps):
    """_apply_rotation_core (src/utils.jl:193-230) on one uniform range: grid values w (cm) and
    its step."""
    if vsini == 0:
        return np.array(flux, dtype=np.float64)
    n = len(w)
    v = vsini * 1e5
    c1 = 2 * (1 - eps)
    c2 = math.pi * eps / 2
    c3 = math.pi * (1 - eps / 3)
    out = np.zeros(n)
    for i in range(n):
        dl = w[i] * v / C_CGS
        lb = int(np.searchsorted(w, w[i] - dl, side="left"))
        ub = int(np.searchsorted(w, w[i] + dl, side="right")) - 1
        fw = flux[lb:ub + 1]
        det = np.concatenate(([-dl], (np.arange(lb - i, ub - i) + 0.5) * step, [dl]))
        ks = _rotation_kernel_integrals(c1, c2, c3 * dl, det, dl)
        out[i] = np.sum(ks[1:] * fw) - np.sum(ks[:-1] * fw)
    return out


def apply_rotation(flux, wls, ranges, vsini, eps=0.6):
    """apply_rotation (src/utils.jl:168-192): each wavelength range (start_cm, step_cm, n) of the
    grid wls (cm) separately."""
    flux = np.asarray(flux, dtype=np.float64)
    out = np.empty_like(flux)
    i0 = 0
    for _, step, n in ranges:
        out[i0:i0 + n] = _rotation_core(flux[i0:i0 + n], wls[i0:i0 + n], step, vsini, eps)
        i0 += n
    return out


def naive_rotation(flux, w, step, vsini, eps=0.6):
    """The reference test's own naive rotation (test/utils.jl:86-111), a coarser scatter form used
    there as the comparison for apply_rotation."""
    v = vsini * 1e5
    n = len(w)
    out = np.zeros(n)
    c1 = 2 * (1 - eps)
    c2 = math.pi * eps / 2
    denominator = math.pi * (1 - eps / 3) / step
    for i in range(n):
        dl = w[i] * v / C_CGS
        nw = int(math.floor(dl / step))
        lo, hi = max(0, i - nw), min(n - 1, i + nw)
        x = (w[i] - w[lo:hi + 1]) / dl
        one = 1 - x ** 2
        out[lo:hi + 1] += flux[i] * (c1 * np.sqrt(one) + c2 * one) / (denominator * dl)
    return out
