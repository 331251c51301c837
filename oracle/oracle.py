"""ctypes wrapper of the FP64 CPU oracle (korg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, as the checker.  The product path never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkorg_oracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)


class KoLines(C.Structure):
    _fields_ = [("n", C.c_int64), ("wl", _dp), ("log_gf", _dp), ("E_lower", _dp),
                ("gamma_rad", _dp), ("gamma_stark", _dp), ("vdW1", _dp), ("vdW2", _dp),
                ("mass", _dp), ("is_mol", _ip), ("species", _ip)]


class KoLayers(C.Structure):
    _fields_ = [("L", C.c_int32), ("S", C.c_int32), ("T", _dp), ("ne", _dp), ("n_eff_vdW", _dp),
                ("xi", _dp), ("n_div_U", _dp)]


class KoCntm(C.Structure):
    _fields_ = [("nk", C.c_int64), ("knots", _dp), ("vals", _dp)]


class KoStark(C.Structure):
    _fields_ = [("ntrans", C.c_int32), ("lower", _ip), ("upper", _ip), ("nT", _ip), ("nNe", _ip),
                ("nD", _ip), ("t_off", _lp), ("ne_off", _lp), ("d_off", _lp), ("p_off", _lp),
                ("l_off", _lp), ("log_gf", _dp), ("temps", _dp), ("nes", _dp), ("logdnu", _dp),
                ("logP", _dp), ("lambda0", _dp)]


class KoSynthIn(C.Structure):
    _fields_ = [("L", C.c_int32), ("T", _dp), ("ne", _dp), ("tau_ref", _dp), ("xi", _dp),
                ("n_eff_vdW", _dp), ("n_div_U", _dp), ("S", C.c_int32), ("nH_I", _dp),
                ("nHe_I", _dp), ("UH_I", _dp), ("alpha_ref_cntm", _dp), ("ref_wl", C.c_double),
                ("cntm", KoCntm), ("hydrogen_lines", C.c_int), ("use_MHD", C.c_int),
                ("hydrogen_window", C.c_double), ("cutoff_threshold", C.c_double),
                ("nthreads", C.c_int)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.ko_voigt_hjerting.restype = C.c_double
        L.ko_voigt_hjerting.argtypes = [C.c_double, C.c_double]
        L.ko_line_profile.restype = C.c_double
        L.ko_line_profile.argtypes = [C.c_double] * 5
        L.ko_exponential_integral_1.restype = C.c_double
        L.ko_exponential_integral_1.argtypes = [C.c_double]
        L.ko_exponential_integral_2.restype = C.c_double
        L.ko_exponential_integral_2.argtypes = [C.c_double]
        L.ko_blackbody.restype = C.c_double
        L.ko_blackbody.argtypes = [C.c_double, C.c_double]
        L.ko_hummer_mihalas_w.restype = C.c_double
        L.ko_hummer_mihalas_w.argtypes = [C.c_double] * 5
        L.ko_line_absorption.restype = C.c_int64
        L.ko_hydrogen_line_absorption.restype = None
        L.ko_brackett_profile.restype = C.c_double
        L.ko_brackett_profile.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, _dp, _dp]
        L.ko_rt_flux_expint.restype = None
        L.ko_rt_general.restype = C.c_int
        L.ko_synthesize.restype = C.c_int64
        _lib = L
    return _lib


def _p(a, kind=_dp):
    return a.ctypes.data_as(kind) if a is not None else None


class _Keep:
    """Holds numpy arrays alive as long as the ctypes struct that points into them."""

    def __init__(self):
        self.arrays = []

    def f64(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.arrays.append(a)
        return a

    def i32(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.arrays.append(a)
        return a

    def i64(self, a):
        a = np.ascontiguousarray(a, dtype=np.int64)
        self.arrays.append(a)
        return a


def make_lines(ll, keep: _Keep):
    return KoLines(len(ll), _p(keep.f64(ll.wl)), _p(keep.f64(ll.log_gf)), _p(keep.f64(ll.E_lower)),
                   _p(keep.f64(ll.gamma_rad)), _p(keep.f64(ll.gamma_stark)), _p(keep.f64(ll.vdW1)),
                   _p(keep.f64(ll.vdW2)), _p(keep.f64(ll.mass)), _p(keep.i32(ll.is_mol), _ip),
                   _p(keep.i32(ll.species_idx), _ip))


def make_stark(st, keep: _Keep):
    return KoStark(st["ntrans"], *[_p(keep.i32(st[k]), _ip) for k in ["lower", "upper", "nT", "nNe", "nD"]],
                   *[_p(keep.i64(st[k]), _lp) for k in ["t_off", "ne_off", "d_off", "p_off", "l_off"]],
                   *[_p(keep.f64(st[k])) for k in ["log_gf", "temps", "nes", "logdnu", "logP", "lambda0"]])


def line_profile(wl0, sigma, gamma, amp, wls):
    wls = np.ascontiguousarray(wls, dtype=np.float64)
    out = np.empty_like(wls)
    lib().ko_line_profile_many(C.c_int64(len(wls)), C.c_double(wl0), C.c_double(sigma),
                               C.c_double(gamma), C.c_double(amp), _p(wls), _p(out))
    return out


def voigt_hjerting(a, v):
    a, v = np.broadcast_arrays(np.asarray(a, np.float64), np.asarray(v, np.float64))
    a, v = np.ascontiguousarray(a), np.ascontiguousarray(v)
    out = np.empty_like(a)
    lib().ko_voigt_many(C.c_int64(a.size), _p(a), _p(v), _p(out))
    return out


def exponential_integral_2(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lib().ko_expint2_many(C.c_int64(x.size), _p(x), _p(out))
    return out


def line_absorption(alpha, ll, wls, T, ne, n_eff_vdW, xi, n_div_U, cntm_knots, cntm_vals,
                    cutoff=3e-4, nthreads=1, want_bounds=False):
    """alpha (nwl, L) C-order == Korg's L x nwl column-major; accumulated in place."""
    keep = _Keep()
    L = len(T)
    lines = make_lines(ll, keep)
    lay = KoLayers(L, n_div_U.shape[0], _p(keep.f64(T)), _p(keep.f64(ne)), _p(keep.f64(n_eff_vdW)),
                   _p(keep.f64(xi)), _p(keep.f64(n_div_U)))
    cn = KoCntm(len(cntm_knots) if cntm_knots is not None else 1,
                _p(keep.f64(cntm_knots)) if cntm_knots is not None else None, _p(keep.f64(cntm_vals)))
    wls = keep.f64(wls)
    assert alpha.flags.c_contiguous and alpha.dtype == np.float64 and alpha.shape == (len(wls), L)
    lb = np.zeros(len(ll), np.int64) if want_bounds else None
    ub = np.zeros(len(ll), np.int64) if want_bounds else None
    n = lib().ko_line_absorption(_p(alpha), C.byref(lines), _p(wls), C.c_int64(len(wls)),
                                 C.byref(lay), C.byref(cn), C.c_double(cutoff), C.c_int(nthreads),
                                 _p(lb, _lp), _p(ub, _lp))
    return (n, lb, ub) if want_bounds else n


def hydrogen_line_absorption(alphas, wls, T, ne, nH_I, nHe_I, UH_I, xi, window, use_MHD, stark):
    keep = _Keep()
    st = make_stark(stark, keep)
    wls = keep.f64(wls)
    assert alphas.flags.c_contiguous and alphas.dtype == np.float64
    lib().ko_hydrogen_line_absorption(_p(alphas), _p(wls), C.c_int64(len(wls)), C.c_double(T),
                                      C.c_double(ne), C.c_double(nH_I), C.c_double(nHe_I),
                                      C.c_double(UH_I), C.c_double(xi), C.c_double(window),
                                      C.c_int(int(use_MHD)), C.byref(st))


def rt_flux_expint(alpha, S, tau_ref, alpha_ref, nthreads=1):
    alpha = np.ascontiguousarray(alpha, np.float64)
    S = np.ascontiguousarray(S, np.float64)
    nwl, L = alpha.shape
    flux = np.empty(nwl)
    tr = np.ascontiguousarray(tau_ref, np.float64)
    ar = np.ascontiguousarray(alpha_ref, np.float64)
    lib().ko_rt_flux_expint(_p(alpha), _p(S), C.c_int32(L), C.c_int64(nwl), _p(tr), _p(ar), _p(flux),
                            C.c_int(nthreads))
    return flux


def rt_general(alpha, S, spatial, spherical, tau_ref, alpha_ref, mu, mu_w, include_inward_rays,
               tau_scheme, I_scheme):
    alpha = np.ascontiguousarray(alpha, np.float64)
    S = np.ascontiguousarray(S, np.float64)
    nwl, L = alpha.shape
    keep = _Keep()
    flux = np.empty(nwl)
    rc = lib().ko_rt_general(_p(alpha), _p(S), C.c_int32(L), C.c_int64(nwl), _p(keep.f64(spatial)),
                             C.c_int(int(spherical)), _p(keep.f64(tau_ref)), _p(keep.f64(alpha_ref)),
                             _p(keep.f64(mu)), _p(keep.f64(mu_w)), C.c_int(len(mu)),
                             C.c_int(int(include_inward_rays)), C.c_int(tau_scheme), C.c_int(I_scheme),
                             _p(flux))
    if rc != 0:
        raise ValueError("bad RT scheme")
    return flux


def blackbody(T, wl):
    return lib().ko_blackbody(float(T), float(wl))


def synthesize(inp, ll, ll5, stark, wls, nthreads=1):
    """inp: a korg_gb300 SynthesisInputs; returns (flux, cntm, alpha (nwl, L), alpha_ref, evals)."""
    keep = _Keep()
    L = len(inp.T)
    s = KoSynthIn(L, _p(keep.f64(inp.T)), _p(keep.f64(inp.ne)), _p(keep.f64(inp.tau_ref)),
                  _p(keep.f64(inp.xi)), _p(keep.f64(inp.n_eff_vdW)), _p(keep.f64(inp.n_div_U)),
                  inp.n_div_U.shape[0], _p(keep.f64(inp.nH_I)), _p(keep.f64(inp.nHe_I)),
                  _p(keep.f64(inp.UH_I)), _p(keep.f64(inp.alpha_ref_cntm)), inp.ref_wl,
                  KoCntm(len(inp.cntm_knots), _p(keep.f64(inp.cntm_knots)), _p(keep.f64(inp.cntm_vals))),
                  int(inp.hydrogen_lines), int(inp.use_MHD), inp.hydrogen_window, inp.cutoff_threshold,
                  nthreads)
    lines = make_lines(ll, keep)
    lines5 = make_lines(ll5, keep)
    st = make_stark(stark, keep)
    wls = keep.f64(wls)
    nwl = len(wls)
    alpha = np.zeros((nwl, L))
    flux = np.zeros(nwl)
    cntm = np.zeros(nwl)
    aref = np.zeros(L)
    ev = lib().ko_synthesize(C.byref(s), C.byref(lines), C.byref(lines5), C.byref(st), _p(wls),
                             C.c_int64(nwl), _p(alpha), _p(flux), _p(cntm), _p(aref))
    return flux, cntm, alpha, aref, ev
