"""ctypes binding of libkorg_gb300.so (the C ABI declared in include/korg_gb300.h).

The library is built in-tree by ``korg.jl_gb300/build.py``.  Loading fails loudly when it is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "libkorg_gb300.so")

KORG_FP64, KORG_MIXED = 0, 1
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)

ERRORS = {1: "KORG_EINVAL", 2: "KORG_ECUDA", 3: "KORG_ENOMEM", 4: "KORG_ENOTABLES", 5: "KORG_ETOOBIG",
          6: "KORG_ETIMEOUT"}


class KorgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Lines(C.Structure):
    _fields_ = [("n", C.c_int64), ("wl", _dp), ("log_gf", _dp), ("E_lower", _dp), ("gamma_rad", _dp),
                ("gamma_stark", _dp), ("vdW1", _dp), ("vdW2", _dp), ("mass", _dp), ("is_mol", _ip),
                ("species", _ip)]


class Layers(C.Structure):
    _fields_ = [("L", C.c_int32), ("S", C.c_int32), ("T", _dp), ("ne", _dp), ("n_eff_vdW", _dp),
                ("xi", _dp), ("n_div_U", _dp)]


class Cntm(C.Structure):
    _fields_ = [("nk", C.c_int64), ("knots", _dp), ("vals", _dp)]


class StarkTables(C.Structure):
    _fields_ = [("ntrans", C.c_int32), ("lower", _ip), ("upper", _ip), ("nT", _ip), ("nNe", _ip),
                ("nD", _ip), ("t_off", _lp), ("ne_off", _lp), ("d_off", _lp), ("p_off", _lp),
                ("l_off", _lp), ("log_gf", _dp), ("temps", _dp), ("nes", _dp), ("logdnu", _dp),
                ("logP", _dp), ("lambda0", _dp)]


class SynthInputs(C.Structure):
    _fields_ = [("layers", Layers), ("tau_ref", _dp), ("alpha_ref_cntm", _dp), ("nH_I", _dp),
                ("nHe_I", _dp), ("UH_I", _dp), ("ref_wl", C.c_double), ("cntm", Cntm),
                ("hydrogen_lines", C.c_int32), ("use_MHD", C.c_int32), ("hydrogen_window", C.c_double),
                ("cutoff_threshold", C.c_double)]


class SynthGrads(C.Structure):
    _fields_ = [("T", _dp), ("ne", _dp), ("n_eff_vdW", _dp), ("xi", _dp), ("n_div_U", _dp), ("nH_I", _dp),
                ("nHe_I", _dp), ("UH_I", _dp), ("log_gf", _dp), ("cntm_vals", _dp), ("alpha_ref_cntm", _dp)]


KORG_VJP_HYDROGEN, KORG_VJP_REUSE_FORWARD = 1, 2


class BatchItem(C.Structure):
    _fields_ = [("inp", SynthInputs), ("lines", Lines), ("lines5", Lines), ("flux", _dp), ("cntm", _dp)]


class ContinuumTables(C.Structure):
    """korg_continuum_tables (host arrays)."""
    _fields_ = [("h_n", C.c_int32), ("h_E", _dp), ("h_sigma", _dp), ("hm_n", C.c_int64), ("hm_nu", _dp),
                ("hm_sigma", _dp), ("hff_nl", C.c_int32), ("hff_nt", C.c_int32), ("hff_lambda", _dp),
                ("hff_theta", _dp), ("hff_K", _dp), ("heff_nl", C.c_int32), ("heff_nt", C.c_int32),
                ("heff_lambda", _dp), ("heff_theta", _dp), ("heff_K", _dp), ("h2_nT", C.c_int32),
                ("h2_nbf", C.c_int32), ("h2_nff", C.c_int32), ("h2_T", _dp), ("h2_K", _dp), ("h2_bf_lambda", _dp),
                ("h2_bf_sigma", _dp), ("h2_ff_lambda", _dp), ("h2_ff_sigma", _dp), ("g_nu", C.c_int32),
                ("g_ng", C.c_int32), ("g_log_u", _dp), ("g_log_g2", _dp), ("g_ff", _dp), ("p_nT", C.c_int32 * 4),
                ("p_ns", C.c_int32), ("p_T", _dp * 4), ("p_sigma", _dp), ("p_D", _dp * 4)]


class ContinuumLayers(C.Structure):
    """korg_continuum_layers."""
    _fields_ = [("L", C.c_int32)] + [(k, _dp) for k in ("T", "ne", "nH_I", "nH_II", "nHe_I", "nH2", "nH_minus",
                                                          "invU_H_I", "invU_He_I", "n_Z1", "n_Z2")] + \
               [("n_peach", _dp * 4)]


class EquilibriumTables(C.Structure):
    """korg_equilibrium_tables (host arrays)."""
    _fields_ = [("n_knots", C.c_int32), ("lnT", _dp), ("U_u", _dp), ("U_z", _dp), ("chi", _dp), ("n_mol", C.c_int32),
                ("atoms", _ip), ("charge", _ip), ("kind", _ip), ("off", C.POINTER(C.c_int64)), ("spl_t", _dp),
                ("spl_u", _dp), ("spl_z", _dp), ("D00", _dp), ("lmr", _dp)]


class ChemLayers(C.Structure):
    """korg_chem_layers."""
    _fields_ = [("L", C.c_int32), ("T", _dp), ("n_tot", _dp), ("ne_model", _dp), ("abundances", _dp), ("atm", _ip)]


KORG_ECHEM = 7
KORG_CHEM_MOL0 = 278
KORG_CHEM_MAX_MOL = 384


class BatchVjpItem(C.Structure):
    """korg_batch_vjp_item: one spectrum's cotangents and gradient outputs (device pointers)."""
    _fields_ = [("dflux", _dp), ("dcntm", _dp), ("grads", SynthGrads)]


class Stats(C.Structure):
    _fields_ = [("line_evals", C.c_int64), ("lines_in_window", C.c_int64), ("ms_ref_lines", C.c_float),
                ("ms_hydrogen", C.c_float), ("ms_line_prep", C.c_float), ("ms_line_tile", C.c_float),
                ("ms_rt", C.c_float), ("ms_total", C.c_float), ("ms_vjp_alpha", C.c_float),
                ("ms_vjp_rt", C.c_float), ("ms_vjp_hydrogen", C.c_float), ("ms_vjp_lines", C.c_float)]


_lib = None
_lock = threading.Lock()


def lib():
    """Load libkorg_gb300.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: build it with korg.jl_gb300/build.py "
                                  "(the CUDA library is required; there is no CPU path)")
            L = C.CDLL(LIB_PATH)
            vp = C.c_void_p
            L.korg_create.argtypes = [C.POINTER(vp), C.c_int]
            L.korg_destroy.argtypes = [vp]
            L.korg_destroy.restype = None
            L.korg_last_error.argtypes = [vp]
            L.korg_last_error.restype = C.c_char_p
            L.korg_get_stats.argtypes = [vp, C.POINTER(Stats)]
            L.korg_set_timing.argtypes = [vp, C.c_int]
            L.korg_set_stark_tables.argtypes = [vp, C.POINTER(StarkTables)]
            L.korg_line_absorption.argtypes = [vp, _dp, _dp, C.c_int64, C.POINTER(Lines), C.POINTER(Layers),
                                               C.POINTER(Cntm), C.c_double, C.c_int, _lp]
            L.korg_line_absorption_dev.argtypes = [vp, vp, vp, C.c_int64, C.POINTER(Lines), C.POINTER(Layers),
                                                   C.POINTER(Cntm), C.c_double, C.c_int, vp]
            L.korg_hydrogen_line_absorption.argtypes = [vp, _dp, _dp, C.c_int64] + [C.c_double] * 7 + [C.c_int, C.c_int]
            L.korg_hydrogen_lines_dev.argtypes = [vp, vp, vp, C.c_int64, C.c_int32] + [vp] * 6 + \
                [C.c_double, C.c_int, C.c_int, vp]
            L.korg_radiative_transfer.argtypes = [vp, _dp, _dp, C.c_int32, C.c_int64, _dp, _dp, _dp]
            L.korg_radiative_transfer_dev.argtypes = [vp, vp, vp, C.c_int32, C.c_int64, vp, vp, vp, vp]
            L.korg_synthesize.argtypes = [vp, C.POINTER(SynthInputs), C.POINTER(Lines), C.POINTER(Lines), _dp,
                                          C.c_int64, C.c_int, _dp, _dp, _dp, _dp]
            L.korg_synthesize_dev.argtypes = [vp, C.POINTER(SynthInputs), C.POINTER(Lines), C.POINTER(Lines), vp,
                                              C.c_int64, C.c_int, vp, vp, vp, vp]
            L.korg_probe_flops.argtypes = [vp, C.c_int, _dp]
            L.korg_math_selftest.argtypes = [vp, C.c_int64, _dp, _dp]
            L.korg_line_absorption_noalloc.argtypes = [vp, vp, C.c_int64, C.POINTER(Lines), C.POINTER(Layers),
                                                       C.POINTER(Cntm), C.c_double, C.c_int, vp]
            L.korg_radiative_transfer_general.argtypes = [vp, _dp, _dp, C.c_int32, C.c_int64, _dp, C.c_int, _dp, _dp,
                                                          _dp, _dp, C.c_int32, C.c_int, C.c_int, C.c_int, _dp, _dp]
            L.korg_molecular_cross_section_dev.argtypes = [vp, C.POINTER(Lines), vp, C.c_int64, vp, vp, C.c_int32, vp,
                                                           C.c_int32, C.c_double, C.c_int, vp, vp]
            L.korg_interpolate_molecular_cross_section_dev.argtypes = [vp, vp, vp, C.c_int64, C.c_int32, vp, vp, vp,
                                                                       vp, vp, C.c_int64, vp, C.c_int32, vp,
                                                                       C.c_int32, vp]
            L.korg_synthesize_vjp.argtypes = [vp, C.POINTER(SynthInputs), C.POINTER(Lines), C.POINTER(Lines), _dp,
                                              C.c_int64, C.c_int, _dp, _dp, C.POINTER(SynthGrads), C.c_int]
            L.korg_synthesize_vjp_dev.argtypes = [vp, C.POINTER(SynthInputs), C.POINTER(Lines), C.POINTER(Lines), vp,
                                                  C.c_int64, C.c_int, vp, vp, C.POINTER(SynthGrads), C.c_int, vp]
            L.korg_synthesize_batch_dev.argtypes = [vp, C.c_int32, C.POINTER(BatchItem), vp, C.c_int64, C.c_int, vp]
            L.korg_synthesize_batch_vjp_dev.argtypes = [vp, C.c_int32, C.POINTER(BatchItem), C.POINTER(BatchVjpItem),
                                                        vp, C.c_int64, C.c_int, C.c_int, vp]
            L.korg_set_batch_options.argtypes = [vp, C.c_int, C.c_int, C.c_int64]
            L.korg_set_continuum_tables.argtypes = [vp, C.POINTER(ContinuumTables)]
            L.korg_continuum_absorption.argtypes = [vp, _dp, C.c_int64, C.POINTER(ContinuumLayers), _dp]
            L.korg_continuum_absorption_dev.argtypes = [vp, vp, C.c_int64, C.POINTER(ContinuumLayers), vp, vp]
            L.korg_set_equilibrium_tables.argtypes = [vp, C.POINTER(EquilibriumTables)]
            L.korg_chemical_equilibrium.argtypes = [vp, C.POINTER(ChemLayers), C.c_int32, _dp, _ip, _dp]
            L.korg_chemical_equilibrium_dev.argtypes = [vp, C.POINTER(ChemLayers), C.c_int32, vp, vp, vp, vp]
            L.korg_chemical_equilibrium_vjp.argtypes = [vp, C.POINTER(ChemLayers), C.c_int32, _dp, _dp, _dp, _dp,
                                                        _dp]
            L.korg_chemical_equilibrium_vjp_dev.argtypes = [vp, C.POINTER(ChemLayers), C.c_int32, vp, vp, vp, vp, vp,
                                                            vp, vp]
            L.korg_get_tile_config.argtypes = [vp, C.c_int32, C.c_int, _ip, _ip, _ip, _ip]
            L.korg_set_tile_config.argtypes = [vp, C.c_int32, C.c_int, C.c_int32, C.c_int32, C.c_int32]
            L.korg_device_status.argtypes = [vp]
            L.korg_selftest_wait_timeout.argtypes = [vp, C.c_int]
            lsf = [vp, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, C.c_double]
            L.korg_apply_lsf_dev.argtypes = lsf + [vp, C.c_int32, vp, vp]
            L.korg_apply_lsf_vjp_dev.argtypes = lsf + [vp, C.c_int32, vp, vp]
            L.korg_lsf_windows_dev.argtypes = lsf + [vp, vp, vp]
            L.korg_lsf_matrix_values_dev.argtypes = lsf + [vp, vp, vp]
            rot = [vp, vp, C.c_int64, C.POINTER(WlRange), C.c_int32, C.c_double, C.c_double]
            L.korg_apply_rotation_dev.argtypes = rot + [vp, C.c_int32, vp, vp]
            L.korg_apply_rotation_vjp_dev.argtypes = rot + [vp, C.c_int32, vp, vp]
            _lib = L
    return _lib


def exported_symbols():
    """Names declared in include/korg_gb300.h (checked against the library in the tests)."""
    return ["korg_create", "korg_destroy", "korg_last_error", "korg_get_stats", "korg_set_timing",
            "korg_set_stark_tables", "korg_line_absorption", "korg_line_absorption_dev",
            "korg_hydrogen_line_absorption", "korg_hydrogen_lines_dev", "korg_radiative_transfer",
            "korg_radiative_transfer_dev", "korg_synthesize", "korg_synthesize_dev", "korg_probe_flops",
            "korg_math_selftest", "korg_line_absorption_noalloc", "korg_synthesize_batch_dev",
            "korg_synthesize_batch_vjp_dev", "korg_set_batch_options", "korg_get_tile_config", "korg_set_tile_config", "korg_synthesize_vjp", "korg_synthesize_vjp_dev",
            "korg_radiative_transfer_general", "korg_molecular_cross_section_dev",
            "korg_interpolate_molecular_cross_section_dev", "korg_device_status",
            "korg_selftest_wait_timeout", "korg_apply_lsf_dev", "korg_apply_lsf_vjp_dev", "korg_lsf_windows_dev",
            "korg_lsf_matrix_values_dev", "korg_apply_rotation_dev", "korg_apply_rotation_vjp_dev",
            "korg_set_continuum_tables", "korg_continuum_absorption", "korg_continuum_absorption_dev",
            "korg_set_equilibrium_tables", "korg_chemical_equilibrium", "korg_chemical_equilibrium_dev",
            "korg_chemical_equilibrium_vjp", "korg_chemical_equilibrium_vjp_dev"]


def _p(a, kind=_dp):
    return None if a is None else a.ctypes.data_as(kind)


class Keep:
    """Keeps numpy arrays alive while ctypes structs point into them."""

    def __init__(self):
        self.items = []

    def f64(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.items.append(a)
        return a

    def i32(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.items.append(a)
        return a

    def i64(self, a):
        a = np.ascontiguousarray(a, dtype=np.int64)
        self.items.append(a)
        return a


def lines_struct(ll, keep: Keep) -> Lines:
    return Lines(len(ll), _p(keep.f64(ll.wl)), _p(keep.f64(ll.log_gf)), _p(keep.f64(ll.E_lower)),
                 _p(keep.f64(ll.gamma_rad)), _p(keep.f64(ll.gamma_stark)), _p(keep.f64(ll.vdW1)),
                 _p(keep.f64(ll.vdW2)), _p(keep.f64(ll.mass)), _p(keep.i32(ll.is_mol), _ip),
                 _p(keep.i32(ll.species_idx), _ip))


def stark_struct(st, keep: Keep) -> StarkTables:
    return StarkTables(st["ntrans"], *[_p(keep.i32(st[k]), _ip) for k in ["lower", "upper", "nT", "nNe", "nD"]],
                       *[_p(keep.i64(st[k]), _lp) for k in ["t_off", "ne_off", "d_off", "p_off", "l_off"]],
                       *[_p(keep.f64(st[k])) for k in ["log_gf", "temps", "nes", "logdnu", "logP", "lambda0"]])


class WlRange(C.Structure):
    """korg_wl_range: one uniform wavelength range (points, first wavelength and step in cm)."""
    _fields_ = [("n", C.c_int64), ("start", C.c_double), ("step", C.c_double)]


class Context:
    """One korg_ctx (device, scratch arena, Stark tables)."""

    def __init__(self, device=0):
        self.lib = lib()
        self.h = C.c_void_p()
        rc = self.lib.korg_create(C.byref(self.h), device)
        if rc != 0:
            raise KorgError(rc, "korg_create failed (no usable CUDA device?)")
        self.have_stark = False

    def check(self, rc):
        if rc != 0:
            raise KorgError(rc, self.lib.korg_last_error(self.h).decode())

    def ensure_stark(self):
        if not self.have_stark:
            from .data import stark_profiles
            keep = Keep()
            st = stark_struct(stark_profiles(), keep)
            self.check(self.lib.korg_set_stark_tables(self.h, C.byref(st)))
            self.have_stark = True

    def ensure_continuum(self):
        """Upload the continuum-absorption tables once (korg_set_continuum_tables)."""
        if not getattr(self, "have_continuum", False):
            from .data import continuum_tables
            t, keep = continuum_tables(), Keep()
            f = lambda k: _p(keep.f64(t[k]))
            peach = ("HeII", "CII", "SiII", "MgII")
            ct = ContinuumTables(t["H_bf_E"].shape[1], f("H_bf_E"), f("H_bf_sigma"), len(t["Hminus_bf_nu"]),
                                 f("Hminus_bf_nu"), f("Hminus_bf_sigma"), len(t["Hminus_ff_lambda"]),
                                 len(t["Hminus_ff_theta"]), f("Hminus_ff_lambda"), f("Hminus_ff_theta"),
                                 f("Hminus_ff_K"), len(t["Heminus_ff_lambda"]), len(t["Heminus_ff_theta"]),
                                 f("Heminus_ff_lambda"), f("Heminus_ff_theta"), f("Heminus_ff_K"), len(t["H2plus_T"]),
                                 len(t["H2plus_bf_lambda"]), len(t["H2plus_ff_lambda"]), f("H2plus_T"), f("H2plus_K"),
                                 f("H2plus_bf_lambda"), f("H2plus_bf_sigma"), f("H2plus_ff_lambda"),
                                 f("H2plus_ff_sigma"), len(t["gaunt_log_u"]), len(t["gaunt_log_g2"]),
                                 f("gaunt_log_u"), f("gaunt_log_g2"), f("gaunt_ff"),
                                 (C.c_int32 * 4)(*[len(t[f"peach_{p}_T"]) for p in peach]),
                                 len(t["peach_HeII_sigma"]), (_dp * 4)(*[f(f"peach_{p}_T") for p in peach]),
                                 f("peach_HeII_sigma"), (_dp * 4)(*[f(f"peach_{p}_D") for p in peach]))
            self.check(self.lib.korg_set_continuum_tables(self.h, C.byref(ct)))
            self.have_continuum = True

    def ensure_equilibrium(self, tables=None):
        """Upload chemical-equilibrium tables (korg_set_equilibrium_tables): the default ones once,
        or ``tables`` (a statmech.EquilibriumTables) when they are not the ones already loaded.
        Returns the tables in use."""
        from .statmech import EquilibriumTables as HostTables, default_equilibrium_tables
        t = tables if tables is not None else default_equilibrium_tables()
        if getattr(self, "equilibrium_tables", None) is not t:
            keep = Keep()
            f = lambda a: _p(keep.f64(a))
            i = lambda a: _p(keep.i32(a), _ip)
            et = EquilibriumTables(len(t.lnT), f(t.lnT), f(t.U_u), f(t.U_z), f(t.chi), len(t.molecules), i(t.atoms),
                                   i(t.charge), i(t.kind), _p(keep.i64(t.off), C.POINTER(C.c_int64)), f(t.spl_t),
                                   f(t.spl_u), f(t.spl_z), f(t.D00), f(t.lmr))
            self.check(self.lib.korg_set_equilibrium_tables(self.h, C.byref(et)))
            self.equilibrium_tables = t
        assert isinstance(t, HostTables)
        return t

    def stats(self):
        s = Stats()
        self.check(self.lib.korg_get_stats(self.h, C.byref(s)))
        return s

    def close(self):
        if self.h:
            self.lib.korg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
