"""GB300-native (sm_103a) spectral-synthesis hot path with Korg.jl's interface.

The CUDA kernels live in ``libkorg_gb300.so`` (built from ``csrc/`` by ``build.py``); this
package is the host side: wavelength grids, line lists, the host precompute that Korg does
before its hot path, and Python mirrors of ``line_absorption!``,
``hydrogen_line_absorption!``, ``radiative_transfer`` and ``synthesize``.
"""
from .wavelengths import Wavelengths
from .linelist import LineList, make_line, filter_linelist, alpha_5000_linelist
from .species import Species, parse_species
from .cubic_spline import CubicSpline

__all__ = ["Wavelengths", "LineList", "make_line", "filter_linelist", "alpha_5000_linelist", "Species",
           "parse_species", "CubicSpline", "line_absorption_", "hydrogen_line_absorption_",
           "radiative_transfer", "synthesize", "prepare_synthesis", "synthesize_prepared"]


_API = ("line_absorption_", "hydrogen_line_absorption_", "radiative_transfer", "synthesize", "prepare_synthesis",
        "synthesize_prepared", "SynthesisInputs", "SynthesisResult", "ContinuumInterpolant", "synthesize_vjp",
        "loss_and_gradient", "physical_gradient", "atmosphere_gradient")


_STATMECH = ("chemical_equilibrium", "saha_ion_weights", "translational_U", "get_log_nK", "Hminus_nK",
             "ChemicalEquilibriumError")


def __getattr__(name):
    # the API modules (which load the CUDA library binding on first call) are imported on first use
    import importlib
    if name in _API:
        return getattr(importlib.import_module(".api", __name__), name)
    if name in _STATMECH:
        return getattr(importlib.import_module(".statmech", __name__), name)
    raise AttributeError(name)
