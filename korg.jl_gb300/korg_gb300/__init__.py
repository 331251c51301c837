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


def __getattr__(name):
    # the API module is imported on first use (it loads the CUDA library binding); importing it
    # binds the package attribute `synthesize` to the module, whose synthesize() is the function
    if name in ("line_absorption_", "hydrogen_line_absorption_", "radiative_transfer", "synthesize",
                "prepare_synthesis", "synthesize_prepared", "SynthesisInputs", "SynthesisResult",
                "ContinuumInterpolant", "synthesize_vjp", "loss_and_gradient", "physical_gradient"):
        import importlib
        _s = importlib.import_module(".synthesize", __name__)
        return _s if name == "synthesize" else getattr(_s, name)
    raise AttributeError(name)
