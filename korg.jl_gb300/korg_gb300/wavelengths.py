"""Wavelength grids, restating ``Korg.Wavelengths`` (src/wavelengths.jl:29-210).

A grid is a list of uniform ranges (in cm internally).  Korg builds each range as a Julia
``StepRangeLen`` with twice-precision reference and step and then scales Angstrom ranges by
1e-8; element values are therefore the correctly rounded results of exact arithmetic.  This
module reproduces that with vectorised double-double arithmetic (Dekker/Veltkamp products and
Knuth two-sums in plain IEEE double operations, so the grid is identical on x86 and Arm).

``searchsortedfirst`` / ``searchsortedlast`` return 0-based indices with the semantics of
src/wavelengths.jl:188-210 (the first element >= x, the last element <= x).
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np

_SPLIT = 134217729.0  # 2**27 + 1


def _two_sum(a, b):
    s = a + b
    bb = s - a
    e = (a - (s - bb)) + (b - bb)
    return s, e


def _split(a):
    c = _SPLIT * a
    hi = c - (c - a)
    return hi, a - hi


def _two_prod(a, b):
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def _dd_from_fraction(fr: Fraction):
    hi = float(fr)
    lo = float(fr - Fraction(hi))
    return hi, lo


def _julia_rat(x: float):
    """Julia's Base.rat: the continued-fraction convergent a/b with float(a/b) == x, giving up
    when numerator or denominator exceed maxintfloat(Float32)."""
    y = x
    a, d = 1, 1
    b, c = 0, 0
    m = 16777216
    while abs(y) <= m:
        f = int(np.trunc(y))
        y -= f
        a, c = f * a + c, a
        b, d = f * b + d, b
        if max(abs(a), abs(b)) > m:
            return c, d
        if b != 0 and a / b == x:
            break
        if y == 0:
            break
        y = 1.0 / y
    return a, b


def _range_values(start: float, step: float, stop: float, scale: float | None):
    """Element values of Julia's ``start:step:stop`` (optionally times ``scale``)."""
    sn, sd = _julia_rat(start)
    tn, td = _julia_rat(step)
    en, ed = _julia_rat(stop)
    rational = (sd != 0 and td != 0 and ed != 0 and sn / sd == start and tn / td == step
                and en / ed == stop)
    if rational:
        den = np.lcm.reduce([sd, td, ed])
        a = sn * (den // sd)
        st = tn * (den // td)
        b = en * (den // ed)
        n = (b - a) // st + 1
        k = np.arange(n, dtype=np.float64)
        # value_k = (a + k*st)/den  as double-double: exact numerator (integers < 2**53)
        num = a + k * st
        hi = num / den
        p, e = _two_prod(hi, np.full_like(hi, float(den)))
        lo = ((num - p) - e) / den
    else:
        n = int(np.floor((stop - start) / step + 1 + 1e-10))
        k = np.arange(n, dtype=np.float64)
        p, e = _two_prod(k, np.full_like(k, step))
        hi, lo2 = _two_sum(np.full_like(k, start), p)
        lo = lo2 + e
        hi, lo = _two_sum(hi, lo)
    if scale is None:
        return hi + lo
    p, e = _two_prod(hi, np.full_like(hi, scale))
    e = e + lo * scale
    return p + e


class Wavelengths:
    """``Korg.Wavelengths``: one or more uniform ranges.

    Accepts ``(start, stop)``, ``(start, stop, step)`` or a list of such tuples, in Angstrom
    (values >= 1) or cm (values < 1), with Korg's default 0.01 A step.  ``all_wls`` holds every
    grid point in cm; ``ranges`` holds ``(start_cm, step_cm, n)`` per range.
    """

    def __init__(self, spec):
        if isinstance(spec, Wavelengths):
            self.__dict__.update(spec.__dict__)
            return
        if isinstance(spec, tuple):
            spec = [spec]
        ranges, pieces = [], []
        for t in spec:
            if not 2 <= len(t) <= 3:
                raise ValueError("Each wavelength range must be (start, stop) or (start, stop, step)")
            start, stop = float(t[0]), float(t[1])
            step = float(t[2]) if len(t) == 3 else (1e-10 if start < 1 else 0.01)
            if start >= 1:
                vals = _range_values(start, step, stop, 1e-8)
            else:
                vals = _range_values(start, step, stop, None)
            if len(vals) == 0:
                raise ValueError("empty wavelength range")
            pieces.append(vals)
            ranges.append((float(vals[0]), (float(vals[-1]) - float(vals[0])) / max(len(vals) - 1, 1),
                           len(vals)))
        all_wls = np.concatenate(pieces)
        if np.any(np.diff(all_wls) < 0):
            raise ValueError("wl_ranges must be sorted and non-overlapping")
        self.all_wls = all_wls
        self.ranges = ranges
        self.all_freqs = (2.99792458e10 / all_wls)[::-1].copy()

    @classmethod
    def from_array(cls, wls_cm):
        """A grid given directly as an increasing array of wavelengths in cm."""
        self = cls.__new__(cls)
        self.all_wls = np.ascontiguousarray(wls_cm, dtype=np.float64)
        self.ranges = [(float(self.all_wls[0]), 0.0, len(self.all_wls))]
        self.all_freqs = (2.99792458e10 / self.all_wls)[::-1].copy()
        return self

    def __len__(self):
        return len(self.all_wls)

    def __getitem__(self, i):
        return self.all_wls[i]

    def __array__(self, dtype=None, copy=None):
        return self.all_wls if dtype is None else self.all_wls.astype(dtype)

    def eachwindow(self):
        """(first, last) of each range in cm (src/wavelengths.jl:159)."""
        out, i = [], 0
        for _, _, n in self.ranges:
            out.append((float(self.all_wls[i]), float(self.all_wls[i + n - 1])))
            i += n
        return out

    @property
    def all_wls_angstrom(self):
        """every grid point in Angstrom (computed once, shared read-only)"""
        a = self.__dict__.get("_all_wls_A")
        if a is None or len(a) != len(self.all_wls):
            a = self.all_wls * 1e8
            a.flags.writeable = False
            self.__dict__["_all_wls_A"] = a
        return a

    def subspectrum_indices(self):
        out, i = [], 0
        for _, _, n in self.ranges:
            out.append(range(i, i + n))
            i += n
        return out

    def searchsortedfirst(self, x):
        x = x * 1e-8 if x >= 1 else x
        return int(np.searchsorted(self.all_wls, x, side="left"))

    def searchsortedlast(self, x):
        x = x * 1e-8 if x >= 1 else x
        return int(np.searchsorted(self.all_wls, x, side="right")) - 1
