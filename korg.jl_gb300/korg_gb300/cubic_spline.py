"""Natural cubic spline, restating Korg's CubicSplines module (src/CubicSplines.jl:33-83).

Korg evaluates partition functions as ``U(ln T)`` with this spline; line_absorption! computes
``n(species) / U(species, ln T)`` per layer (src/line_absorption.jl:42-44) before the line loop.
That host-side precompute is what the CUDA entry points receive as ``n_div_U``.
"""
import numpy as np


class CubicSpline:
    """``CubicSpline(t, u; extrapolate=False)`` (src/CubicSplines.jl:52-63)."""

    def __init__(self, t, u, extrapolate=False):
        t = np.asarray(t, dtype=np.float64)
        u = np.asarray(u, dtype=np.float64)
        n = len(t) - 1
        h = np.concatenate([[0.0], np.diff(t), [0.0]])
        dl = h[1:n + 1]
        d_tmp = 2 * (h[0:n + 1] + h[1:n + 2])
        du = h[1:n + 1]
        d = np.zeros(n + 1)
        for i in range(1, n):  # 0-based; the first and last rows are zero (natural spline)
            d[i] = 6 * (u[i + 1] - u[i]) / h[i + 1] - 6 * (u[i] - u[i - 1]) / h[i]
        self.t, self.u, self.h, self.extrapolate = t, u, h[:n + 1], extrapolate
        self.z = _solve_tridiagonal(dl, d_tmp, du, d)

    def __call__(self, x):
        """Evaluate at scalar or array ``x`` (src/CubicSplines.jl:65-83)."""
        scalar = np.ndim(x) == 0
        x = np.atleast_1d(np.asarray(x, dtype=np.float64))
        t, u, h, z = self.t, self.u, self.h, self.z
        oob = (x < t[0]) | (x > t[-1])
        if oob.any() and not self.extrapolate:
            raise ValueError(f"Out-of-bounds value passed to interpolant. Must be between "
                             f"{t[0]} and {t[-1]}")
        xc = np.clip(x, t[0], t[-1])
        i = np.clip(np.searchsorted(t, xc, side="right") - 1, 0, len(t) - 2)
        h1 = h[i + 1]
        I = z[i] * (t[i + 1] - xc) ** 3 / (6 * h1) + z[i + 1] * (xc - t[i]) ** 3 / (6 * h1)
        C = (u[i + 1] / h1 - z[i + 1] * h1 / 6) * (xc - t[i])
        D = (u[i] / h1 - z[i] * h1 / 6) * (t[i + 1] - xc)
        out = I + C + D
        out = np.where(x < t[0], u[0], np.where(x > t[-1], u[-1], out))
        return float(out[0]) if scalar else out


    def derivative(self, x):
        """d/dx of the spline (zero outside the knots, where the value is clamped)."""
        x = np.atleast_1d(np.asarray(x, dtype=np.float64))
        t, u, h, z = self.t, self.u, self.h, self.z
        xc = np.clip(x, t[0], t[-1])
        i = np.clip(np.searchsorted(t, xc, side="right") - 1, 0, len(t) - 2)
        h1 = h[i + 1]
        d = (-z[i] * (t[i + 1] - xc) ** 2 / (2 * h1) + z[i + 1] * (xc - t[i]) ** 2 / (2 * h1)
             + (u[i + 1] / h1 - z[i + 1] * h1 / 6) - (u[i] / h1 - z[i] * h1 / 6))
        return np.where((x < t[0]) | (x > t[-1]), 0.0, d)


def _solve_tridiagonal(dl, d, du, rhs):
    """Thomas algorithm for the (n+1)x(n+1) system of CubicSplines.jl:58-61."""
    n = len(d)
    c = np.zeros(n)
    g = np.zeros(n)
    b = d.astype(np.float64).copy()
    c_up = np.concatenate([du, [0.0]])
    a_lo = np.concatenate([[0.0], dl])
    c[0] = c_up[0] / b[0]
    g[0] = rhs[0] / b[0]
    for i in range(1, n):
        m = b[i] - a_lo[i] * c[i - 1]
        c[i] = c_up[i] / m if i < n - 1 else 0.0
        g[i] = (rhs[i] - a_lo[i] * g[i - 1]) / m
    x = np.zeros(n)
    x[-1] = g[-1]
    for i in range(n - 2, -1, -1):
        x[i] = g[i] - c[i] * x[i + 1]
    return x
