"""Imaginary-time grids and Green's function containers used as evaluator inputs.

Keldysh.jl conventions are kept (the reference's call sites: `README.md:60-81`,
`src/expansion.jl:241-248`, `src/spline_gf.jl`): a contour GF carries the factor -i,
G(tau) = -i <T c(tau) c^dag(0)>, so on the imaginary branch i*G is real.  A GF is stored
on the uniform grid tau_j = j*beta/(n_tau-1), j = 0..n_tau-1, as data[j, k, l] = G_kl(tau_j, 0).

Interpolation rules between grid points (the reference delegates them to Keldysh.jl and
Interpolations.jl, which are not available here) are defined once in this module and
reproduced bit-for-bit in the CUDA library and in the CPU oracle:

* ``linear``  -- x = dtau/h, i = min(floor(x), n_tau-2), f = x - i,
  G = d[i] + f*(d[i+1] - d[i]);
* ``cubic``   -- natural cubic spline through the grid values
  (Interpolations.jl ``BSpline(Cubic(Line(OnGrid())))``, `src/spline_gf.jl:195-202`);
* ``incremental quadratic`` -- `IncrementalSpline` of `src/utility.jl:106-157` for P.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class ImaginaryTimeGrid:
    beta: float
    n_tau: int

    @property
    def step(self) -> float:
        return self.beta / (self.n_tau - 1)

    @property
    def taus(self) -> np.ndarray:
        return np.arange(self.n_tau, dtype=np.float64) * self.step

    def __len__(self):
        return self.n_tau

    def tau(self, j: int) -> float:
        """0-based grid point."""
        return j * self.step


class ImaginaryTimeGF:
    """Matrix-valued (norb x norb) or scalar imaginary-time GF on a uniform grid."""

    def __init__(self, grid: ImaginaryTimeGrid, norb: int = 1, fermionic: bool = True,
                 data: np.ndarray | None = None):
        self.grid = grid
        self.norb = norb
        self.xi = -1 if fermionic else 1
        if data is None:
            data = np.zeros((grid.n_tau, norb, norb), dtype=np.complex128)
        self.data = np.asarray(data, dtype=np.complex128).reshape(grid.n_tau, norb, norb)

    def copy(self):
        g = ImaginaryTimeGF(self.grid, self.norb, self.xi == -1, self.data.copy())
        return g

    def __mul__(self, x):
        return ImaginaryTimeGF(self.grid, self.norb, self.xi == -1, self.data * x)

    __rmul__ = __mul__

    def scalar_data(self) -> np.ndarray:
        return self.data[:, 0, 0]

    def __call__(self, dtau: float) -> complex:
        """Linear interpolation at dtau in [0, beta] (scalar GF)."""
        return linear_interp(self.data[:, 0, 0], self.grid.step, dtau)


def linear_interp(d: np.ndarray, h: float, dtau: float):
    n = d.shape[0]
    x = dtau / h
    i = int(math.floor(x))
    i = min(max(i, 0), n - 2)
    f = x - i
    return d[i] + f * (d[i + 1] - d[i])


# --------------------------------------------------------------------------- DOS -> GF

@dataclass(frozen=True)
class BetheDOS:
    """Semi-elliptic DOS with half-bandwidth 2t centred at eps (Keldysh.bethe_dos)."""
    t: float = 1.0
    eps: float = 0.0


@dataclass(frozen=True)
class DeltaDOS:
    """Sum of delta peaks, weights w_k at energies e_k (Keldysh.DeltaDOS)."""
    energies: tuple
    weights: tuple

    @staticmethod
    def make(energies, weights=None):
        energies = tuple(float(e) for e in np.atleast_1d(energies))
        if weights is None:
            weights = (1.0,) * len(energies)
        return DeltaDOS(energies, tuple(float(w) for w in np.atleast_1d(weights)))


def _greater_kernel(eps: np.ndarray, tau: np.ndarray, beta: float) -> np.ndarray:
    """(1 - n_F(eps)) * exp(-eps*tau) for 0 <= tau <= beta, evaluated without overflow."""
    eps = np.asarray(eps, dtype=np.float64)[None, :]
    tau = np.asarray(tau, dtype=np.float64)[:, None]
    pos = eps >= 0
    out_pos = np.exp(-eps * tau) / (1.0 + np.exp(-beta * np.abs(eps)))
    out_neg = np.exp(eps * (beta - tau)) / (1.0 + np.exp(-beta * np.abs(eps)))
    return np.where(pos, out_pos, out_neg)


def gf_from_dos(dos, grid: ImaginaryTimeGrid, n_quad: int = 4096) -> ImaginaryTimeGF:
    """G(tau) = -i * int d(eps) A(eps) (1 - n_F(eps)) exp(-eps*tau) on the grid."""
    taus = grid.taus
    if isinstance(dos, DeltaDOS):
        e = np.array(dos.energies)
        w = np.array(dos.weights)
        vals = _greater_kernel(e, taus, grid.beta) @ w
    elif isinstance(dos, BetheDOS):
        # Gauss-Chebyshev quadrature of the second kind for the sqrt(D^2-eps^2) weight.
        D = 2.0 * dos.t
        k = np.arange(1, n_quad + 1)
        theta = k * np.pi / (n_quad + 1)
        x = np.cos(theta)
        w = (2.0 / (n_quad + 1)) * np.sin(theta) ** 2
        vals = _greater_kernel(dos.eps + D * x, taus, grid.beta) @ w
    else:
        raise TypeError(f"unsupported DOS {dos!r}")
    return ImaginaryTimeGF(grid, 1, True, (-1j * vals).reshape(-1, 1, 1))


def ph_conj(g: ImaginaryTimeGF) -> ImaginaryTimeGF:
    """g(beta - tau) on the grid (`src/utility.jl:210-217`)."""
    return ImaginaryTimeGF(g.grid, g.norb, g.xi == -1, g.data[::-1].copy())


# --------------------------------------------------------------------------- splines

def natural_cubic_second_derivatives(y: np.ndarray, h: float) -> np.ndarray:
    """Second derivatives M_j of the natural cubic spline through (j*h, y_j)."""
    y = np.asarray(y)
    n = y.shape[0]
    M = np.zeros_like(y)
    if n < 3:
        return M
    # (M_{j-1} + 4 M_j + M_{j+1}) = 6 (y_{j+1} - 2 y_j + y_{j-1}) / h^2, M_0 = M_{n-1} = 0
    m = n - 2
    rhs = 6.0 * (y[2:] - 2.0 * y[1:-1] + y[:-2]) / (h * h)
    a = np.ones(m - 1)
    b = np.full(m, 4.0)
    c = np.ones(m - 1)
    # Thomas algorithm
    cp = np.zeros(m - 1)
    dp = np.zeros(m, dtype=y.dtype)
    if m == 1:
        M[1] = rhs[0] / 4.0
        return M
    cp[0] = c[0] / b[0]
    dp[0] = rhs[0] / b[0]
    for i in range(1, m):
        den = b[i] - a[i - 1] * cp[i - 1]
        if i < m - 1:
            cp[i] = c[i] / den
        dp[i] = (rhs[i] - a[i - 1] * dp[i - 1]) / den
    x = np.zeros(m, dtype=y.dtype)
    x[-1] = dp[-1]
    for i in range(m - 2, -1, -1):
        x[i] = dp[i] - cp[i] * x[i + 1]
    M[1:-1] = x
    return M


def cubic_segment_coeffs(y: np.ndarray, h: float) -> np.ndarray:
    """Per-segment polynomial S_j(t) = a0 + a1 t + a2 t^2 + a3 t^3, t = (x - x_j)/h."""
    y = np.asarray(y)
    M = natural_cubic_second_derivatives(y, h)
    h2 = h * h
    y0, y1 = y[:-1], y[1:]
    M0, M1 = M[:-1], M[1:]
    a0 = y0
    a1 = (y1 - y0) - h2 * (2.0 * M0 + M1) / 6.0
    a2 = h2 * M0 / 2.0
    a3 = h2 * (M1 - M0) / 6.0
    return np.stack([a0, a1, a2, a3], axis=-1)


class SplineInterpolatedGF:
    """Natural cubic spline wrapper of a scalar GF (`src/spline_gf.jl:65-241`)."""

    def __init__(self, gf: ImaginaryTimeGF):
        self.GF = gf
        self.grid = gf.grid
        self.M = natural_cubic_second_derivatives(gf.data[:, 0, 0], gf.grid.step)

    def __call__(self, dtau: float):
        y = self.GF.data[:, 0, 0]
        h = self.grid.step
        n = y.shape[0]
        x = dtau / h
        j = min(max(int(math.floor(x)), 0), n - 2)
        t = x - j
        return ((1 - t) * y[j] + t * y[j + 1]
                + h * h / 6.0 * (((1 - t) ** 3 - (1 - t)) * self.M[j] + (t ** 3 - t) * self.M[j + 1]))


class IncrementalSpline:
    """Quadratic spline built one knot at a time (`src/utility.jl:106-157`)."""

    def __init__(self, h: float, n_knots: int, val1, der1):
        self.h = h
        self.n_knots = n_knots
        self.data = [val1]
        self.der_data = [der1 * h]

    def extend(self, val):
        self.data.append(val)
        self.der_data.append(2 * (self.data[-1] - self.data[-2]) - self.der_data[-1])

    def __call__(self, z):
        x = 1 + z / self.h
        i = int(math.floor(x))
        i = min(i, len(self.data) - 1)
        dx = x - i
        d0 = self.data[i - 1]
        d1 = self.data[i]
        c3 = self.der_data[i - 1] - 2 * d1
        return d0 * (1 - dx ** 2) + d1 * (1 - (1 - dx) ** 2) + c3 * (0.25 - (dx - 0.5) ** 2)
