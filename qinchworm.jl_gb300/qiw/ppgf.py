"""Pseudo-particle Green's function utilities (`src/ppgf.jl`).

P is a list of per-sector ImaginaryTimeGF (data[j] = P_s(tau_j, 0), carrying -i) or of
IncSplineImaginaryTimeGF (incremental quadratic spline interpolation, `src/spline_gf.jl:273-425`).
These run on the host once per inch step: `set_ppgf!` writes P(tau_f), `normalize!`
rescales by exp(-lambda tau); both stay in FP64.
"""
from __future__ import annotations

import math
from typing import List

import numpy as np

from .gf import ImaginaryTimeGF, ImaginaryTimeGrid, IncrementalSpline

# `normalize!` rebuilds the first spline segment with
# derivative_at_0 = der_data[1]/h - 1im*lambda*data[1] (src/ppgf.jl:689).  The spline only
# serves this bookkeeping: the diagram evaluator reads P by linear interpolation of the
# grid data (`kd.interpolate!` on the wrapped GF, src/topology_eval.jl:368), which the
# reference's own fixture test/inchworm.h5 confirms.


def atomic_ppgf(grid: ImaginaryTimeGrid, ed) -> List[ImaginaryTimeGF]:
    """P_s(tau) = -i exp(-tau (E_s + lambda)), lambda = log(Z)/beta (`src/ppgf.jl:128-207`)."""
    beta = grid.beta
    Z = ed.partition_function(beta)
    lam = math.log(Z) / beta
    taus = grid.taus
    P = []
    for E in ed.energies:
        d = len(E)
        data = np.zeros((grid.n_tau, d, d), dtype=np.complex128)
        ex = np.exp(-np.outer(taus, E + lam))
        for k in range(d):
            data[:, k, k] = -1j * ex[:, k]
        P.append(ImaginaryTimeGF(grid, d, True, data))
    return P


def initial_ppgf_derivative(ed, beta: float) -> List[np.ndarray]:
    """dP_s/dtau at tau = 0 (`src/ppgf.jl:706-719`)."""
    Z = sum(np.exp(-beta * E).sum() for E in ed.eigenvalues)
    lam = math.log(Z) / beta
    return [-1j * np.diag(-E - lam) for E in ed.eigenvalues]


class IncSplineImaginaryTimeGF:
    """Matrix-valued GF with one IncrementalSpline per element."""

    def __init__(self, gf: ImaginaryTimeGF, derivative_at_0: np.ndarray):
        self.GF = gf
        self.grid = gf.grid
        self.norb = gf.norb
        self.xi = gf.xi
        self._make(np.asarray(derivative_at_0, dtype=np.complex128))

    def _make(self, der0):
        h = self.grid.step
        self.interpolants = [[IncrementalSpline(h, self.grid.n_tau, self.GF.data[0, k, l], der0[k, l])
                              for l in range(self.norb)] for k in range(self.norb)]

    @property
    def data(self):
        return self.GF.data

    @property
    def n_valid(self) -> int:
        return len(self.interpolants[0][0].data)

    def extend(self, val: np.ndarray):
        for k in range(self.norb):
            for l in range(self.norb):
                self.interpolants[k][l].extend(val[k, l])
        self.GF.data[self.n_valid - 1] = val

    def der0(self) -> np.ndarray:
        """derivative_at_0 of every element, as passed to the first segment."""
        h = self.grid.step
        return np.array([[self.interpolants[k][l].der_data[0] / h for l in range(self.norb)]
                         for k in range(self.norb)])

    def normalize(self, lam: float):
        n = self.n_valid
        taus = self.grid.taus
        self.GF.data[:n] *= np.exp(-taus[:n] * lam)[:, None, None]
        h = self.grid.step
        old = self.interpolants
        der0 = np.zeros((self.norb, self.norb), dtype=np.complex128)
        for k in range(self.norb):
            for l in range(self.norb):
                it = old[k][l]
                der0[k, l] = it.der_data[0] / h - 1j * lam * it.data[0]
        self._make(der0)
        for j in range(1, n):
            for k in range(self.norb):
                for l in range(self.norb):
                    self.interpolants[k][l].extend(self.GF.data[j, k, l])


def set_ppgf(P, j_f: int, val) -> None:
    """P[s](tau_{j_f}, 0) = val[s] (`src/ppgf.jl:474-504`); j_f is 0-based."""
    for s, (sf, mat) in val.items():
        assert s == sf, "Boldification must preserve the block structure"
        if isinstance(P[s], IncSplineImaginaryTimeGF):
            assert P[s].n_valid == j_f, "incremental spline must be extended in order"
            P[s].extend(mat)
        else:
            P[s].data[j_f] = mat


def _normalize_sector(P_s, lam: float):
    if isinstance(P_s, IncSplineImaginaryTimeGF):
        P_s.normalize(lam)
    else:
        P_s.data *= np.exp(-P_s.grid.taus * lam)[:, None, None]


def partition_function(P) -> complex:
    """Z = Tr[i P(beta, 0)] (`src/ppgf.jl:611-617`)."""
    return complex(sum(1j * np.trace(P_s.data[-1]) for P_s in P))


def normalize_beta(P, beta: float) -> float:
    """normalize!(P, beta): Tr[i P(beta)] = 1 (`src/ppgf.jl:629-636`)."""
    Z = partition_function(P)
    lam = (np.log(Z) / beta)
    lam = float(np.real(lam)) if abs(np.imag(lam)) == 0 else lam
    for P_s in P:
        _normalize_sector(P_s, lam)
    return lam


def normalize_tau(P, j: int) -> float:
    """normalize!(P, tau_j): max_s,i -Im P_s,ii(tau_j) = 1 (`src/ppgf.jl:646-654`)."""
    tau = P[0].grid.tau(j)
    P_max = max(float(np.max(-np.imag(np.diag(P_s.data[j])))) for P_s in P)
    lam = math.log(P_max) / tau
    for P_s in P:
        _normalize_sector(P_s, lam)
    return lam


def density_matrix(P) -> List[np.ndarray]:
    return [1j * P_s.data[-1] for P_s in P]
