"""Impurity models of the benchmark configurations, built as `Expansion` objects.

These are synthetic inputs in the reference's own parametrisation: the README Anderson
model (`README.md:51-99`), the Kanamori Hamiltonian of
`bench/two_band_eg_model_discrete_bath/two_band_eg_model_discrete_bath.jl:36-56`, the
single-level model of the reference's `test/inchworm.jl:55-212` fixture, and the two dimers
that the reference checks against exact diagonalisation (`test/dimers.jl`).
"""
from __future__ import annotations

from typing import List

import numpy as np

from . import operators as op
from .ed import EDCore
from .expansion import Expansion, InteractionPair
from .gf import (BetheDOS, DeltaDOS, ImaginaryTimeGrid, SplineInterpolatedGF, gf_from_dos,
                 ph_conj)


def _diag_pairs(labels, deltas, spline: bool = False) -> List[InteractionPair]:
    pairs = []
    for l, D in zip(labels, deltas):
        Dr = ph_conj(D)
        pairs.append(InteractionPair(op.c_dag(l), op.c(l), SplineInterpolatedGF(D) if spline else D))
        pairs.append(InteractionPair(op.c(l), op.c_dag(l), SplineInterpolatedGF(Dr) if spline else Dr))
    return pairs


def anderson(eps: float = 0.1, U: float = 1.0, D: float = 2.0, V: float = 0.5, beta: float = 10.0,
             n_tau: int = 200, corr: bool = False) -> Expansion:
    """Single-orbital Anderson impurity with a semi-elliptic bath (README.md:51-99)."""
    H = eps * (op.n("up") + op.n("dn")) + U * op.n("up") * op.n("dn")
    soi = op.SetOfIndices([["up"], ["dn"]])
    ed = EDCore(H, soi)
    grid = ImaginaryTimeGrid(beta, n_tau)
    Delta = V ** 2 * gf_from_dos(BetheDOS(t=D / 2), grid)
    pairs = _diag_pairs([("up",), ("dn",)], [Delta, Delta])
    exp = Expansion(ed, grid, pairs)
    if corr:
        exp.add_corr_operators((-op.c("up"), op.c_dag("up")))
        exp.add_corr_operators((op.n("up"), op.n("dn")))
        exp.add_corr_operators((op.c_dag("up") * op.c("dn"), op.c_dag("dn") * op.c("up")))
    return exp


def single_level(beta: float = 10.0, mu: float = 0.1, eps: float = 0.1, V: float = -0.1,
                 n_tau: int = 20, spline: bool = True) -> Expansion:
    """H = -mu n coupled to one bath level (test/inchworm.jl:55-212)."""
    H = -mu * op.n("0")
    soi = op.SetOfIndices([["0"]])
    ed = EDCore(H, soi)
    grid = ImaginaryTimeGrid(beta, n_tau)
    Delta = V ** 2 * gf_from_dos(DeltaDOS.make([eps]), grid)
    return Expansion(ed, grid, _diag_pairs([("0",)], [Delta], spline=spline), interpolate_ppgf=spline)


def dimer(beta: float = 1.0, eps_1: float = 0.5, eps_2: float = 2.0, V: float = 0.5,
          n_tau: int = 32, spline: bool = False) -> Expansion:
    """Level 1 (H = eps_1 n_1) hybridised with one bath level eps_2 (test/dimers.jl:35-90);
    ``spline`` selects the SplineInterpolatedGF / interpolate_ppgf variant of :68-72."""
    ed = EDCore(eps_1 * op.n(1), op.SetOfIndices([[1]]))
    grid = ImaginaryTimeGrid(beta, n_tau)
    Delta = V ** 2 * gf_from_dos(DeltaDOS.make([eps_2]), grid)
    return Expansion(ed, grid, _diag_pairs([(1,)], [Delta], spline=spline), interpolate_ppgf=spline)


def hubbard_dimer(beta: float = 1.0, U: float = 4.0, eps_2: float = 0.0, V: float = 0.5,
                  n_tau: int = 32) -> Expansion:
    """Hubbard atom at half filling (eps_1 = -U/2) with one bath level per spin
    (test/dimers.jl:118-175)."""
    eps_1 = -0.5 * U
    H = U * op.n(1) * op.n(2) + eps_1 * (op.n(1) + op.n(2))
    ed = EDCore(H, op.SetOfIndices([[1], [2]]))
    grid = ImaginaryTimeGrid(beta, n_tau)
    Delta = V ** 2 * gf_from_dos(DeltaDOS.make([eps_2]), grid)
    return Expansion(ed, grid, _diag_pairs([(1,), (2,)], [Delta, Delta]))


def kanamori_hamiltonian(n_orb: int, mu: float, U: float, J: float):
    """bench/two_band_eg_model_discrete_bath/two_band_eg_model_discrete_bath.jl:36-56."""
    labels = [(s, o) for s in ("up", "dn") for o in range(1, n_orb + 1)]
    soi = op.SetOfIndices(labels)
    orbs = range(1, n_orb + 1)
    H = op.OperatorExpr()
    H += -mu * sum((op.n("up", o) + op.n("dn", o) for o in orbs), op.OperatorExpr())
    H += U * sum((op.n("up", o) * op.n("dn", o) for o in orbs), op.OperatorExpr())
    H += (U - 2 * J) * sum((op.n("up", o1) * op.n("dn", o2) for o1 in orbs for o2 in orbs if o1 != o2),
                           op.OperatorExpr())
    H += (U - 3 * J) * sum((op.n(s, o1) * op.n(s, o2) for s in ("up", "dn") for o1 in orbs for o2 in orbs if o2 < o1),
                           op.OperatorExpr())
    H += -J * sum((op.c_dag("up", o1) * op.c_dag("dn", o1) * op.c("up", o2) * op.c("dn", o2)
                   for o1 in orbs for o2 in orbs if o1 != o2), op.OperatorExpr())
    H += -J * sum((op.c_dag("up", o1) * op.c_dag("dn", o2) * op.c("up", o2) * op.c("dn", o1)
                   for o1 in orbs for o2 in orbs if o1 != o2), op.OperatorExpr())
    return soi, labels, H


def orbital_mixing_breakers(n_orb: int):
    """Symmetry breakers that leave only (N_up, N_dn) conserved, as the reference's eg bench
    passes to EDCore (two_band_eg_model_discrete_bath.jl:76-79)."""
    br = []
    for s in ("up", "dn"):
        for o1 in range(1, n_orb + 1):
            for o2 in range(o1 + 1, n_orb + 1):
                br.append(op.c_dag(s, o1) * op.c(s, o2) + op.c_dag(s, o2) * op.c(s, o1))
    return br


def eg_discrete_bath(U: float = 2.0, J: float = 0.2, beta: float = 8.0, n_tau: int = 256,
                     n_bath: int = 4, V: float = 0.5, corr: bool = False) -> Expansion:
    """Two-orbital eg Kanamori model, eps_d = -U/2, 4 bath levels per spin-orbital on [-1, 1];
    (N_up, N_dn) sectors, largest 4 x 4."""
    soi, labels, H = kanamori_hamiltonian(2, mu=U / 2, U=U, J=J)
    ed = EDCore(H, soi, symmetry_breakers=orbital_mixing_breakers(2))
    grid = ImaginaryTimeGrid(beta, n_tau)
    e_k = np.linspace(-1.0, 1.0, n_bath)
    Delta = gf_from_dos(DeltaDOS.make(e_k, [V ** 2] * n_bath), grid)
    exp = Expansion(ed, grid, _diag_pairs(labels, [Delta] * len(labels)))
    if corr:
        for l in labels:
            exp.add_corr_operators((op.c(*l), op.c_dag(*l)))
    return exp


def t2g_bethe(U: float = 2.3, J: float = 0.4, beta: float = 20.0, n_tau: int = 512, D: float = 2.0,
              V: float = 0.4, corr: bool = False) -> Expansion:
    """Three-orbital t2g Kanamori model at half filling with a semi-elliptic bath."""
    mu = 2.5 * U - 5.0 * J
    soi, labels, H = kanamori_hamiltonian(3, mu=mu, U=U, J=J)
    ed = EDCore(H, soi, symmetry_breakers=orbital_mixing_breakers(3))
    grid = ImaginaryTimeGrid(beta, n_tau)
    Delta = V ** 2 * gf_from_dos(BetheDOS(t=D / 2), grid)
    exp = Expansion(ed, grid, _diag_pairs(labels, [Delta] * len(labels)))
    if corr:
        # G(tau) and <S+(tau) S-> of orbital 1; correlator_2p takes single monomials only
        # (src/inchworm.jl:1003-1004), as in README.md:132-137
        exp.add_corr_operators((-op.c("up", 1), op.c_dag("up", 1)))
        exp.add_corr_operators((op.c_dag("up", 1) * op.c("dn", 1), op.c_dag("dn", 1) * op.c("up", 1)))
    return exp
