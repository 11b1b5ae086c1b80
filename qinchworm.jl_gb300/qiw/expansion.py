"""Pseudo-particle strong-coupling expansion problem (`src/expansion.jl:107-310`).

`Expansion` gathers what the diagram evaluator reads: the exact atomic propagator P0
(`src/exact_atomic_ppgf.jl:109-135`), the bold propagator P on the imaginary-time grid
(`src/ppgf.jl:128-207`), the interaction pairs (operator_f, operator_i, propagator), the
block matrices of their operators, of the identity and of the correlator operators, and
`subspace_attachable_pairs` (`:184-187`).  Sector indices are 0-based here.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np

from .ed import EDCore, SectorBlockMatrix
from .gf import ImaginaryTimeGF, ImaginaryTimeGrid, SplineInterpolatedGF
from .operators import OperatorExpr
from . import ppgf as _ppgf


@dataclass
class InteractionPair:
    """operator_f at the later (tail) time, operator_i at the earlier (head) time."""
    operator_f: OperatorExpr
    operator_i: OperatorExpr
    propagator: Union[ImaginaryTimeGF, SplineInterpolatedGF]

    def __getitem__(self, idx: int):
        return [self.operator_i, self.operator_f][idx - 1]


class ExactAtomicPPGF:
    """P0_s(tau) = -i exp(-tau (E_s + lambda)) (diagonal)."""

    def __init__(self, beta: float, E: np.ndarray):
        self.beta = beta
        self.E = np.asarray(E, dtype=np.float64)

    def __call__(self, dtau: float) -> np.ndarray:
        return -1j * np.diag(np.exp(-dtau * self.E))


class Expansion:
    def __init__(self, ed: EDCore, grid: ImaginaryTimeGrid, interaction_pairs: Sequence[InteractionPair],
                 corr_operators: Sequence[Tuple[OperatorExpr, OperatorExpr]] = (),
                 interpolate_ppgf: bool = False):
        self.ed = ed
        self.grid = grid
        beta = grid.beta
        Z = ed.partition_function(beta)
        lam = np.log(Z) / beta
        self.P0 = [ExactAtomicPPGF(beta, E + lam) for E in ed.energies]
        self.P = _ppgf.atomic_ppgf(grid, ed)
        self.interpolate_ppgf = interpolate_ppgf
        if interpolate_ppgf:
            dP = _ppgf.initial_ppgf_derivative(ed, beta)
            self.P = [_ppgf.IncSplineImaginaryTimeGF(P_s, dP_s) for P_s, dP_s in zip(self.P, dP)]
        self.pairs: List[InteractionPair] = list(interaction_pairs)
        self.corr_operators: List[Tuple[OperatorExpr, OperatorExpr]] = []
        self.identity_mat = ed.operator_blocks(OperatorExpr.scalar(1.0))
        self.pair_operator_mat = [(ed.operator_blocks(p.operator_i), ed.operator_blocks(p.operator_f))
                                  for p in self.pairs]
        self.corr_operators_mat: List[Tuple[SectorBlockMatrix, SectorBlockMatrix]] = []
        for ops in corr_operators:
            self.add_corr_operators(ops)
        self.subspace_attachable_pairs = [
            [p for p, (oi, of) in enumerate(self.pair_operator_mat) if s in oi]
            for s in range(ed.n_sectors)
        ]

    def add_corr_operators(self, ops: Tuple[OperatorExpr, OperatorExpr]):
        """`add_corr_operators!` (`src/expansion.jl:303-310`)."""
        self.corr_operators.append(ops)
        self.corr_operators_mat.append((self.ed.operator_blocks(ops[0]), self.ed.operator_blocks(ops[1])))

    @property
    def n_sectors(self) -> int:
        return self.ed.n_sectors

    @property
    def dims(self) -> List[int]:
        return self.ed.dims


def expansion_from_hybridization(hamiltonian: OperatorExpr, soi, grid: ImaginaryTimeGrid,
                                 hybridization: List[List[Optional[ImaginaryTimeGF]]],
                                 corr_operators=(), interpolate_ppgf: bool = False,
                                 spline_delta: bool = False) -> Expansion:
    """Higher-level constructor (`src/expansion.jl:222-291`) from a matrix of scalar
    hybridization functions Delta_ij(tau) (None for zero entries)."""
    from .operators import c, c_dag
    from .gf import ph_conj
    pairs: List[InteractionPair] = []
    breakers: List[OperatorExpr] = []
    labels = list(soi)
    for i1, l1 in enumerate(labels):
        for i2, l2 in enumerate(labels):
            D = hybridization[i1][i2]
            if D is None or not np.any(D.data):
                continue
            D_rev = ph_conj(D)
            P1 = SplineInterpolatedGF(D) if spline_delta else D
            P2 = SplineInterpolatedGF(D_rev) if spline_delta else D_rev
            pairs.append(InteractionPair(c_dag(l1), c(l2), P1))
            pairs.append(InteractionPair(c(l2), c_dag(l1), P2))
            breakers.append(c_dag(l1) * c(l2))
            breakers.append(c(l2) * c_dag(l1))
    ed = EDCore(hamiltonian, soi, symmetry_breakers=breakers)
    return Expansion(ed, grid, pairs, corr_operators=corr_operators, interpolate_ppgf=interpolate_ppgf)
