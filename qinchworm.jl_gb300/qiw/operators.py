"""Fermionic many-body operator expressions acting on a finite Fock space.

This is the input-side counterpart of KeldyshED.Operators as used by the reference
(`op.c`, `op.c_dag`, `op.n`, sums and products of monomials with real coefficients;
`src/expansion.jl:42` binds `Operator = op.RealOperatorExpr`). It only has to produce
the matrices that the diagram evaluator consumes, so it stays small: an expression is a
dictionary monomial -> coefficient, and a monomial is a tuple of (dagger, label) factors
read left to right.
"""
from __future__ import annotations

from typing import Dict, Iterable, List, Sequence, Tuple

import numpy as np

Label = Tuple
Factor = Tuple[bool, Label]          # (is_creation, label)
Monomial = Tuple[Factor, ...]


def _as_label(args) -> Label:
    if len(args) == 1 and isinstance(args[0], tuple):
        return args[0]
    return tuple(args)


class OperatorExpr:
    """Linear combination of products of creation/annihilation operators."""

    __slots__ = ("terms",)

    def __init__(self, terms: Dict[Monomial, float] | None = None):
        self.terms: Dict[Monomial, float] = {}
        if terms:
            for m, c in terms.items():
                if c != 0:
                    self.terms[m] = self.terms.get(m, 0.0) + c

    # -- algebra -------------------------------------------------------------
    @staticmethod
    def scalar(c: float) -> "OperatorExpr":
        return OperatorExpr({(): float(c)})

    def __add__(self, other):
        if not isinstance(other, OperatorExpr):
            other = OperatorExpr.scalar(other)
        out = dict(self.terms)
        for m, c in other.terms.items():
            out[m] = out.get(m, 0.0) + c
        return OperatorExpr({m: c for m, c in out.items() if c != 0})

    __radd__ = __add__

    def __neg__(self):
        return OperatorExpr({m: -c for m, c in self.terms.items()})

    def __sub__(self, other):
        return self + (-other if isinstance(other, OperatorExpr) else -other)

    def __rsub__(self, other):
        return (-self) + other

    def __mul__(self, other):
        if isinstance(other, OperatorExpr):
            out: Dict[Monomial, float] = {}
            for m1, c1 in self.terms.items():
                for m2, c2 in other.terms.items():
                    m = m1 + m2
                    out[m] = out.get(m, 0.0) + c1 * c2
            return OperatorExpr(out)
        return OperatorExpr({m: c * other for m, c in self.terms.items()})

    def __rmul__(self, other):
        return OperatorExpr({m: other * c for m, c in self.terms.items()})

    def monomials(self) -> List[Monomial]:
        return list(self.terms.keys())

    def is_single_monomial(self) -> bool:
        return len(self.terms) == 1

    def n_factors(self) -> int:
        """Length of the (single) monomial; odd length means a fermionic operator."""
        return len(next(iter(self.terms)))

    def __repr__(self):
        if not self.terms:
            return "0"
        parts = []
        for m, c in self.terms.items():
            s = "".join(("c†" if d else "c") + repr(l) for d, l in m)
            parts.append(f"{c}*{s}" if s else f"{c}")
        return " + ".join(parts)

    # -- Fock-space representation ------------------------------------------
    def fock_matrix(self, soi: "SetOfIndices") -> np.ndarray:
        """Dense matrix in the Fock basis |n_0 n_1 ...>, state index = sum_i n_i 2^i.

        Fermionic sign: a creation/annihilation operator on mode i picks up
        (-1)^(number of occupied modes with index < i).
        """
        n = len(soi)
        dim = 1 << n
        M = np.zeros((dim, dim))
        for mono, coef in self.terms.items():
            idx = [(dag, soi[label]) for dag, label in mono]
            for st in range(dim):
                s = st
                sign = 1.0
                ok = True
                for dag, i in reversed(idx):
                    bit = 1 << i
                    occ = bool(s & bit)
                    if dag == occ:
                        ok = False
                        break
                    if bin(s & (bit - 1)).count("1") & 1:
                        sign = -sign
                    s ^= bit
                if ok:
                    M[s, st] += coef * sign
        return M


class SetOfIndices:
    """Ordered set of operator labels (KeldyshED.Hilbert.SetOfIndices)."""

    def __init__(self, labels: Iterable[Sequence]):
        self.labels: List[Label] = [tuple(l) for l in labels]
        self._index = {l: i for i, l in enumerate(self.labels)}

    def __len__(self):
        return len(self.labels)

    def __getitem__(self, label) -> int:
        return self._index[tuple(label)]

    def __iter__(self):
        return iter(self.labels)


def c(*label) -> OperatorExpr:
    return OperatorExpr({((False, _as_label(label)),): 1.0})


def c_dag(*label) -> OperatorExpr:
    return OperatorExpr({((True, _as_label(label)),): 1.0})


def n(*label) -> OperatorExpr:
    return c_dag(*label) * c(*label)
