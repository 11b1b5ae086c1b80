"""Exact-diagonalisation references for the dimer tests (test infrastructure).

Restates the three KeldyshED helpers that the reference's test/dimers.jl uses:
``reduced_density_matrix`` (thermal state of the whole dimer, bath modes traced out),
``full_hs_matrix`` (sector blocks of the impurity density matrix placed in the impurity's
Fock basis) and the rho = i P(beta) / Tr[i P(beta)] step of ``normalize!(P, beta)`` followed by
``density_matrix`` (src/ppgf.jl:611-636).

Fock states follow qiw.operators: mode k of the set of indices is bit k, and the fermionic
sign counts the occupied modes below k.  The impurity modes are listed first, so impurity
operators carry no sign strings over the bath modes and the plain partial trace over the
higher bits is the fermionic reduced density matrix.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np
from scipy.linalg import expm

from qiw import operators as op


def reduced_density_matrix(H: op.OperatorExpr, imp_labels: Sequence, bath_labels: Sequence,
                           beta: float) -> np.ndarray:
    soi = op.SetOfIndices([list(l) for l in imp_labels] + [list(l) for l in bath_labels])
    Hm = H.fock_matrix(soi)
    rho = expm(-beta * (Hm - np.linalg.eigvalsh(Hm).min() * np.eye(Hm.shape[0])))
    rho /= np.trace(rho)
    ni, nb = 1 << len(imp_labels), 1 << len(bath_labels)
    return np.einsum("bibj->ij", rho.reshape(nb, ni, nb, ni))


def full_hs_matrix(rho_sectors: List[np.ndarray], ed) -> np.ndarray:
    out = np.zeros((ed.fock_dim, ed.fock_dim), dtype=np.complex128)
    for states, U, r in zip(ed.subspaces, ed.unitaries, rho_sectors):
        out[np.ix_(states, states)] = U @ r @ U.T
    return out


def rho_from_P(P_beta: List[np.ndarray]) -> List[np.ndarray]:
    """Sector density matrices from the un-normalised P_s(beta) blocks."""
    Z = sum(np.trace(1j * p) for p in P_beta)
    return [1j * p / Z for p in P_beta]
