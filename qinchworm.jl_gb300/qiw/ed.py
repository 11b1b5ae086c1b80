"""Exact diagonalization of the local (atomic) problem.

Plays the role KeldyshED.EDCore plays for the reference (`src/expansion.jl:222-291`,
`src/sector_block_matrix.jl:52-66`, `src/ppgf.jl:157-173`): it splits the Fock space
into invariant subspaces (sectors), diagonalises the Hamiltonian in each of them and
represents operators as sector block matrices in the eigenbasis.

Sector discovery follows the usual two-phase automatic partition: (1) connected
components of the Fock-state graph induced by the Hamiltonian (and any symmetry
breakers); (2) sectors are merged until every creation and annihilation operator maps
each sector into at most one sector.  Sectors are ordered by lowest eigenvalue (ties by
smallest Fock state), states inside a sector by Fock index.  Eigenbasis phases are whatever LAPACK returns, so
raw block entries are basis dependent while Z, rho's spectrum and G(tau) are not.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

from .operators import OperatorExpr, SetOfIndices, c, c_dag


class SectorBlockMatrix(dict):
    """s_i -> (s_f, block) with at most one block per column (0-based sectors).

    Mirrors `SectorBlockMatrix = Dict{Int64, Tuple{Int64, Matrix{ComplexF64}}}`
    (`src/sector_block_matrix.jl:44`).
    """

    def copy(self):
        return SectorBlockMatrix({k: (sf, m.copy()) for k, (sf, m) in self.items()})

    def __add__(self, other):
        out = self.copy()
        for k, (sf, m) in other.items():
            if k in out:
                assert out[k][0] == sf
                out[k] = (sf, out[k][1] + m)
            else:
                out[k] = (sf, m.copy())
        return out

    def __mul__(self, x):
        return SectorBlockMatrix({k: (sf, m * x) for k, (sf, m) in self.items()})

    __rmul__ = __mul__

    def trace(self) -> complex:
        return complex(sum(np.trace(m) for k, (sf, m) in self.items() if k == sf))

    def norm_inf(self) -> float:
        return max((float(np.max(np.abs(m))) if m.size else 0.0) for _, (_, m) in self.items())


class EDCore:
    def __init__(self, hamiltonian: OperatorExpr, soi: SetOfIndices,
                 symmetry_breakers: Sequence[OperatorExpr] = ()):
        self.soi = soi
        self.hamiltonian = hamiltonian
        n = len(soi)
        self.fock_dim = 1 << n
        H = hamiltonian.fock_matrix(soi)
        if not np.allclose(H, H.T, atol=1e-14):
            raise ValueError("Hamiltonian is not real symmetric")
        self._H = H

        parent = list(range(self.fock_dim))

        def find(a):
            while parent[a] != a:
                parent[a] = parent[parent[a]]
                a = parent[a]
            return a

        def union(a, b):
            ra, rb = find(a), find(b)
            if ra != rb:
                parent[max(ra, rb)] = min(ra, rb)

        conn = np.abs(H) > 0
        for sb in symmetry_breakers:
            conn |= np.abs(sb.fock_matrix(soi)) > 0
        for i, j in zip(*np.nonzero(conn)):
            union(int(i), int(j))

        # Phase 2: every c / c^dag must map a sector into at most one sector.
        ops = []
        for label in soi:
            ops.append(c_dag(label).fock_matrix(soi))
            ops.append(c(label).fock_matrix(soi))
        changed = True
        while changed:
            changed = False
            for M in ops:
                targets: Dict[int, int] = {}
                for f, i in zip(*np.nonzero(M)):
                    ri = find(int(i))
                    rf = find(int(f))
                    if ri in targets and find(targets[ri]) != rf:
                        union(targets[ri], rf)
                        changed = True
                    targets.setdefault(ri, rf)

        roots: Dict[int, List[int]] = {}
        for st in range(self.fock_dim):
            roots.setdefault(find(st), []).append(st)
        blocks = []
        for states in roots.values():
            Hs = H[np.ix_(states, states)]
            E, U = np.linalg.eigh(Hs)
            blocks.append((float(E[0]), states[0], states, E, U))
        # Sectors ordered by their lowest eigenvalue, ties by smallest Fock state (the
        # order KeldyshED produces for the reference's fixtures).
        blocks.sort(key=lambda b: (round(b[0], 12), b[1]))
        self.subspaces: List[List[int]] = [b[2] for b in blocks]
        self.eigenvalues: List[np.ndarray] = [b[3] for b in blocks]
        self.unitaries: List[np.ndarray] = [b[4] for b in blocks]
        self.state_sector = np.empty(self.fock_dim, dtype=np.int64)
        for s, states in enumerate(self.subspaces):
            for st in states:
                self.state_sector[st] = s
        self.gs_energy = min(float(E.min()) for E in self.eigenvalues)
        self.energies = [E - self.gs_energy for E in self.eigenvalues]

    @property
    def n_sectors(self) -> int:
        return len(self.subspaces)

    @property
    def dims(self) -> List[int]:
        return [len(s) for s in self.subspaces]

    def operator_blocks(self, op: OperatorExpr) -> SectorBlockMatrix:
        """Blocks of `op` in the eigenbasis (KeldyshED.operator_blocks semantics)."""
        M = op.fock_matrix(self.soi)
        sbm = SectorBlockMatrix()
        for si, states_i in enumerate(self.subspaces):
            cols = M[:, states_i]
            rows = np.nonzero(np.any(cols != 0, axis=1))[0]
            if rows.size == 0:
                continue
            targets = sorted({int(self.state_sector[r]) for r in rows})
            if len(targets) > 1:
                raise ValueError(
                    f"Operator {op} is not representable by a SectorBlockMatrix "
                    "(more than one non-zero blocks per column)")
            sf = targets[0]
            states_f = self.subspaces[sf]
            blk = self.unitaries[sf].T @ M[np.ix_(states_f, states_i)] @ self.unitaries[si]
            sbm[si] = (sf, blk.astype(np.complex128))
        return sbm

    def partition_function(self, beta: float) -> float:
        return float(sum(np.exp(-beta * E).sum() for E in self.energies))

    def density_matrix(self, beta: float) -> List[np.ndarray]:
        Z = self.partition_function(beta)
        return [np.diag(np.exp(-beta * E)) / Z for E in self.energies]

    def sector_particle_numbers(self) -> List[int]:
        return [bin(s[0]).count("1") for s in self.subspaces]
