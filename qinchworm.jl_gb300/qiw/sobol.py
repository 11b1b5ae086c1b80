"""Host side of the scrambled Sobol sequence (`src/scrambled_sobol.jl:50-208`).

The device only needs the direction matrix m[D][32] (uint32) and the initial point x0[D]
(the digital shift, zero when unscrambled); it then forms point n with the Gray-code
identity x(n) = x0 ^ XOR_{b in bits(n ^ (n >> 1))} m[:, b], which equals the reference's
sequential `next!` recurrence x(n) = x(n-1) ^ m[:, ctz(n)] (`:158-173`).  Scrambling
(linear matrix scramble + digital shift, `:102-140`) stays on the host so a caller's own
RNG decides the parameters, exactly as in the reference.

Direction-number tables: the reference takes `sobol_a` / `sobol_minit` from Sobol.jl
(`:79,83`), which are the Joe-Kuo primitive polynomials and initial direction numbers.
SciPy ships the same published table (`scipy/stats/_sobol_direction_numbers.npz`, arrays
`poly` and `vinit`); it is read at run time, not copied into this repository.
"""
from __future__ import annotations

import math
import os
from functools import lru_cache
from typing import Optional

import numpy as np

MAX_DIM = 21201


@lru_cache(maxsize=1)
def _joe_kuo_table():
    import scipy  # the published direction-number table lives in SciPy's data files
    path = os.path.join(os.path.dirname(scipy.__file__), "stats", "_sobol_direction_numbers.npz")
    with np.load(path) as f:
        return f["poly"].astype(np.int64), f["vinit"].astype(np.int64)


def direction_numbers(D: int) -> np.ndarray:
    """m[D, 32] uint32, columns already multiplied by 2^(32-j)."""
    if D < 0 or D > MAX_DIM:
        raise ValueError(f"Invalid Sobol dimension {D}")
    poly, vinit = _joe_kuo_table()
    m = np.ones((D, 32), dtype=np.uint64)
    for d in range(2, D + 1):
        a = int(poly[d - 1])
        deg = int(math.floor(math.log2(a)))
        m[d - 1, :deg] = vinit[d - 1, :deg]
        for j in range(deg + 1, 33):
            ac = a
            v = int(m[d - 1, j - deg - 1])
            for k in range(deg):
                v ^= ((ac & 1) * int(m[d - 1, j - deg + k - 1])) << (deg - k)
                ac >>= 1
            m[d - 1, j - 1] = v & 0xFFFFFFFF
    for j in range(1, 33):
        m[:, j - 1] = (m[:, j - 1] << (32 - j)) & 0xFFFFFFFF
    return m.astype(np.uint32)


class MockRNG:
    """Deterministic stand-in RNG of the reference tests (`test/scrambled_sobol.jl:97-105`).

    rand(S, dims...) returns S[popcount(i) % len(S)] for the column-major linear index i.
    """

    def rand(self, S, *dims):
        size = int(np.prod(dims))
        vals = np.array([S[bin(i).count("1") % len(S)] for i in range(size)], dtype=np.uint64)
        return vals.reshape(dims, order="F")


class NumpyBitRNG:
    """Scrambling RNG backed by numpy's PCG64 (same call shapes as the reference)."""

    def __init__(self, seed):
        self.g = np.random.default_rng(seed)

    def rand(self, S, *dims):
        idx = self.g.integers(0, len(S), size=dims)
        return np.asarray(S, dtype=np.uint64)[idx]


def scramble(m: np.ndarray, rng) -> tuple[np.ndarray, np.ndarray]:
    """Linear matrix scramble + digital shift; returns (m_scrambled, x0)."""
    D = m.shape[0]
    shift_bits = rng.rand([0, 1], D, 32)
    x0 = np.zeros(D, dtype=np.uint64)
    for j in range(32):
        x0 += shift_bits[:, j].astype(np.uint64) << np.uint64(j)
    ltm = rng.rand([0, 1], D, 32, 32).astype(np.uint64)
    for d in range(D):
        ltm[d] = np.tril(ltm[d])
        np.fill_diagonal(ltm[d], 1)
    # bit p of the scrambled m[d, j] (from the top: 31 - p) is the GF(2) dot product of row p of
    # the lower-triangular matrix with the bits of m[d, j] (k-th bit from the top, 31 - k)
    shifts = (31 - np.arange(32)).astype(np.uint64)
    mbits = ((m.astype(np.uint64)[:, None, :] >> shifts[None, :, None]) & np.uint64(1)).astype(np.int64)  # [D][k][j]
    prod = np.einsum("dpk,dkj->dpj", ltm.astype(np.int64), mbits) & 1                                     # [D][p][j]
    out = (prod.astype(np.uint64) << shifts[None, :, None]).sum(axis=1, dtype=np.uint64)                   # [D][j]
    return out.astype(np.uint32), (x0 & 0xFFFFFFFF).astype(np.uint32)


class ScrambledSobolSeq:
    """Host-side sequence object with the reference's `next!` / `skip!` semantics."""

    def __init__(self, D: int, scramble_rng=None):
        self.D = D
        m = direction_numbers(D)
        if scramble_rng is None:
            self.m = m
            self.x0 = np.zeros(D, dtype=np.uint32)
        else:
            self.m, self.x0 = scramble(m, scramble_rng)
        self.x = self.x0.copy()
        self.n = 0

    def ndims(self) -> int:
        return self.D

    def next(self) -> np.ndarray:
        if self.n == 0:
            self.n = 1
            return np.ldexp(self.x.astype(np.float64), -32)
        self.n += 1
        c = ((self.n - 1) & -(self.n - 1)).bit_length() - 1
        self.x ^= self.m[:, c]
        return np.ldexp(self.x.astype(np.float64), -32)

    def skip(self, n: int, exact: bool = False):
        if n < 0:
            raise ValueError(f"{n} is not non-negative")
        if n == 0:
            return self
        nskip = n if exact else (1 << int(math.floor(math.log2(n + 1))))
        for _ in range(nskip):
            self.next()
        return self

    @staticmethod
    def point_uint(m: np.ndarray, x0: np.ndarray, n: int) -> np.ndarray:
        """Point number n (0-based) by the Gray-code jump."""
        g = n ^ (n >> 1)
        x = x0.astype(np.uint32).copy()
        b = 0
        while g:
            if g & 1:
                x ^= m[:, b]
            g >>= 1
            b += 1
        return x


def sobol_points(m: np.ndarray, first: int, n: int, x0: Optional[np.ndarray] = None) -> np.ndarray:
    """Points first .. first+n-1 in [0, 1)^D (rows), by the Gray-code jump of point_uint."""
    D = m.shape[0]
    idx = np.arange(first, first + n, dtype=np.uint64)
    g = idx ^ (idx >> np.uint64(1))
    x = np.broadcast_to(np.zeros(D, np.uint32) if x0 is None else np.asarray(x0, np.uint32), (n, D)).copy()
    for b in range(32):
        sel = ((g >> np.uint64(b)) & np.uint64(1)).astype(bool)
        x[sel] ^= m[:, b].astype(np.uint32)
    return np.ldexp(x.astype(np.float64), -32)
