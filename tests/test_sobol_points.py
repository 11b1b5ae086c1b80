"""The kernels' Sobol integers, bit for bit (src/scrambled_sobol.jl:66-208).

The evaluation kernels form point k of a group's sequence by the Gray-code jump
x(k) = x0 ^ XOR_{b in bits(k ^ k>>1)} m[:, b]; qiw_sobol_points returns those UInt32 values
from the same device function.  They are compared with

  * the oracle's sequential generator, a restatement of the reference's next!/skip!
    (the state after k + 1 calls of next!), where the index is small enough to step to;
  * the oracle's closed form of that recurrence (pinned here against the sequential generator
    and SciPy's Sobol), at indices near 2^31 and 2^32 that multi-rank sample offsets reach;
  * next!'s recurrence itself, x(k) = x(k-1) ^ m[:, ctz(k)], over every consecutive pair of
    the kernel's output;
  * for scrambled sequences, the linear matrix scramble applied to SciPy's unscrambled point:
    x_scr(k) = shift ^ L_d(x(k)) per dimension, with L_d recovered from the scrambled direction
    numbers (the 32 unscrambled ones form a triangular basis of GF(2)^32);
  * the reference's own vectors (test/scrambled_sobol.jl), unscrambled and MockRNG-scrambled.
"""
import json
import os

import numpy as np
import pytest

import oracle as orc
from qiw import sobol

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIRSTS = [0, 1, 1000, (1 << 31) - 3, (1 << 32) - 64]
N_PTS = 64


def _scrambles(D):
    """(name, m, x0): unscrambled, MockRNG- and PCG64-scrambled tables of dimension D."""
    m = sobol.direction_numbers(D)
    out = [("plain", m, np.zeros(D, np.uint32))]
    ms, xs = sobol.scramble(m, sobol.MockRNG())
    out.append(("mock", ms, xs))
    ms, xs = sobol.scramble(m, sobol.NumpyBitRNG(100 + D))
    out.append(("pcg", ms, xs))
    return out


def _scipy_u32(D, first, n):
    import warnings
    from scipy.stats import qmc
    s = qmc.Sobol(d=D, scramble=False, bits=32)
    if first:
        s.fast_forward(first)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")   # balance properties want power-of-2 n; only the values matter
        x = s.random(n)
    return np.ldexp(x, 32).astype(np.uint64).astype(np.uint32)


def _lms_apply(m_plain_d, m_scr_d, v):
    """L(v) for the GF(2)-linear L with L(m_plain_d[j]) = m_scr_d[j] (j = 0..31).  m_plain_d[j]
    has lowest set bit 31 - j, so v is reduced from the lowest bit upwards."""
    out, v = 0, int(v)
    for j in range(31, -1, -1):
        bit = 31 - j
        if (v >> bit) & 1:
            v ^= int(m_plain_d[j])
            out ^= int(m_scr_d[j])
    assert v == 0
    return out


def _recurrence_ok(m, first, pts):
    for i in range(1, len(pts)):
        k = first + i
        c = (k & -k).bit_length() - 1
        if not np.array_equal(pts[i], pts[i - 1] ^ m[:, c]):
            return False
    return True


# ----------------------------------------------------------------------- CPU: the checker

@pytest.mark.parametrize("D", [1, 3, 8, 24])
def test_oracle_closed_form_equals_sequential_next(D):
    for name, m, x0 in _scrambles(D):
        seq = np.ldexp(orc.sobol_points(m, x0, 0, 600), 32).astype(np.uint64).astype(np.uint32)
        for k in (0, 1, 2, 3, 5, 64, 255, 256, 511, 599):
            assert np.array_equal(orc.sobol_point_u32(m, x0, k), seq[k]), (name, k)


@pytest.mark.parametrize("D", [2, 12])
def test_oracle_closed_form_equals_scipy_at_an_offset(D):
    m = sobol.direction_numbers(D)
    first = (1 << 20) + 3
    ref = _scipy_u32(D, first, 8)
    for i in range(8):
        assert np.array_equal(orc.sobol_point_u32(m, None, first + i), ref[i])


def test_scrambled_points_are_the_scrambled_plain_points():
    D = 5
    m = sobol.direction_numbers(D)
    ms, xs = sobol.scramble(m, sobol.NumpyBitRNG(3))
    plain = _scipy_u32(D, 0, 40)
    seq = np.ldexp(orc.sobol_points(ms, xs, 0, 40), 32).astype(np.uint64).astype(np.uint32)
    for k in range(40):
        for d in range(D):
            assert seq[k, d] == xs[d] ^ _lms_apply(m[d], ms[d], plain[k, d])


# ----------------------------------------------------------------------- GPU: the kernels

@pytest.mark.gpu
@pytest.mark.parametrize("D", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 16, 24, 32])
def test_kernel_sobol_integers_bit_exact(device, D):
    for name, m, x0 in _scrambles(D):
        for first in FIRSTS:
            got = device.sobol_points(m, x0, first, N_PTS)
            assert got.dtype == np.uint32 and got.shape == (N_PTS, D)
            for i in (0, 1, N_PTS // 2, N_PTS - 1):
                assert np.array_equal(got[i], orc.sobol_point_u32(m, x0, first + i)), (name, first, i)
            assert _recurrence_ok(m, first, got), (name, first)
            if first <= 1000 and D <= 24:
                seq = np.ldexp(orc.sobol_points(m, x0, first, N_PTS), 32).astype(np.uint64).astype(np.uint32)
                assert np.array_equal(got, seq), (name, first)


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 6, 12])
def test_kernel_scrambled_points_against_scipy(device, D):
    m = sobol.direction_numbers(D)
    first = (1 << 18) + 7
    plain = _scipy_u32(D, first, 16)
    assert np.array_equal(device.sobol_points(m, None, first, 16), plain)
    for name, ms, xs in _scrambles(D)[1:]:
        got = device.sobol_points(ms, xs, first, 16)
        for k in range(16):
            want = [xs[d] ^ _lms_apply(m[d], ms[d], plain[k, d]) for d in range(D)]
            assert [int(v) for v in got[k]] == want, (name, k)


@pytest.mark.gpu
def test_kernel_sobol_reference_vectors(device):
    with open(os.path.join(GOLD, "sobol_vectors.json")) as f:
        g = json.load(f)
    for D, key in ((1, "D1"), (5, "D5")):
        m = sobol.direction_numbers(D)
        ref = np.array(g["unscrambled"][key])
        assert np.array_equal(np.ldexp(device.sobol_points(m, None, 0, len(ref)).astype(np.float64), -32), ref)
        ms, xs = sobol.scramble(m, sobol.MockRNG())
        ref = np.array(g["scrambled_mockrng"][key])
        got = np.ldexp(device.sobol_points(ms, xs, 0, len(ref)).astype(np.float64), -32)
        assert np.allclose(got, ref, atol=g["tolerance_scrambled"], rtol=0)


@pytest.mark.gpu
def test_kernel_sobol_rejects_out_of_range(device):
    from qiw._lib import QiwError
    m = sobol.direction_numbers(2)
    with pytest.raises(QiwError):
        device.sobol_points(m, None, (1 << 32) - 8, 16)
