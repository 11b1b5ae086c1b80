"""The CPU oracle pinned against the reference's own golden vectors and known answers."""
import json
import math
import os

import numpy as np
import pytest

import oracle as orc
from qiw import models, sobol
from qiw.diagrammatics import (generate_topologies, get_topologies_at_order, isvalid,
                               count_doubly_k_connected, is_k_connected, Topology)

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("D", [1, 5, 12])
def test_sobol_unscrambled_matches_scipy(D):
    from scipy.stats import qmc
    ref = qmc.Sobol(d=D, scramble=False, bits=32).random_base2(m=9)
    m = orc.sobol_directions(D)
    assert np.array_equal(m, sobol.direction_numbers(D))
    assert np.array_equal(orc.sobol_points(m, None, 0, 512), ref)


def test_sobol_golden_and_skip():
    g = _load("sobol_vectors.json")
    for D, key in ((1, "D1"), (5, "D5")):
        ref = np.array(g["unscrambled"][key])
        m = orc.sobol_directions(D)
        assert np.array_equal(orc.sobol_points(m, None, 0, 8), ref)
        # skip!(s, 3, exact=true) then 5 points
        assert np.array_equal(orc.sobol_points(m, None, 3, 5), ref[3:])
        s = sobol.ScrambledSobolSeq(D)
        s.skip(3)  # skips 4 points (2^m < n <= 2^(m+1))
        assert np.array_equal(np.array([s.next() for _ in range(4)]), ref[4:])


def test_sobol_scrambled_mockrng_golden():
    g = _load("sobol_vectors.json")
    for D, key in ((1, "D1"), (5, "D5")):
        ref = np.array(g["scrambled_mockrng"][key])
        m, x0 = sobol.scramble(sobol.direction_numbers(D), sobol.MockRNG())
        pts = orc.sobol_points(m, x0, 0, 8)
        assert np.allclose(pts, ref, atol=1e-10, rtol=0)
        pts = orc.sobol_points(m, x0, 3, 5)
        assert np.allclose(pts, ref[3:], atol=1e-10, rtol=0)


def test_gray_code_jump_equals_sequential():
    m = sobol.direction_numbers(8)
    x0 = np.arange(8, dtype=np.uint32) * 12345
    seq = orc.sobol_points(m, x0, 0, 300)
    for n in (0, 1, 2, 3, 77, 128, 255, 299):
        x = sobol.ScrambledSobolSeq.point_uint(m, x0, n)
        assert np.array_equal(np.ldexp(x.astype(np.float64), -32), seq[n])


def test_topology_counts():
    for n in range(1, 7):
        tops = generate_topologies(n)
        assert len(tops) == math.prod(range(2 * n - 1, 0, -2))
        assert all(isvalid(t) for t in tops)
        for t in tops:
            for k in range(1, n + 1):
                assert (-1) ** k == (-1) ** count_doubly_k_connected(t.pairs, k)
        # irreducible chord diagrams, OEIS A000699 (test/diagrammatics.jl:59)
        assert len(get_topologies_at_order(n, 1)) == [1, 1, 4, 27, 248, 2830][n - 1]
    ra = _load("readme_anderson.json")
    assert [len(get_topologies_at_order(k)) for k in range(5)] == ra["topology_counts_bare"]
    for k, counts in enumerate(ra["topology_counts_bold"]):
        rng = [0] if k == 0 else range(1, 2 * k)
        got = [len(get_topologies_at_order(k, npa)) for npa in rng] if k else [1]
        assert got == counts
    # oracle's own restatement agrees with the product's generator, parities included
    for n in range(0, 5):
        for k in ([None] + list(range(1, 2 * n))):
            a = [(t.pairs, t.parity) for t in get_topologies_at_order(n, k)]
            assert a == orc.topologies(n, k)


def test_k_connectivity_cases():
    # test/diagrammatics.jl:62-85
    t = Topology(2, ((1, 2), (3, 4)), 1)
    assert [is_k_connected(t, k) for k in range(5)] == [False, False, False, True, True]
    t = Topology(2, ((1, 4), (2, 3)), 1)
    assert [is_k_connected(t, k) for k in range(5)] == [False, False, True, True, True]
    t = Topology(2, ((1, 3), (2, 4)), -1)
    assert [is_k_connected(t, k) for k in range(5)] == [False, True, True, True, True]


def test_simplex_volume_known_answer():
    """Constant integrand: the qMC estimate equals the (double-)simplex volume exactly."""
    exp = models.single_level(n_tau=8, spline=False)
    pb = orc.OracleProblem(exp)
    # order-0 of a bold group is exact: P(t_f - t_w) P(t_w - t_i) with the grid values
    g = exp.grid
    blk = pb.integrate("bold", 0, 0, orc.topologies(0), g.tau(0), g.tau(3), g.tau(5), 1)
    for s in range(pb.S):
        d = exp.P[s].data
        want = -1j * (1j * d[2]) @ (1j * d[3])
        assert np.allclose(blk[s], want, rtol=1e-14, atol=0)


def test_oracle_reproduces_reference_golden_inchworm():
    """test/inchworm.jl:180-212 via the reference's own fixture test/inchworm.h5."""
    gold = _load("inchworm_h5.json")
    exp = models.single_level()
    pb = orc.inchworm(exp, range(0, 4), range(0, 3), 2 ** 8)
    for s in range(2):
        want = np.array(gold["P"][s]["re"]) + 1j * np.array(gold["P"][s]["im"])
        got = pb.P_data[s][:, 0, 0]
        # pinned at 3e-8 (norm): bare step bit-exact, residual from the bold P lookups
        assert np.linalg.norm(got - want) <= 5e-8 * np.linalg.norm(want)
    from qiw import operators as op
    exp.add_corr_operators((op.c("0"), op.c_dag("0")))
    pb2 = orc.OracleProblem(exp)
    pb2.P_data, pb2.P_der, pb2.n_valid = pb.P_data, pb.P_der, pb.n_valid
    g = -orc.correlator_2p(pb2, range(0, 4), 2 ** 8)[0]
    want = np.array(gold["g"]["re"]) + 1j * np.array(gold["g"]["im"])
    assert np.linalg.norm(g - want) <= 1e-6 * np.linalg.norm(want)


def test_golden_inchworm_residual_is_bounded_per_step():
    """Where the oracle departs from test/inchworm.h5, and by how much per step.

    The final P of inchworm! carries every later normalize!(P, tau) factor exp(-tau_j lambda_n)
    (src/inchworm.jl:488).  Taking out one common factor exp(-tau_j dL), dL fitted on the bare
    point tau_1 (whose raw value is bit-exact), leaves the shape of P: it matches the fixture to
    rounding through the first bold step (tau_2) and departs by ~2e-10 at the second (tau_3),
    growing about quadratically with the step index after that -- a deviation of the order of
    1e-10 in each step's integral (source not identified: the incremental-spline P lookups are
    ruled out, they depart by 1e-5 already at the first bold step).  The reference checks its
    own run against this fixture only to Julia's default isapprox tolerance, sqrt(eps) = 1.5e-8
    in norm (test/inchworm.jl:45-51)."""
    gold = _load("inchworm_h5.json")
    exp = models.single_level()
    pb = orc.inchworm(exp, range(0, 4), range(0, 3), 2 ** 8)
    taus = np.array([exp.grid.tau(j) for j in range(exp.grid.n_tau)])
    r = [pb.P_data[s][:, 0, 0] / (np.array(gold["P"][s]["re"]) + 1j * np.array(gold["P"][s]["im"])) for s in range(2)]
    dL = -np.log(r[0][1].real) / taus[1]
    assert abs(dL) < 2e-8                                   # the accumulated normalisation drift
    for s in range(2):
        shape = np.abs(r[s] * np.exp(taus * dL) - 1)
        assert shape[:3].max() < 1e-14                      # bare step and first bold step
        assert shape[3] < 5e-10                             # second bold step
        assert shape.max() < 2e-7


def test_oracle_reproduces_reference_golden_diff_inchworm():
    """test/inchworm.jl:214-239 (diff_inchworm!, orders 0:3, N = 2^8) via test/inchworm.h5."""
    gold = _load("inchworm_h5.json")
    pb, _ = orc.diff_inchworm(models.single_level(), range(0, 4), 2 ** 8)
    for s in range(2):
        want = np.array(gold["diff_P"][s]["re"]) + 1j * np.array(gold["diff_P"][s]["im"])
        got = pb.P_data[s][:, 0, 0]
        assert np.array_equal(got[:2], want[:2])            # the first Euler step is exact
        # 1.5e-8 (norm), the residual of the bold P lookups seen in the inchworm! fixture too
        assert np.linalg.norm(got - want) <= 5e-8 * np.linalg.norm(want)


def test_oracle_rank_split_matches_single_rank():
    exp = models.anderson(n_tau=16)
    pb = orc.OracleProblem(exp)
    g = exp.grid
    tops = orc.topologies(3, 2)
    a = pb.integrate("bold", 3, 2, tops, g.tau(0), g.tau(4), g.tau(5), 128, n_ranks=1)
    b = pb.integrate("bold", 3, 2, tops, g.tau(0), g.tau(4), g.tau(5), 128, n_ranks=3)
    for x, y in zip(a, b):
        assert np.allclose(x, y, rtol=1e-13, atol=1e-18)


def test_bare_domain_maps_estimate_the_same_integral():
    """RootTransform, SortTransform and ExpModelFunctionTransform (src/qmc_integrate.jl:99-334)
    are unbiased maps of the same simplex integral: their qMC estimates of a bare group agree
    within the qMC error, which falls with N (test/qmc_integrate.jl checks the maps the same way,
    against analytic integrals)."""
    from qiw import models
    from qiw.diagrammatics import get_topologies_at_order
    exp = models.anderson(n_tau=40)
    ob = orc.OracleProblem(exp)
    t_f = exp.grid.tau(6)
    for k, tol_sort, tol_exp in [(1, 1e-4, 2e-3), (2, 5e-4, 5e-3)]:
        tops = [(t.pairs, t.parity) for t in get_topologies_at_order(k)]
        errs = []
        for N in (2 ** 12, 2 ** 16):
            r = ob.integrate("bare", k, 0, tops, 0.0, 0.0, t_f, N)
            s = ob.integrate("bare", k, 0, tops, 0.0, 0.0, t_f, N, transform="sort")
            e = ob.integrate("bare", k, 0, tops, 0.0, 0.0, t_f, N, transform="expmodel", decay=t_f / (2 * k))
            sc = max(np.abs(b).max() for b in r)
            errs.append((max(np.abs(x - y).max() for x, y in zip(s, r)) / sc,
                         max(np.abs(x - y).max() for x, y in zip(e, r)) / sc))
        assert errs[1][0] < tol_sort and errs[1][1] < tol_exp, (k, errs)
        assert errs[1][1] < errs[0][1]
