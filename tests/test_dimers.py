"""The reference's exact-diagonalisation checks (test/dimers.jl) on the oracle and on the GPU.

The reference solves an impurity coupled to one bath level with inchworm! and asserts that
the impurity density matrix matches the exact one of the whole dimer, max |rho_ref - rho| <
1e-4 (test/dimers.jl:97-116 and :177-196).  The oracle must pass that bar on CPU; the CUDA
path must pass it too and agree with the oracle to 1e-11 over the whole loop.
"""
import numpy as np
import pytest

import oracle as orc
from qiw import models
from qiw import operators as op

from edref import full_hs_matrix, reduced_density_matrix, rho_from_P

ED_TOL = 1e-4

# (model, spline, orders, N_samples) of test/dimers.jl:97-116 and :177-196
CASES = [
    ("dimer", False, range(0, 2), 8 * 2 ** 4),
    ("dimer", True, range(0, 2), 8 * 2 ** 4),
    ("dimer", False, range(0, 4), 8 * 2 ** 4),
    ("dimer", True, range(0, 4), 8 * 2 ** 4),
    ("hubbard", False, range(0, 2), 8 * 2 ** 5),
    ("hubbard", False, range(0, 3), 8 * 2 ** 5),
]


def _case(name, spline):
    """(expansion, exact impurity rho in the impurity Fock basis)."""
    if name == "dimer":
        exp = models.dimer(spline=spline)
        H = 0.5 * op.n(1) + 2.0 * op.n(2) + 0.5 * (op.c_dag(1) * op.c(2) + op.c_dag(2) * op.c(1))
        return exp, reduced_density_matrix(H, [(1,)], [(2,)], 1.0)
    U, V = 4.0, 0.5
    exp = models.hubbard_dimer(U=U, V=V)
    H = U * op.n(1) * op.n(2) - 0.5 * U * (op.n(1) + op.n(2))
    H = H + V * (op.c_dag(1) * op.c(3) + op.c_dag(3) * op.c(1))
    H = H + V * (op.c_dag(2) * op.c(4) + op.c_dag(4) * op.c(2))
    return exp, reduced_density_matrix(H, [(1,), (2,)], [(3,), (4,)], 1.0)


def _rho(exp, P_beta):
    return full_hs_matrix(rho_from_P(P_beta), exp.ed)


@pytest.mark.parametrize("name,spline,orders,N", CASES)
def test_oracle_matches_exact_dimer(name, spline, orders, N):
    exp, rho_ref = _case(name, spline)
    pb = orc.inchworm(exp, orders, orders, N)
    rho = _rho(exp, [P[-1] for P in pb.P_data])
    assert np.abs(rho_ref - rho).max() < ED_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name,spline,orders,N", CASES)
def test_gpu_matches_exact_dimer_and_oracle(device, name, spline, orders, N):
    from qiw.inchworm import inchworm
    exp, rho_ref = _case(name, spline)
    exp_o, _ = _case(name, spline)
    inchworm(exp, orders, orders, N, dev=device)
    pb = orc.inchworm(exp_o, orders, orders, N)
    for s in range(len(exp.P)):
        a, b = exp.P[s].data, pb.P_data[s]
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()
    rho = _rho(exp, [P.data[-1] for P in exp.P])
    assert np.abs(rho_ref - rho).max() < ED_TOL
