"""seq_offset: every sampled group skips the first k points of its sequence, as
skip!(seq, k, exact=true) would before the reference's qMC sum (src/scrambled_sobol.jl:189-208,
src/qmc_integrate.jl:497-507).  Checked against the oracle integrating the sample range
[k, k + N) with weight 1/N, through the oracle stand-in (host logic) and on the GPU."""
import numpy as np
import pytest

import oracle as orc
from qiw import models
from qiw.diagrammatics import get_topologies_at_order
from qiw.inchworm import TopologiesInputData, inchworm_step
from test_multirank import OracleDevice

N = 64


def _want(exp, t, k):
    ob = orc.OracleProblem(exp)
    tot = None
    for o in range(0, 3):
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = [(x.pairs, x.parity) for x in (get_topologies_at_order(0) if o == 0 else get_topologies_at_order(o, npa))]
            rng = (0, 1) if o == 0 else (k, N)
            blk = ob.integrate("bold", o, npa, tops, *t, 1 if o == 0 else N, sample_range=rng)
            v = np.concatenate([b.ravel() for b in blk])
            tot = v if tot is None else tot + v
    return tot


@pytest.mark.parametrize("kind", ["oracle", pytest.param("gpu", marks=pytest.mark.gpu)])
@pytest.mark.parametrize("k", [0, 1, 5])
def test_seq_offset_skips_leading_points(kind, k, request):
    exp = models.anderson(n_tau=10)
    g = exp.grid
    t = (g.tau(0), g.tau(4), g.tau(5))
    tds = [TopologiesInputData(o, npa, get_topologies_at_order(0) if o == 0 else get_topologies_at_order(o, npa), N)
           for o in range(0, 3) for npa in ([0] if o == 0 else range(1, 2 * o))]
    dev = OracleDevice() if kind == "oracle" else request.getfixturevalue("device")
    value, _, _ = inchworm_step(exp, *t, tds, dev=dev, seq_offset=k)
    got = np.concatenate([value[s][1].ravel() for s in range(len(exp.dims))])
    want = _want(exp, t, k)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    if k:
        assert np.abs(got - _want(exp, t, 0)).max() > 1e-6 * np.abs(want).max()   # the offset changes the points


def test_seq_offset_must_be_non_negative():
    with pytest.raises(ValueError):
        inchworm_step(models.anderson(n_tau=6), 0.0, 1.0, 2.0, [], dev=OracleDevice(), seq_offset=-1)
