"""Batched independent solves (qiw_batch_*): several whole inchworm! loops with different
parameters, grids, orders and sample counts in one device-resident launch queue, checked
solve by solve against the host-driven loop (qiw.inchworm.inchworm, one qiw_integrate per
step) and against the oracle's inchworm! restatement."""
import numpy as np
import pytest

import oracle as orc
from qiw import _lib, models
from qiw.batch import Batch, inchworm_batch
from qiw.inchworm import inchworm

pytestmark = pytest.mark.gpu

# (eps, U, V, beta, n_tau, max order, N)
SOLVES = [(0.1, 1.0, 0.5, 10.0, 24, 3, 64), (-0.4, 2.5, 0.8, 4.0, 17, 2, 256),
          (0.6, 0.7, 0.3, 20.0, 33, 4, 32), (-1.0, 3.5, 1.0, 2.0, 12, 1, 128)]


def _model(p):
    eps, U, V, beta, n_tau, _, _ = p
    return models.anderson(eps=eps, U=U, V=V, beta=beta, n_tau=n_tau)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _build():
    exps = [_model(p) for p in SOLVES]
    b = Batch(0)
    for e, p in zip(exps, SOLVES):
        b.add(e, range(0, p[5] + 1), range(0, p[5] + 1), p[6])
    return b, exps


def test_batch_matches_host_loop_per_solve(device):
    b, exps = _build()
    res = b.run(_lib.QIW_PREC_FP64, graph=True, autotune=True)
    assert res.graph_nodes > 3 * 31 and res.tiles_per_step > 0
    for sid, p in enumerate(SOLVES):
        ref = _model(p)
        inchworm(ref, range(0, p[5] + 1), range(0, p[5] + 1), p[6], dev=device)
        b.store_P(sid)
        for s in range(len(ref.P)):
            assert _rel(exps[sid].P[s].data, ref.P[s].data) < 1e-12, (sid, s)


def test_batch_matches_oracle():
    p = SOLVES[0]
    exp = _model(p)
    inchworm_batch([exp], range(0, p[5] + 1), range(0, p[5] + 1), p[6])
    ob = orc.inchworm(_model(p), range(0, p[5] + 1), range(0, p[5] + 1), p[6])
    for s in range(len(exp.P)):
        assert _rel(exp.P[s].data, ob.P_data[s]) < 1e-11


def test_graph_direct_and_tile_sizes_agree():
    b, _ = _build()
    b.run(_lib.QIW_PREC_FP64, graph=True, autotune=False)
    ref = [b.P_table(s) for s in range(len(SOLVES))]
    b.run(_lib.QIW_PREC_FP64, graph=False, autotune=False)   # direct launches, same tiles: bit-identical
    assert all(np.array_equal(b.P_table(s), ref[s]) for s in range(len(SOLVES)))
    res = b.run(_lib.QIW_PREC_FP64, graph=True, autotune=True)   # the tuned tile size sums in another grouping
    assert min(t for t in res.tune_ms if t > 0) > 0
    assert all(_rel(b.P_table(s), ref[s]) < 1e-13 for s in range(len(SOLVES)))


def test_batch_fp32_error_is_small():
    b, _ = _build()
    b.run(_lib.QIW_PREC_FP64)
    ref = [b.P_table(s) for s in range(len(SOLVES))]
    b.run(_lib.QIW_PREC_FP32)
    err = max(_rel(b.P_table(s), ref[s]) for s in range(len(SOLVES)))
    print(f"batch FP32 vs FP64: max |dP| / max |P| = {err:.2e}")
    assert err < 1e-5
