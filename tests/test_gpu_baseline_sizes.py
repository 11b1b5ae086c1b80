"""GPU vs oracle parity at the benchmark sizes (one GB300, FP64 1e-12, FP32 1e-4 relative).

The oracle restates the reference evaluator (src/topology_eval.jl:350-556) sample by sample, so
the full sizes are checked on Sobol sample-range slices: the kernel integrates samples
[first, first + n) of an N-point sequence (the way a rank of the reference's
rank_sub_range does, src/inchworm.jl:168-191) and the oracle integrates the same slice with
the same weights.  Slices sit at large Sobol indices, where the Gray-code jump is exercised.

  * eg Kanamori (U = 2, J = 0.2, beta = 8, n_tau = 256, orders 0:4, N = 1024): every group of
    the inch step at tau_w index 128, P taken from a GPU inchworm loop up to that step;
  * t2g Kanamori (U = 2.3, J = 0.4, beta = 20, n_tau = 512, orders 0:3, N = 2^14): every
    order-3 group at tau_w index 256, a 16-sample slice at first_index 2^14 - 40;
  * the reference README's Anderson run (n_tau = 200, orders 0:4, bare 0:4, N = 1024): the
    whole inchworm! loop, GPU against the oracle's loop, first 20 steps, 1e-11.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle as orc
from qiw import _lib, models
from qiw.device import Work
from qiw.diagrammatics import get_topologies_at_order

pytestmark = pytest.mark.gpu

REL64 = 1e-12
REL32 = 1e-4


def _rel(got, want):
    scale = max(np.abs(w).max() for w in want)
    err = max(np.abs(a - b).max() for a, b in zip(got, want))
    return err / scale if scale > 0 else err


def _bold_groups(orders):
    out = []
    for o in orders:
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = get_topologies_at_order(o, npa)
            if tops:
                out.append((o, npa, tops))
    return out


def _slice_parity(device, exp, groups, t, N, slices):
    """Per (group, slice): relative error of the kernel (FP64, FP32) against the oracle."""
    ob = orc.OracleProblem(exp)
    device.set_ppgf(exp.P)
    works, jobs = [], []
    for (o, npa, tops) in groups:
        gid = device.create_group(_lib.QIW_GROUP_BOLD, o, npa, tops)
        tl = [(x.pairs, x.parity) for x in tops]
        for (k, n) in ([(0, 1)] if o == 0 else slices):
            works.append(Work(gid, *t, k, n, 1 if o == 0 else N))
            jobs.append((o, npa, tl, (k, n), 1 if o == 0 else N))
    got64 = device.integrate(works, _lib.QIW_PREC_FP64)
    got32 = device.integrate(works, _lib.QIW_PREC_FP32)

    def ref(j):   # ctypes releases the GIL: the oracle runs on every host core
        o, npa, tl, sr, n_tot = j
        return ob.integrate("bold", o, npa, tl, *t, n_tot, sample_range=sr)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        want = list(ex.map(ref, jobs))
    return [(j[0], j[1], j[3], _rel(a, w), _rel(b, w)) for j, a, b, w in zip(jobs, got64, got32, want)]


def test_eg_inch_step_every_group_at_benchmark_size(device):
    from qiw.inchworm import inchworm
    exp = models.eg_discrete_bath(n_tau=256)
    n = 128
    inchworm(exp, range(0, 5), range(0, 5), 64, dev=device, n_steps=n - 1)   # P up to tau_n
    g = exp.grid
    rows = _slice_parity(device, exp, _bold_groups(range(0, 5)), (g.tau(0), g.tau(n), g.tau(n + 1)), 1024,
                         [(0, 16), (333, 16), (1008, 16)])
    worst64 = max(r[3] for r in rows)
    worst32 = max(r[4] for r in rows)
    print(f"eg n_tau=256 step {n}: {len(rows)} slices, max rel err FP64 {worst64:.2e}, FP32 {worst32:.2e}")
    assert worst64 < REL64, [r for r in rows if r[3] >= REL64]
    assert worst32 < REL32


def test_t2g_order3_groups_at_benchmark_size(device):
    from qiw.inchworm import inchworm
    exp = models.t2g_bethe(n_tau=512)
    n = 256
    inchworm(exp, range(0, 4), range(0, 4), 16, dev=device, n_steps=n - 1)
    g = exp.grid
    N = 1 << 14
    rows = _slice_parity(device, exp, _bold_groups([3]), (g.tau(0), g.tau(n), g.tau(n + 1)), N,
                         [(N - 40, 16)])
    worst64 = max(r[3] for r in rows)
    worst32 = max(r[4] for r in rows)
    print(f"t2g n_tau=512 step {n}: {len(rows)} order-3 slices, max rel err FP64 {worst64:.2e}, FP32 {worst32:.2e}")
    assert worst64 < REL64, rows
    assert worst32 < REL32


def test_readme_anderson_loop_first_steps_match_oracle(device):
    from qiw.inchworm import inchworm
    exp = models.anderson()          # README model: n_tau = 200
    exp_o = models.anderson()
    steps = 20
    inchworm(exp, range(0, 5), range(0, 5), 1024, dev=device, n_steps=steps)
    pb = orc.inchworm(exp_o, range(0, 5), range(0, 5), 1024, n_ranks=os.cpu_count() or 4, n_steps=steps)
    for s in range(len(exp.P)):
        a, b = exp.P[s].data[:steps + 2], pb.P_data[s][:steps + 2]
        assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()
