"""Randomized qMC (src/randomization.jl:86-100) in inchworm_step and correlator_2p.

The host driver runs all scrambled sequences of a step in one launch and then applies the
reference's stopping rule (stop after sequence s > 1 once the largest |std| is at most
target_std), setting the scrambling generator back to where the reference leaves it.  These
tests compare it with the oracle's sequential restatement -- one sequence at a time, each
scramble drawn only when it is used -- on the same seeded generator: means, standard
deviations and the generator state afterwards must agree.  Each test runs twice: through a
stand-in for the device backed by the CPU oracle (host logic only), and through the CUDA
library on the GPU (scrambled direction numbers and digital shifts in the kernel; FP64 parity
1e-12 relative to the value scale).
"""
import numpy as np
import pytest

import oracle as orc
from qiw import models, sobol
from qiw.diagrammatics import get_topologies_at_order
from qiw.inchworm import RandomizationParams, TopologiesInputData, correlator_2p, inchworm_step
from test_multirank import OracleDevice

SEED = 11
N_SEQS = 6
N = 32

DEVICES = ["oracle", pytest.param("gpu", marks=pytest.mark.gpu)]


def _dev(kind, request):
    return OracleDevice() if kind == "oracle" else request.getfixturevalue("device")


def _tol(kind):
    """(relative bound on means, bound on stds relative to the mean scale)."""
    return (1e-13, 1e-12) if kind == "oracle" else (1e-12, 1e-12)


def _bold_tds(orders, rp):
    tds = []
    for o in orders:
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = get_topologies_at_order(0) if o == 0 else get_topologies_at_order(o, npa)
            tds.append(TopologiesInputData(o, npa, tops, N, rp))
    return tds


def _pack(blocks):
    return np.concatenate([b.ravel(order="F") for b in blocks])


def _ref_step(exp, tds, t, target):
    """inchworm_step's randomized groups, one sequence at a time (src/inchworm.jl:147-196)."""
    ob = orc.OracleProblem(exp)
    rng = sobol.NumpyBitRNG(SEED)
    contrib, stds = {}, {}
    for td in tds:
        tl = [(x.pairs, x.parity) for x in td.topologies]
        D = 2 * td.order
        if D == 0:
            mean = _pack(ob.integrate("bold", 0, 0, tl, *t, N, sample_range=(0, 1)))
            std = np.zeros_like(mean, dtype=float)
        else:
            f = lambda m, x0, td=td, tl=tl: _pack(ob.integrate("bold", td.order, td.n_pts_after, tl, *t, N,
                                                               m=m, x0=x0))
            new_seq = lambda D=D: sobol.scramble(orc.sobol_directions(D), rng)
            mean, std = orc.mean_std_from_randomization(f, new_seq, N_SEQS, target)
        contrib[td.order] = contrib.get(td.order, 0) + mean
        stds[td.order] = stds.get(td.order, 0) + std
    return contrib, stds, rng


def _sbm_vec(sbm, S):
    return _pack([sbm[s][1] for s in range(S)])


def _targets(stds):
    """Never stop (0), stop after two sequences (huge), and a threshold between the groups."""
    mid = 0.5 * min(float(np.max(np.abs(v))) for o, v in stds.items() if o > 0)
    return [0.0, 1e9, mid]


@pytest.mark.parametrize("kind", DEVICES)
@pytest.mark.parametrize("which", [0, 1, 2])
def test_inchworm_step_randomization_matches_sequential_reference(which, kind, request):
    exp = models.anderson(n_tau=10)
    g = exp.grid
    t = (g.tau(0), g.tau(4), g.tau(5))
    target = _targets(_ref_step(exp, _bold_tds(range(0, 3), None), t, 0.0)[1])[which]
    want, want_std, rng_ref = _ref_step(exp, _bold_tds(range(0, 3), None), t, target)
    rp = RandomizationParams(rng=sobol.NumpyBitRNG(SEED), N_seqs=N_SEQS, target_std=target)
    _, contribs, stds = inchworm_step(exp, *t, _bold_tds(range(0, 3), rp), dev=_dev(kind, request))
    S = len(exp.dims)
    rel, srel = _tol(kind)
    for o in want:
        got = _sbm_vec(contribs[o], S)
        scale = np.abs(want[o]).max()
        assert np.abs(got - want[o]).max() <= rel * scale
        if o > 0:
            gs = _sbm_vec(stds[o], S).real
            bound = 1e-12 * max(np.abs(want_std[o]).max(), 1e-300) if kind == "oracle" else srel * scale
            assert np.abs(gs - want_std[o]).max() <= bound
    # the generator is left where the sequential reference leaves it
    assert rp.rng.g.integers(1 << 62) == rng_ref.g.integers(1 << 62)


def _ref_corr(exp, orders, taus, target):
    """correlator_2p with RequestStdDev, sequentially (src/inchworm.jl:805-889, 995-1045)."""
    ob = orc.OracleProblem(exp)
    rng = sobol.NumpyBitRNG(SEED)
    groups = []
    for o in orders:
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = get_topologies_at_order(o, npa, with_external_arc=True)
            if tops:
                groups.append((o, npa, [(x.pairs, x.parity) for x in tops]))
    Z = ob.partition_function()
    gs, ss = [], []
    for c in range(len(exp.corr_operators)):
        gv, sv = np.zeros(len(taus), complex), np.zeros(len(taus))
        for q, j in enumerate(taus):
            t = (exp.grid.tau(0), exp.grid.tau(j), exp.grid.tau(exp.grid.n_tau - 1))
            val, sd = 0j, 0.0
            for (o, npa, tl) in (groups[:1] if j == 0 else groups):
                if o == 0:
                    val += sum(np.trace(b) for b in ob.integrate("corr", 0, 0, tl, *t, N, corr=c, sample_range=(0, 1)))
                    continue
                f = lambda m, x0, o=o, npa=npa, tl=tl, t=t: sum(
                    np.trace(b) for b in ob.integrate("corr", o, npa, tl, *t, N, corr=c, m=m, x0=x0))
                mean, std = orc.mean_std_from_randomization(
                    f, lambda o=o: sobol.scramble(orc.sobol_directions(2 * o), rng), N_SEQS, target)
                val += mean[0]
                sd += float(std[0].real)
            gv[q], sv[q] = val / Z, sd / Z.real
        gs.append(gv)
        ss.append(sv)
    return gs, ss, rng


@pytest.mark.parametrize("kind", DEVICES)
@pytest.mark.parametrize("target", [0.0, 1e9, 2e-3])
def test_correlator_request_std_matches_sequential_reference(target, kind, request):
    exp = models.anderson(n_tau=10, corr=True)
    taus = [0, 4, 9]
    want, want_std, rng_ref = _ref_corr(exp, range(0, 3), taus, target)
    rp = RandomizationParams(rng=sobol.NumpyBitRNG(SEED), N_seqs=N_SEQS, target_std=target)
    got, got_std = correlator_2p(exp, range(0, 3), N, rand_params=rp, dev=_dev(kind, request), request_std=True,
                                 taus=taus)
    rel, srel = _tol(kind)
    for a, b in zip(got, want):
        assert np.abs(a - b).max() <= rel * np.abs(b).max()
    for a, b, g in zip(got_std, want_std, want):
        bound = 1e-12 * max(np.abs(b).max(), 1e-300) if kind == "oracle" else srel * np.abs(g).max()
        assert np.abs(a - b).max() <= bound
    assert rp.rng.g.integers(1 << 62) == rng_ref.g.integers(1 << 62)


@pytest.mark.parametrize("kind", DEVICES)
@pytest.mark.parametrize("target", [0.0, 1e9, 2e-3])
def test_diff_inchworm_randomization_matches_sequential_reference(target, kind, request):
    """diff_inchworm! with scrambled sequences: order 1 exact (no draws), order k >= 2 draws
    2k-dimensional scrambles of which the transform reads the first 2k - 2 coordinates
    (src/inchworm.jl:566-597)."""
    from qiw.inchworm import diff_inchworm
    rng_ref = sobol.NumpyBitRNG(SEED)
    exp_ref = models.anderson(n_tau=6)
    pb, _, want_std = orc.diff_inchworm(
        exp_ref, range(0, 4), N,
        rand=(lambda D: sobol.scramble(orc.sobol_directions(D), rng_ref), N_SEQS, target))
    exp = models.anderson(n_tau=6)
    rp = RandomizationParams(rng=sobol.NumpyBitRNG(SEED), N_seqs=N_SEQS, target_std=target)
    _, sig_std = diff_inchworm(exp, range(0, 4), N, rand_params=rp, dev=_dev(kind, request))
    rel = 1e-13 if kind == "oracle" else 1e-11
    for s, P_s in enumerate(exp.P):
        want = pb.P_data[s]
        assert np.abs(P_s.data - want).max() <= rel * np.abs(want).max()
    S = len(exp.dims)
    for n in range(exp.grid.n_tau - 1):
        got = np.concatenate([sum(sig_std[o][s].data[n + 1] for o in sig_std).ravel() for s in range(S)]).real
        assert got.shape == want_std[n].shape
        assert np.all(np.isfinite(got))
        assert np.abs(got - want_std[n]).max() <= 1e-12 * max(np.abs(want_std[n]).max(), 1.0)
    assert rp.rng.g.integers(1 << 62) == rng_ref.g.integers(1 << 62)
