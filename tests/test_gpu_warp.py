"""Learned simplex warp on the GPU: hand-written forward/backward kernels against the CPU
reference (tests/warp_ref.py), the sampler against the reference, and what a trained warp
gains over plain qMC on a real topology group (variance over randomized Sobol sequences, with
the warped estimate checked for bias against the plain one)."""
import numpy as np
import pytest

import oracle as orc
import warp_ref as wr
from qiw import _lib, models
from qiw import warp as qwarp
from qiw.device import Work
from qiw.diagrammatics import get_topologies_at_order
from qiw.sobol import direction_numbers

pytestmark = pytest.mark.gpu


def _random_params(D, seed):
    rng = np.random.default_rng(seed)
    return wr.bf16(rng.normal(0, 0.3, wr.Layout(D).n) * wr.masks(D))


def test_warp_gradient_matches_cpu_reference(device):
    D = 6
    wid = device.warp_create(D, seed=1)
    p = _random_params(D, 7)
    device.warp_set_params(wid, p)
    assert np.array_equal(device.warp_params(wid), p)
    rng = np.random.default_rng(3)
    X = rng.random((777, D))
    w = rng.random(777) + 0.05
    g_gpu, loss_gpu = device.warp_grad(wid, X, w)
    loss_cpu, g_cpu = wr.loss_grad(p, X, w)
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * abs(loss_cpu)
    assert np.linalg.norm(g_gpu - g_cpu) <= 1e-3 * np.linalg.norm(g_cpu)


def test_warp_masks_match_cpu_reference(device):
    D = 5
    wid = device.warp_create(D, seed=4)
    device.warp_set_params(wid, np.ones(wr.Layout(D).n))
    assert np.array_equal(device.warp_params(wid), wr.masks(D))


def test_warp_map_matches_cpu_reference(device):
    D = 4
    wid = device.warp_create(D, seed=2)
    p = _random_params(D, 11)
    device.warp_set_params(wid, p)
    n = 4096
    pts = device.warp_map(wid, D, 0, n)
    Y = orc.sobol_points(direction_numbers(D), None, 0, n)
    X, wt = wr.warp_map(p, Y.astype(np.float32).astype(np.float64))
    close = np.all(np.abs(pts[:, :D] - X) < 1e-5, axis=1)
    assert close.mean() > 0.999          # bin-edge ties may resolve differently in FP32
    # FP32 knot heights: the weight 1/q carries a relative error of a few 1e-6 per dimension
    assert np.mean(np.isclose(pts[close, D], wt[close], rtol=1e-4, atol=0)) > 0.999
    assert abs(pts[:, D].mean() - 1.0) < 0.02   # E_y[1/q(x(y))] = 1


def test_trained_warp_reduces_variance_without_bias(device):
    """Anderson model at beta = 40, U = 4: |f| of the order-3 group is concentrated near short
    hybridization lines, and the trained warp lowers the randomized-qMC variance."""
    exp = models.anderson(beta=40.0, U=4.0, eps=-2.0, n_tau=128)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    order, npa = 3, 3
    gid = device.create_group(_lib.QIW_GROUP_BOLD, order, npa, get_topologies_at_order(order, npa))
    work = Work(gid, g.tau(0), g.tau(32), g.tau(33), 0, 0, 0)
    fit = qwarp.fit_group_warp(device, work, R=16)
    print(f"variance gain of the trained warp: {fit.gain:.2f} (bias {fit.bias_sigma:.2f} sigma, "
          f"training loss {fit.loss:.3f}; 0 is the uniform density)")
    assert fit.bias_sigma <= 4
    assert fit.warp_id is not None
    assert fit.gain > 5


def test_warp_dropped_where_plain_qmc_is_better(device):
    """eg model (n_tau = 256) at inch step 200, order 3 with 5 points after t_w: the fitted warp
    has a far larger variance than plain Sobol, so fit_group_warp drops it; at an early step
    (|f| nearly flat) the warp gains little, and a caller asking for a real gain (min_gain) gets
    plain qMC."""
    exp = models.eg_discrete_bath(n_tau=256)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 3, 5, get_topologies_at_order(3, 5))
    fit = qwarp.fit_group_warp(device, Work(gid, g.tau(0), g.tau(200), g.tau(201), 0, 0, 0))
    assert fit.bias_sigma <= 4
    assert fit.gain < 1 and fit.warp_id is None
    exp = models.eg_discrete_bath(n_tau=64)
    g = exp.grid
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    gid = device.create_group(_lib.QIW_GROUP_BOLD, 2, 2, get_topologies_at_order(2, 2))
    fit = qwarp.fit_group_warp(device, Work(gid, g.tau(0), g.tau(16), g.tau(17), 0, 0, 0), min_gain=3.0)
    assert fit.bias_sigma <= 4
    assert fit.gain < 3.0 and fit.warp_id is None


def test_inchworm_with_warp_policy_is_unbiased(device):
    """Whole inchworm! with warps refitted every few steps (kept where they lower the variance):
    the result stays an estimate of the same P -- its error against a plain 2^15 reference is
    of the plain run's size or smaller."""
    from qiw.inchworm import inchworm
    from qiw.warp import WarpPolicy

    def solve(N, policy=None):
        exp = models.eg_discrete_bath(n_tau=24)
        inchworm(exp, range(0, 4), range(0, 4), N, dev=device, warp_policy=policy)
        return [P_s.data.copy() for P_s in exp.P]

    ref = solve(2 ** 15)
    err = lambda P: max(np.abs(a - b).max() for a, b in zip(P, ref))
    e_plain = err(solve(1024))
    e_warp = err(solve(1024, WarpPolicy(refit_every=6, first_step=4, n_train=2 ** 14, R=8)))
    print(f"eg n_tau=24, N=1024: error plain {e_plain:.2e}, warped {e_warp:.2e}")
    assert np.isfinite(e_warp) and e_warp < 1.5 * e_plain


def test_concurrent_training_equals_one_at_a_time(device):
    """qiw_warp_train_batch trains distinct warps concurrently on several streams; each warp's
    parameters and final loss equal those of training it alone (qiw_warp_train)."""
    rng = np.random.default_rng(21)
    data = []
    for D in (2, 4, 6, 8, 4):
        n = int(rng.integers(3000, 9000))
        data.append((D, rng.random((n, D)), rng.random(n) + 0.01))
    solo, solo_loss = [], []
    for k, (D, X, w) in enumerate(data):
        wid = device.warp_create(D, seed=30 + k)
        solo_loss.append(device.warp_train(wid, X, w, steps=40, batch=1024, lr=3e-3))
        solo.append(device.warp_params(wid))
    wids = [device.warp_create(D, seed=30 + k) for k, (D, _, _) in enumerate(data)]
    loss = device.warp_train_batch(wids, [X for (_, X, _) in data], [w for (_, _, w) in data], steps=40,
                                   batch=1024, lr=3e-3)
    for k, wid in enumerate(wids):
        assert np.array_equal(device.warp_params(wid), solo[k]), k
        assert loss[k] == solo_loss[k]


def test_per_sample_values_of_several_items_in_one_launch(device):
    """qiw_integrate_samples_batch returns each item's per-sample values, equal to one
    qiw_integrate_samples call per item (batches of a sample are summed by atomics, so the
    last bit may differ), and sums equal to the items' integrals; qiw_integrate_sample_norms
    returns their norms."""
    exp = models.eg_discrete_bath(n_tau=40)
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    g = exp.grid
    works = []
    for (o, npa, first, n) in ((1, 1, 0, 64), (2, 2, 5, 100), (3, 3, 1000, 37)):
        gid = device.create_group(_lib.QIW_GROUP_BOLD, o, npa, get_topologies_at_order(o, npa))
        works.append(Work(gid, g.tau(0), g.tau(20), g.tau(21), first, n, 4096))
    blocks, samples = device.integrate_samples_batch(works, _lib.QIW_PREC_FP64)
    _, norms = device.integrate_sample_norms(works, _lib.QIW_PREC_FP64)
    for s, nr in zip(samples, norms):   # the training weights ||f_i||, computed on the device
        assert np.allclose(nr, np.linalg.norm(s, axis=1), rtol=1e-14, atol=0)
    for wk, b, s in zip(works, blocks, samples):
        b1, s1 = device.integrate_samples(wk, _lib.QIW_PREC_FP64)
        assert s.shape == s1.shape == (wk.n_samples, s1.shape[1])
        assert np.allclose(s, s1, rtol=1e-13, atol=1e-13 * np.abs(s1).max())
        for x, y in zip(b, b1):
            assert np.allclose(x, y, rtol=1e-13, atol=1e-15)


def test_fitting_groups_together_equals_one_at_a_time(device):
    """fit_group_warps (one launch for all training samples, concurrent training, one launch per
    estimator for the replicas) gives every group the gain and loss of fitting it alone."""
    exp = models.eg_discrete_bath(n_tau=64)
    device.set_problem(exp)
    device.set_ppgf(exp.P)
    g = exp.grid
    t = (g.tau(0), g.tau(60), g.tau(61))
    works = []
    for (o, npa) in ((1, 1), (2, 1), (2, 2), (3, 3)):
        gid = device.create_group(_lib.QIW_GROUP_BOLD, o, npa, get_topologies_at_order(o, npa))
        works.append(Work(gid, *t, 0, 0, 0))
    kw = dict(n_train=2 ** 12, steps=60, R=4, N_test=256)
    together = qwarp.fit_group_warps(device, works, **kw)
    for wk, f in zip(works, together):
        alone = qwarp.fit_group_warp(device, wk, **kw)
        assert np.isclose(f.gain, alone.gain, rtol=1e-6) and np.isclose(f.loss, alone.loss, rtol=1e-6)
        assert (f.warp_id is None) == (alone.warp_id is None)


def test_training_the_same_warp_twice_at_once_is_rejected(device):
    from qiw._lib import QiwError
    wid = device.warp_create(4, seed=1)
    X = np.random.default_rng(0).random((256, 4))
    with pytest.raises(QiwError, match="twice"):
        device.warp_train_batch([wid, wid], [X, X], [np.ones(256)] * 2, steps=2, batch=128)
