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
