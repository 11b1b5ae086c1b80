"""The CPU reference of the learned warp: analytic gradient against finite differences,
and the sampler's density integrating to one."""
import numpy as np

import warp_ref as wr


def _params(D, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, wr.Layout(D).n) * wr.masks(D)
    return wr.bf16(p)   # exactly representable in BF16, so rounding is the identity


def test_gradient_matches_finite_differences():
    D = 4
    p = _params(D, 1)
    rng = np.random.default_rng(2)
    X = rng.random((200, D))
    w = rng.random(200) + 0.1
    loss, g = wr.loss_grad(p, X, w)
    m = wr.masks(D)
    idx = np.flatnonzero(m)[::97][:40]
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        # evaluate without BF16 rounding of the perturbed entry: use the float64 path
        lp = _loss64(pp, X, w)
        lm = _loss64(pm, X, w)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i]))


def _loss64(p, X, w):
    old = wr.bf16
    wr.bf16 = lambda q: np.asarray(q, dtype=np.float64)
    try:
        return wr.loss_grad(p, X, w)[0]
    finally:
        wr.bf16 = old


def test_sampler_density_integrates_to_one():
    D = 3
    p = _params(D, 3)
    from scipy.stats import qmc
    Y = qmc.Sobol(d=D, scramble=False).random_base2(m=13)
    X, wt = wr.warp_map(p, Y)
    assert np.all((X >= 0) & (X < 1))
    assert abs(wt.mean() - 1.0) < 0.02


def test_sobol_points_match_oracle():
    import oracle as orc
    from qiw.sobol import direction_numbers, sobol_points, scramble, NumpyBitRNG
    m = direction_numbers(6)
    assert np.array_equal(sobol_points(m, 37, 500), orc.sobol_points(m, None, 37, 500))
    ms, x0 = scramble(m, NumpyBitRNG(3))
    assert np.array_equal(sobol_points(ms, 0, 300, x0), orc.sobol_points(ms, x0, 0, 300))
