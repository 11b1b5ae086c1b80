"""Learned warps for the qMC integral of one topology group: training and the keep/drop choice.

A warp (qiw_warp_* in the C ABI) is a triangular monotone map of the Sobol hypercube fitted to
|f| of one group at one inch time.  It lowers the randomized-qMC variance where |f| is
concentrated (late inch steps, large beta) and raises it where |f| is nearly flat, because
plain Sobol points are then already close to optimal and the map adds kinks to a smooth
integrand.  ``fit_group_warps`` therefore trains a warp and keeps it only when R scrambled
replicas of both estimators show the warped one to have the smaller variance.

The reference has no counterpart: its qMC integrals always use the fixed simplex transforms
(src/qmc_integrate.jl:99-334).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .device import Device, Work
from .sobol import NumpyBitRNG, direction_numbers, scramble, sobol_points


@dataclass
class WarpPolicy:
    """When inchworm() fits warps: at step first_step and every refit_every steps after it, for
    every bold group of order >= 1 (2*order <= 8), kept only where they lower the variance."""
    refit_every: int = 16
    first_step: int = 4
    n_train: int = 2 ** 15
    train_steps: int = 600
    uniform_mix: float = 0.3
    N_test: int = 1024
    R: int = 8
    min_gain: float = 1.0


@dataclass
class WarpFit:
    warp_id: Optional[int]      # None: plain qMC is the better estimator
    gain: float                 # measured variance ratio plain / warped
    loss: float                 # final |f|-weighted negative log-likelihood (0 = uniform)
    bias_sigma: float           # |mean difference| of the two estimators in standard errors


def _replicas(dev: Device, items, N: int, precision, warped: bool):
    """Each item's N-point estimate on each of its scrambled sequences, all in one launch.
    items: (work, seqs [(m, x0)], warp id); returns per item an array [len(seqs)][sum d^2]."""
    wk, ids = [], []
    for (work, seqs, wid) in items:
        wk += [Work(work.group, work.t_i, work.t_w, work.t_f, 0, N, N, m, x0) for (m, x0) in seqs]
        ids += [wid] * len(seqs)
    res = dev.integrate(wk, precision, warps=ids if warped else None)
    flat = [np.concatenate([b.ravel() for b in blocks]) for blocks in res]
    out, k = [], 0
    for (_, seqs, _) in items:
        out.append(np.array(flat[k:k + len(seqs)]))
        k += len(seqs)
    return out


def fit_group_warps(dev: Device, works: Sequence[Work], n_train: int = 2 ** 15, steps: int = 600,
                    batch: int = 4096, lr: float = 3e-3, uniform_mix: float = 0.3,
                    N_test: int = 1024, R: int = 8, seed: int = 0,
                    min_gain: float = 1.0, precision: int = _lib.QIW_PREC_FP32) -> List[WarpFit]:
    """Train a warp for each work item's group at its inch times and decide whether to use it.

    Training data are ``n_train`` plain Sobol samples of the group (weight ||f|| of their
    per-sample values, qiw_integrate_sample_norms).  The decision compares the variances of R
    scrambled replicas of N_test points each; the warp is kept when plain/warped > min_gain.
    The fit's own integrand evaluations run in ``precision`` (FP32 chains by default: the fit
    needs |f| and variance ratios, not 1e-12 values).  All groups share each step: one launch
    for the training samples, one concurrent training of all warps, one launch per estimator
    for the replicas; the results equal fitting the groups one at a time.
    """
    fits: List[Optional[WarpFit]] = [None] * len(works)
    live = []
    for i, work in enumerate(works):
        D = 2 * dev.group_info[work.group][1]
        if D < 2:
            fits[i] = WarpFit(None, 1.0, 0.0, 0.0)
        else:
            live.append((i, work, D))
    if live:
        _, norms = dev.integrate_sample_norms(
            [Work(w.group, w.t_i, w.t_w, w.t_f, 0, n_train, n_train) for (_, w, _) in live], precision)
        train = []
        for (i, work, D), w in zip(live, norms):
            if np.any(w > 0):
                train.append((i, work, D, w))
            else:
                fits[i] = WarpFit(None, 1.0, 0.0, 0.0)
        X, seqs = {}, {}
        for (_, _, D, _) in train:
            if D not in X:
                X[D] = sobol_points(direction_numbers(D), 0, n_train)
                seqs[D] = [scramble(direction_numbers(D), NumpyBitRNG(1000 + seed + r)) for r in range(R)]
        wids = [dev.warp_create(D, seed=seed + 5, uniform_mix=uniform_mix) for (_, _, D, _) in train]
        if train:
            losses = dev.warp_train_batch(wids, [X[D] for (_, _, D, _) in train],
                                          [w + 1e-300 for (_, _, _, w) in train], steps=steps, batch=batch, lr=lr)
            items = [(work, seqs[D], wid) for (_, work, D, _), wid in zip(train, wids)]
            plain = _replicas(dev, items, N_test, precision, warped=False)
            warped = _replicas(dev, items, N_test, precision, warped=True)
            for (i, _, _, _), wid, loss, vp_r, vw_r in zip(train, wids, losses, plain, warped):
                vp = float(np.sum(np.var(vp_r, axis=0, ddof=1)))
                vw = float(np.sum(np.var(vw_r, axis=0, ddof=1)))
                gain = vp / vw if vw > 0 else np.inf
                noise = np.sqrt((vp + vw) / R)
                bias = float(np.linalg.norm(vp_r.mean(0) - vw_r.mean(0)) / noise) if noise > 0 else 0.0
                fits[i] = WarpFit(wid if gain > min_gain else None, gain, float(loss), bias)
    return fits


def fit_group_warp(dev: Device, work: Work, n_train: int = 2 ** 15, steps: int = 600,
                   batch: int = 4096, lr: float = 3e-3, uniform_mix: float = 0.3,
                   N_test: int = 1024, R: int = 8, seed: int = 0,
                   min_gain: float = 1.0, precision: int = _lib.QIW_PREC_FP32) -> WarpFit:
    """fit_group_warps of one work item."""
    return fit_group_warps(dev, [work], n_train=n_train, steps=steps, batch=batch, lr=lr,
                           uniform_mix=uniform_mix, N_test=N_test, R=R, seed=seed, min_gain=min_gain,
                           precision=precision)[0]
