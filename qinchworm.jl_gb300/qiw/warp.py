"""Learned warps for the qMC integral of one topology group: training and the keep/drop choice.

A warp (qiw_warp_* in the C ABI) is a triangular monotone map of the Sobol hypercube fitted to
|f| of one group at one inch time.  It lowers the randomized-qMC variance where |f| is
concentrated (late inch steps, large beta) and raises it where |f| is nearly flat, because
plain Sobol points are then already close to optimal and the map adds kinks to a smooth
integrand.  ``fit_group_warp`` therefore trains a warp and keeps it only when R scrambled
replicas of both estimators show the warped one to have the smaller variance.

The reference has no counterpart: its qMC integrals always use the fixed simplex transforms
(src/qmc_integrate.jl:99-334).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

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


def _replicas(dev: Device, work: Work, seqs, N: int, warp_id, precision):
    """The group's N-point estimate on each scrambled sequence (m, x0) of seqs, in one launch."""
    R = len(seqs)
    wk = [Work(work.group, work.t_i, work.t_w, work.t_f, 0, N, N, m, x0) for (m, x0) in seqs]
    res = dev.integrate(wk, precision, warps=None if warp_id is None else [warp_id] * R)
    return np.array([np.concatenate([b.ravel() for b in blocks]) for blocks in res])


def fit_group_warp(dev: Device, work: Work, n_train: int = 2 ** 15, steps: int = 600,
                   batch: int = 4096, lr: float = 3e-3, uniform_mix: float = 0.3,
                   N_test: int = 1024, R: int = 8, seed: int = 0,
                   min_gain: float = 1.0, precision: int = _lib.QIW_PREC_FP32) -> WarpFit:
    """Train a warp for ``work``'s group at its inch times and decide whether to use it.

    Training data are ``n_train`` plain Sobol samples of the group (their per-sample values
    from qiw_integrate_samples, weight ||f||).  The decision compares the variances of R
    scrambled replicas of N_test points each (one launch per estimator); the warp is kept when
    plain/warped > min_gain.  The fit's own integrand evaluations run in ``precision`` (FP32
    chains by default: the fit needs |f| and variance ratios, not 1e-12 values).
    """
    order = dev.group_info[work.group][1]
    D = 2 * order
    if D < 2:
        return WarpFit(None, 1.0, 0.0, 0.0)
    _, samples = dev.integrate_samples(Work(work.group, work.t_i, work.t_w, work.t_f, 0, n_train, n_train), precision)
    w = np.linalg.norm(samples, axis=1)
    if not np.any(w > 0):
        return WarpFit(None, 1.0, 0.0, 0.0)
    X = sobol_points(direction_numbers(D), 0, n_train)
    wid = dev.warp_create(D, seed=seed + 5, uniform_mix=uniform_mix)
    loss = dev.warp_train(wid, X, w + 1e-300, steps=steps, batch=batch, lr=lr)
    seqs = [scramble(direction_numbers(D), NumpyBitRNG(1000 + seed + r)) for r in range(R)]
    plain = _replicas(dev, work, seqs, N_test, None, precision)
    warped = _replicas(dev, work, seqs, N_test, wid, precision)
    vp = float(np.sum(np.var(plain, axis=0, ddof=1)))
    vw = float(np.sum(np.var(warped, axis=0, ddof=1)))
    gain = vp / vw if vw > 0 else np.inf
    noise = np.sqrt((vp + vw) / R)
    bias = float(np.linalg.norm(plain.mean(0) - warped.mean(0)) / noise) if noise > 0 else 0.0
    return WarpFit(wid if gain > min_gain else None, gain, float(loss), bias)
