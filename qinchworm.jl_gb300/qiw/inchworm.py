"""Host mirror of the reference's inchworm driver (`src/inchworm.jl`) on the GPU path.

Same entry points, argument meaning and results as the reference:
  * `inchworm_step`, `inchworm_step_bare`  (src/inchworm.jl:123-304)
  * `inchworm`  == inchworm!               (src/inchworm.jl:332-498)
  * `correlator_2p`                        (src/inchworm.jl:805-1084)
Every qMC integral -- the `contour_integral(t -> eval(td.topologies, t), ...)` closures -- runs
in the CUDA library; one inch step issues a single launch covering all its topology groups.
The host keeps what the reference keeps on the host: topology generation, set_ppgf!,
normalize! and the (optional) rank decomposition and all-reduce.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from . import ppgf as _ppgf
from .device import Device, Work, blocks_to_sbm
from .diagrammatics import Topology, get_topologies_at_order
from .ed import SectorBlockMatrix
from .gf import ImaginaryTimeGF
from .sobol import scramble


@dataclass
class RandomizationParams:
    """src/randomization.jl:46-57: rng None means unscrambled (and one sequence)."""
    rng: Optional[object] = None
    N_seqs: int = 1
    target_std: float = 0.0


@dataclass
class TopologiesInputData:
    """src/inchworm.jl:76-87."""
    order: int
    n_pts_after: int
    topologies: List[Topology]
    N_samples: int
    rand_params: RandomizationParams = field(default_factory=RandomizationParams)


class Comm:
    """Rank decomposition of the sample range (src/mpi.jl:49-54, 104-127).  The default is a
    single rank; `TorchComm` provides an all-reduce over torch.distributed."""
    rank = 0
    size = 1

    def allreduce(self, v: np.ndarray) -> np.ndarray:
        return v


class TorchComm(Comm):
    def __init__(self):
        import torch.distributed as dist
        self.dist = dist
        self.rank = dist.get_rank()
        self.size = dist.get_world_size()

    def allreduce(self, v: np.ndarray) -> np.ndarray:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(v))
        self.dist.all_reduce(t)
        return t.numpy()


def split_count(N: int, n: int) -> List[int]:
    q, r = divmod(N, n)
    return [q + 1 if i < r else q for i in range(n)]


def rank_sub_range(N: int, comm: Comm) -> Tuple[int, int]:
    """0-based (start, length) of this rank's chunk."""
    chunks = split_count(N, comm.size)
    return sum(chunks[:comm.rank]), chunks[comm.rank]


def _pack_blocks(blocks: List[np.ndarray]) -> np.ndarray:
    return np.concatenate([b.ravel(order="F") for b in blocks])


def _unpack_blocks(v: np.ndarray, dims) -> List[np.ndarray]:
    out, o = [], 0
    for d in dims:
        out.append(v[o:o + d * d].reshape(d, d, order="F").copy())
        o += d * d
    return out


def _rng_state(rng):
    return copy.deepcopy(rng.__dict__)


def _rng_set(rng, state) -> None:
    rng.__dict__.clear()
    rng.__dict__.update(copy.deepcopy(state))


def _mean_std(vs: np.ndarray):
    std = vs.std(axis=0, ddof=1) if len(vs) > 1 else np.full(vs.shape[1], np.nan)
    return vs.mean(axis=0), std


def _randomized(groups, sobol, launch, stat):
    """mean_std_from_randomization (src/randomization.jl:86-100) for every group of one call,
    with the reference's draws: groups in order, group g draws the scramble of sequence s only
    when it evaluates it, and stops after s > 1 once the largest |std(samples[1:s])| is at most
    target_std.  Unscrambled sequences are all the same sequence: one evaluation, std 0 (NaN for
    N_seqs = 1, as Julia's std of one sample).  D = 0 marks an exact group (order 0, and order 1
    of the self-energy, src/inchworm.jl:566-571): one evaluation, no draws, std 0.

    groups[i] is None or (D, RandomizationParams), D the dimension of the scrambled sequence
    (2k; the kernel may read fewer coordinates); launch(items), items a list of (i, [(m, x0),
    ...]) (m None for D = 0), returns {i: [all-reduced packed value per sequence]} from one
    qiw_integrate call; stat(i, v) is the quantity the statistics apply to.  Every sequence of
    every pending group runs in one launch; when a group stops early, the scrambling generators
    are set back to where the reference leaves them and the later groups are drawn and run
    again.  Returns per group (mean, std) of stat."""
    out = [None] * len(groups)
    todo = [i for i, g in enumerate(groups) if g is not None]
    while todo:
        items, snaps = [], {}
        for i in todo:
            D, rp = groups[i]
            if D == 0 or rp.rng is None:
                items.append((i, [(sobol(D), np.zeros(D, np.uint32)) if D else (None, None)]))
                continue
            pre, post, seqs = _rng_state(rp.rng), [], []
            for _ in range(rp.N_seqs):
                seqs.append(scramble(sobol(D), rp.rng))
                post.append(_rng_state(rp.rng))
            snaps[i] = (pre, post)
            items.append((i, seqs))
        vals = launch(items)
        restart = None
        for pos, i in enumerate(todo):
            D, rp = groups[i]
            vs = np.array([stat(i, v) for v in vals[i]])
            if D == 0 or rp.rng is None:
                exact_or_many = D == 0 or rp.N_seqs > 1
                out[i] = (vs[0], np.zeros(vs.shape[1]) if exact_or_many else np.full(vs.shape[1], np.nan))
                continue
            k = len(vs)
            for s_ in range(2, len(vs) + 1):
                if np.max(vs[:s_].std(axis=0, ddof=1)) <= rp.target_std:
                    k = s_
                    break
            out[i] = _mean_std(vs[:k])
            if k < len(vs):
                restart = (pos, i, k)
                break
        if restart is None:
            break
        pos, i, k = restart
        rng = groups[i][1].rng
        _rng_set(rng, snaps[i][1][k - 1])
        todo = todo[pos + 1:]
        seen = {id(rng)}
        for j in todo:   # other generators: back to their state before this round's later draws
            Dj, rpj = groups[j]
            if j in snaps and id(rpj.rng) not in seen:
                _rng_set(rpj.rng, snaps[j][0])
                seen.add(id(rpj.rng))
    return out


class _Session:
    """Per-run state: device, problem upload and planned groups."""

    def __init__(self, dev: Optional[Device], expansion, seq_offset: int = 0):
        if seq_offset < 0:
            raise ValueError("seq_offset must be non-negative")
        self.seq_offset = int(seq_offset)   # leading Sobol points skipped by every sampled group
        self.dev = dev if dev is not None else Device(0)
        key = (id(expansion), len(expansion.corr_operators), len(expansion.pairs))
        if getattr(self.dev, "_expansion", None) is not expansion or getattr(self.dev, "_problem_key", None) != key:
            self.dev.set_problem(expansion)
            self.dev._expansion = expansion
            self.dev._problem_key = key
            self.dev._groups = {}
        self.exp = expansion
        self._by_td: Dict[tuple, tuple] = {}

    def group(self, kind: int, td: TopologiesInputData, corr: Optional[int] = None) -> int:
        hit = self._by_td.get((kind, id(td), corr))
        if hit is not None and hit[0] is td:
            return hit[1]
        key = (kind, td.order, td.n_pts_after, corr, tuple((t.pairs, t.parity) for t in td.topologies))
        g = self.dev._groups.get(key)
        if g is None:
            g = self.dev.create_group(kind, td.order, td.n_pts_after, td.topologies, corr)
            self.dev._groups[key] = g
        self._by_td[(kind, id(td), corr)] = (td, g)   # td kept alive, so its id stays its own
        return g

    def run(self, kind: int, tds: Sequence[TopologiesInputData], t_i, t_w, t_f, precision, comm: Comm,
            corr: Optional[int] = None, warps: Optional[Dict[int, int]] = None):
        """All groups of a step; returns per group (mean blocks, std blocks or None).  `warps`
        maps a group id to a learned warp its samples are drawn through."""
        dims = self.exp.dims
        entries = []
        for td in tds:
            D = 2 * td.order - (2 if kind == _lib.QIW_GROUP_SIGMA else 0)   # integrated times
            if D > 0 and td.N_samples <= 0:
                entries.append(None)
                continue
            entries.append((self.group(kind, td, corr), td, D))
        # Scrambled-sequence dimension: 2k for every sampled group.  Self-energy groups integrate
        # 2k - 2 times but the reference draws a 2k-dimensional sequence and the transform reads
        # its first 2k - 2 coordinates (src/inchworm.jl:582-594), so the kernel gets those rows.
        seq_dims = [None if e is None else (0 if e[2] == 0 else 2 * e[1].order) for e in entries]

        def launch(items):
            # one launch for every (group, sequence) of the step
            works, index = [], []
            for i, seqs in items:
                gid, td, D = entries[i]
                start, length = (0, 1) if D == 0 else rank_sub_range(td.N_samples, comm)  # exact: once per rank
                if D > 0:
                    start += self.seq_offset
                for m, x0 in seqs:
                    if m is not None and m.shape[0] > D:
                        m, x0 = np.ascontiguousarray(m[:D]), np.ascontiguousarray(x0[:D])
                    works.append(Work(gid, t_i, t_w, t_f, start, length, td.N_samples, m, x0))
                    index.append(i)
            wl = [warps.get(w.group, -1) for w in works] if warps else None
            if wl is not None and all(x < 0 for x in wl):
                wl = None
            if not works:
                packed = []
            elif wl is None and hasattr(self.dev, "integrate_packed"):
                packed = list(self.dev.integrate_packed(works, precision))
            elif wl is None:
                packed = [_pack_blocks(blocks) for blocks in self.dev.integrate(works, precision)]
            else:
                packed = [_pack_blocks(blocks) for blocks in self.dev.integrate(works, precision, warps=wl)]
            red = [k for k, i in enumerate(index) if entries[i][2] > 0]   # exact groups: every rank has it
            if red and comm.size > 1:   # one all-reduce for every sampled work item of the launch
                summed = comm.allreduce(np.stack([packed[k] for k in red]))
                for r, k in enumerate(red):
                    packed[k] = summed[r]
            vals: Dict[int, List[np.ndarray]] = {}
            for i, v in zip(index, packed):
                vals.setdefault(i, []).append(v)
            return vals

        # per group (mean, std) as packed vectors in sector order (see _pack_blocks)
        return _randomized([None if e is None else (sd, e[1].rand_params) for e, sd in zip(entries, seq_dims)],
                           self.dev.sobol, launch, lambda i, v: v)


def inchworm_step(expansion, t_i: float, t_w: float, t_f: float, top_data: Sequence[TopologiesInputData],
                  dev: Optional[Device] = None, precision: int = _lib.QIW_PREC_FP64, comm: Comm = Comm(),
                  seq_offset: int = 0):
    """Regular inch step; returns (value, order_contribs, order_contribs_std) as SectorBlockMatrix.
    seq_offset skips that many leading points of every sequence (skip!(seq, seq_offset,
    exact=true) before the sum, src/scrambled_sobol.jl:189-208); 0 is the reference's run."""
    ses = _Session(dev, expansion, seq_offset)
    ses.dev.set_ppgf(expansion.P)
    return _accumulate(ses.run(_lib.QIW_GROUP_BOLD, top_data, t_i, t_w, t_f, precision, comm), top_data,
                       expansion.dims)


def inchworm_step_bare(expansion, t_i: float, t_f: float, top_data: Sequence[TopologiesInputData],
                       dev: Optional[Device] = None, precision: int = _lib.QIW_PREC_FP64, comm: Comm = Comm(),
                       seq_offset: int = 0):
    """Initial step with bare propagators (all diagrams); seq_offset as in inchworm_step."""
    ses = _Session(dev, expansion, seq_offset)
    return _accumulate(ses.run(_lib.QIW_GROUP_BARE, top_data, t_i, 0.0, t_f, precision, comm), top_data,
                       expansion.dims)


def _accumulate(results, top_data, dims):
    """Sums the groups of a step per order, then the orders (the reference's order of sums,
    src/inchworm.jl:192-200), on packed vectors; returns SectorBlockMatrix values."""
    orders = sorted({td.order for td in top_data})
    L = int(sum(int(d) * int(d) for d in dims))
    contribs = {o: np.zeros(L, np.complex128) for o in orders}
    stds = {o: np.zeros(L, np.complex128) for o in orders}
    for td, r in zip(top_data, results):
        if r is None:
            continue
        mean, std = r
        contribs[td.order] = contribs[td.order] + mean
        if td.order > 0:
            stds[td.order] = stds[td.order] + std
    total = np.zeros(L, np.complex128)
    for o in orders:
        total = total + contribs[o]
    sbm = lambda v: blocks_to_sbm(_unpack_blocks(v, dims))
    return sbm(total), {o: sbm(v) for o, v in contribs.items()}, {o: sbm(v) for o, v in stds.items()}


def _zero_P(expansion):
    return [ImaginaryTimeGF(P_s.grid, P_s.norb, True) for P_s in expansion.P]


def inchworm(expansion, orders, orders_bare, N_samples: int, n_pts_after_max: Optional[int] = None,
             rand_params: Optional[RandomizationParams] = None, dev: Optional[Device] = None,
             precision: int = _lib.QIW_PREC_FP64, comm: Comm = Comm(), n_steps: Optional[int] = None,
             step_callback=None, warp_policy=None, seq_offset: int = 0):
    """inchworm!(expansion, grid, orders, orders_bare, N_samples; n_pts_after_max, rand_params).

    Writes the bold propagator into expansion.P and returns (P_orders, P_orders_std):
    dict order -> list of per-sector ImaginaryTimeGF.  `n_steps` stops after that many
    regular steps (the remaining grid points keep their atomic values).  `warp_policy`
    (qiw.warp.WarpPolicy) draws the samples of each bold group through a learned warp, refitted
    every few steps and kept only where it lowers the variance; the estimates stay unbiased.
    `seq_offset` > 0 skips that many leading points of every sequence (0: the reference's run).
    With the unscrambled sequence its first point is the origin, where every integrated time
    sits at the start of its segment; its single value can dominate the error of an N-point
    estimate as an O(1/N) term, and seq_offset=1 leaves it out."""
    assert N_samples == 0 or (N_samples & (N_samples - 1)) == 0, "N_samples must be a power of 2"
    rp = rand_params or RandomizationParams()
    assert rp.N_seqs > 0
    grid = expansion.grid
    ses = _Session(dev, expansion, seq_offset)
    orders_all = sorted(set(orders) | set(orders_bare))
    P_orders = {o: _zero_P(expansion) for o in orders_all}
    P_orders_std = {o: _zero_P(expansion) for o in orders_all}

    top_bare = [TopologiesInputData(o, 2 * o, get_topologies_at_order(o), N_samples, rp) for o in orders_bare]
    res = ses.run(_lib.QIW_GROUP_BARE, top_bare, grid.tau(0), 0.0, grid.tau(1), precision, comm)
    value, contribs, stds = _accumulate(res, top_bare, expansion.dims)
    _ppgf.set_ppgf(expansion.P, 1, value)
    for o in contribs:
        for s, (sf, m) in contribs[o].items():
            P_orders[o][s].data[1] = m
            P_orders_std[o][s].data[1] = stds[o][s][1]

    top_bold = []
    for o in orders:
        rng = [0] if o == 0 else range(1, min(2 * o - 1, n_pts_after_max or 2 * o) + 1)
        for npa in rng:
            tops = get_topologies_at_order(o, npa)
            if tops:
                top_bold.append(TopologiesInputData(o, npa, tops, N_samples, rp))

    last = grid.n_tau - 1 if n_steps is None else min(grid.n_tau - 1, 1 + n_steps)
    warps: Dict[int, int] = {}
    for n in range(1, last):
        ses.dev.set_ppgf(expansion.P)
        if warp_policy is not None and n >= warp_policy.first_step and \
                (n - warp_policy.first_step) % warp_policy.refit_every == 0:
            from .warp import fit_group_warps
            gids = [ses.group(_lib.QIW_GROUP_BOLD, td) for td in top_bold if 0 < td.order and 2 * td.order <= 8]
            fits = fit_group_warps(ses.dev, [Work(gid, grid.tau(0), grid.tau(n), grid.tau(n + 1), 0, 0, 0)
                                             for gid in gids],
                                   n_train=warp_policy.n_train, steps=warp_policy.train_steps,
                                   uniform_mix=warp_policy.uniform_mix, N_test=warp_policy.N_test,
                                   R=warp_policy.R, min_gain=warp_policy.min_gain)
            for gid, fit in zip(gids, fits):
                if fit.warp_id is None:
                    warps.pop(gid, None)
                else:
                    warps[gid] = fit.warp_id
        res = ses.run(_lib.QIW_GROUP_BOLD, top_bold, grid.tau(0), grid.tau(n), grid.tau(n + 1), precision, comm,
                      warps=warps)
        value, contribs, stds = _accumulate(res, top_bold, expansion.dims)
        _ppgf.set_ppgf(expansion.P, n + 1, value)
        _ppgf.normalize_tau(expansion.P, n + 1)  # suppress exponential growth (src/inchworm.jl:488)
        for o in contribs:
            for s, (sf, m) in contribs[o].items():
                P_orders[o][s].data[n + 1] = m
                P_orders_std[o][s].data[n + 1] = stds[o][s][1]
        if step_callback is not None:
            step_callback(n)
    return P_orders, P_orders_std


def diff_inchworm(expansion, orders, N_samples: int, rand_params: Optional[RandomizationParams] = None,
                  dev: Optional[Device] = None, precision: int = _lib.QIW_PREC_FP64, comm: Comm = Comm(),
                  seq_offset: int = 0):
    """diff_inchworm!(expansion, grid, orders, N_samples; rand_params) (src/inchworm.jl:666-786).

    Differential inchworm: at every grid point tau_n the pseudo-particle self-energy
    Sigma(tau_n) is the sum over orders k >= 1 of the diagrams with PairNodes at tau_0 and tau_n
    (one launch of QIW_GROUP_SIGMA groups, src/inchworm.jl:529-616); then (host, FP64)
    conv = -i h sum_j w_j Sigma(tau_n - tau_j) P(tau_j) (trapezoid; Keldysh's integrate on the
    imaginary branch) and P(tau_{n+1}) = P(tau_n) + h (conv - H P(tau_n)), H_s = diag(E_s + lambda)
    (src/inchworm.jl:618-634).  With spline-interpolated P the stored Sigma lags one grid point,
    as the reference's incremental-spline container does (it is created holding the tau_0
    point, src/spline_gf.jl:333-336).  Writes expansion.P; returns (Sigma_orders,
    Sigma_orders_std): order -> per-sector ImaginaryTimeGF."""
    assert N_samples == 0 or (N_samples & (N_samples - 1)) == 0, "N_samples must be a power of 2"
    rp = rand_params or RandomizationParams()
    assert rp.N_seqs > 0
    grid = expansion.grid
    ses = _Session(dev, expansion, seq_offset)
    top_data = []
    for o in orders:
        if o == 0:
            continue   # no 0-th order contribution to the self-energy
        tops = get_topologies_at_order(o, 1)
        if tops:
            top_data.append(TopologiesInputData(o, 1, tops, N_samples, rp))
    sig_orders = {td.order: _zero_P(expansion) for td in top_data}
    sig_orders_std = {td.order: _zero_P(expansion) for td in top_data}
    H = [np.diag(P0.E).astype(np.complex128) for P0 in expansion.P0]
    spline = bool(getattr(expansion, "interpolate_ppgf", False))
    sigma = [np.zeros_like(P_s.data) for P_s in expansion.P]
    h = grid.step
    dims = expansion.dims
    for n in range(0, grid.n_tau - 1):
        ses.dev.set_ppgf(expansion.P)
        res = ses.run(_lib.QIW_GROUP_SIGMA, top_data, grid.tau(0), 0.0, grid.tau(n), precision, comm)
        value, contribs, stds = _accumulate(res, top_data, dims)
        j_store = n + 1 if spline else n
        if j_store < grid.n_tau:
            for s, (sf, m) in value.items():
                sigma[s][j_store] = m
        new = {}
        w = np.ones(n + 1)
        w[0] = w[n] = 0.5
        if n == 0:
            w[0] = 0.0
        for s, P_s in enumerate(expansion.P):
            P_prev = P_s.data[n]
            # sum_j w_j Sigma(tau_n - tau_j) P(tau_j), j = 0..n, as one batched product
            prods = np.matmul(sigma[s][n::-1], P_s.data[:n + 1])
            conv = -1j * h * np.tensordot(w, prods, axes=(0, 0))
            new[s] = (s, P_prev + h * (conv - H[s] @ P_prev))
        _ppgf.set_ppgf(expansion.P, n + 1, new)
        for o in contribs:
            for s, (sf, m) in contribs[o].items():
                sig_orders[o][s].data[n + 1] = m
                sig_orders_std[o][s].data[n + 1] = stds[o][s][1]
    return sig_orders, sig_orders_std


def correlator_2p(expansion, orders, N_samples: int, rand_params: Optional[RandomizationParams] = None,
                  dev: Optional[Device] = None, precision: int = _lib.QIW_PREC_FP64, comm: Comm = Comm(),
                  seq_offset: int = 0,
                  request_std: bool = False, taus: Optional[Sequence[int]] = None):
    """correlator_2p(expansion, grid, orders, N_samples[, RequestStdDev()]).

    Returns one array of <A(tau) B(0)> values on the grid per registered (A, B) pair (and the
    standard deviations when request_std).  All correlators, tau points and groups run in a
    single launch: with P final, they are independent (src/inchworm.jl:1003-1045 loops over
    them one by one)."""
    assert N_samples == 0 or (N_samples & (N_samples - 1)) == 0, "N_samples must be a power of 2"
    rp = rand_params or RandomizationParams()
    grid = expansion.grid
    ses = _Session(dev, expansion, seq_offset)
    ses.dev.set_ppgf(expansion.P)
    top_data = []
    for o in orders:
        rng = [0] if o == 0 else range(1, 2 * o)
        for npa in rng:
            tops = get_topologies_at_order(o, npa, with_external_arc=True)
            if tops:
                top_data.append(TopologiesInputData(o, npa, tops, N_samples, rp))
    Z = _ppgf.partition_function(expansion.P)
    idx = list(range(grid.n_tau)) if taus is None else list(taus)
    n_c = len(expansion.corr_operators)
    # one launch for every (correlator, tau point, group): with P final they are independent
    all_tds, spans, per_tau, corrs = [], [], [], []
    for c in range(n_c):
        A, B = expansion.corr_operators[c]
        assert A.is_single_monomial(), "Operator A must be a single monomial in C/C^+"
        assert B.is_single_monomial(), "Operator B must be a single monomial in C/C^+"
        for q, j in enumerate(idx):
            tds = top_data[:1] if j == 0 else top_data
            if j == 0 and top_data[0].order != 0:
                tds = []
            spans.append((q, j, len(all_tds), len(tds)))
            all_tds += tds
            per_tau.append((grid.tau(0), grid.tau(j), grid.tau(grid.n_tau - 1)))
            corrs.append(c)
    works_res = _run_multi_tau(ses, all_tds, spans, per_tau, precision, comm, corrs)
    gs = [np.zeros(len(idx), np.complex128) for _ in range(n_c)]
    stds = [np.zeros(len(idx)) for _ in range(n_c)]
    for (q, j, a, n), c, r in zip(spans, corrs, works_res):
        val, sd = 0j, 0.0
        for mean, std, td in r:   # result += order_contrib, result_std += order_contrib_std
            val += mean
            if td.order > 0:
                sd += std
        gs[c][q] = val / Z
        stds[c][q] = sd / Z.real
    return (gs, stds) if request_std else gs


def _run_multi_tau(ses: _Session, all_tds, spans, times, precision, comm, corrs):
    """Runs the correlator groups of every span (correlator corrs[i], one tau point) in one
    qiw_integrate call.  The randomized quantity is the trace of the group's result, as in the
    reference's tr(eval(...)) integrand (src/inchworm.jl:861-879).  Returns per span a list of
    (mean trace, std of the trace, TopologiesInputData)."""
    dims = [int(d) for d in ses.exp.dims]
    offs = np.concatenate([[0], np.cumsum([d * d for d in dims])[:-1]]).astype(int)
    diag = np.array([o + k * d + k for o, d in zip(offs, dims) for k in range(d)], dtype=np.int64)
    entries = []   # (span, td index, gid, D) in the reference's order: correlator, tau, group
    for si, (q, j, a, n) in enumerate(spans):
        for k in range(n):
            td = all_tds[a + k]
            if td.order > 0 and td.N_samples <= 0:
                continue
            entries.append((si, a + k, ses.group(_lib.QIW_GROUP_CORRELATOR, td, corrs[si]), 2 * td.order))

    def launch(items):
        works, index = [], []
        for i, seqs in items:
            si, ti, gid, D = entries[i]
            td = all_tds[ti]
            t_i, t_w, t_f = times[si]
            start, length = rank_sub_range(td.N_samples, comm) if D > 0 else (0, 1)
            if D > 0:
                start += ses.seq_offset
            for m, x0 in seqs:
                works.append(Work(gid, t_i, t_w, t_f, start, length, td.N_samples, m, x0))
                index.append(i)
        if not works:
            return {}
        if hasattr(ses.dev, "integrate_packed"):   # traces straight from the packed result
            tr = ses.dev.integrate_packed(works, precision)[:, diag].sum(axis=1)
        else:
            tr = np.array([sum(np.trace(b) for b in blocks) for blocks in ses.dev.integrate(works, precision)],
                          np.complex128)
        red = np.array([entries[i][3] > 0 for i in index])
        if red.any() and comm.size > 1:   # one all-reduce for every sampled work item of the launch
            tr[red] = comm.allreduce(np.ascontiguousarray(tr[red]))
        vals: Dict[int, List[np.ndarray]] = {}
        for i, t in zip(index, tr):
            vals.setdefault(i, []).append(np.array([t]))
        return vals

    stats = _randomized([(e[3], all_tds[e[1]].rand_params) for e in entries], ses.dev.sobol, launch,
                        lambda i, v: v)
    out = [[] for _ in spans]
    for e, (mean, std) in zip(entries, stats):
        out[e[0]].append((complex(mean[0]), float(std[0]), all_tds[e[1]]))
    return out
