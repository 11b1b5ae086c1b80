"""Many independent inchworm! solves in one device-resident launch queue (qiw_batch_* C ABI).

``inchworm_batch`` runs, for every expansion, what ``qiw.inchworm.inchworm`` runs for one --
the bare step tau_0 -> tau_1, then the bold steps with set_ppgf! and normalize!(P, tau)
(src/inchworm.jl:332-498) with one unscrambled Sobol sequence -- but all solves advance
together: each step is one persistent kernel over the tiles of every (solve, group) still
running, followed by the per-solve P update on the device.  The whole loop is launched as
one CUDA graph.  Solves may differ in model parameters, grids, orders and sample counts.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import List, Optional, Sequence, Union

import numpy as np

from . import _lib
from .diagrammatics import get_topologies_at_order
from .sobol import direction_numbers


@dataclass
class BatchResult:
    kernel_ms: float             # device time of the run (all steps of all solves)
    flops: float                 # algorithmic flops (planner counts)
    topology_samples: float      # (topology, qMC sample) evaluations
    threads: int                 # samples per tile
    grid: int                    # CTAs per evaluation launch
    persistent: bool
    graph_nodes: int
    n_plans: int                 # distinct group programs shared by the solves
    tiles_per_step: int
    tune_ms: List[float]         # autotuner step times: threads 32/64/128 x (persistent, one per tile)


class Batch:
    """Owns a qiw_batch: solves are added once, then run (repeatedly) on the device."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.qiw_batch_create(C.byref(h), device)
        if rc != _lib.QIW_OK:
            raise _lib.QiwError(rc, "qiw_batch_create failed (no CUDA device?)")
        self.h = h
        self._keep = []
        self.expansions = []
        self.max_D = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.qiw_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != _lib.QIW_OK:
            raise _lib.QiwError(rc, self.lib.qiw_batch_last_error(self.h).decode())

    def add(self, expansion, orders: Sequence[int], orders_bare: Sequence[int], N_samples: int,
            n_pts_after_max: Optional[int] = None, n_steps: Optional[int] = None) -> int:
        """Registers one inchworm! solve of ``expansion`` (its P is the initial P)."""
        assert N_samples > 0 and (N_samples & (N_samples - 1)) == 0, "N_samples must be a power of 2"
        grid = expansion.grid
        packed = _lib.PackedProblem(expansion)
        bare, bold, keep = [], [], [packed]
        for o in orders_bare:
            gd, k = _lib.pack_group(_lib.QIW_GROUP_BARE, o, 2 * o, get_topologies_at_order(o))
            bare.append(gd)
            keep.append(k)
            self.max_D = max(self.max_D, 2 * o)
        for o in sorted(orders):
            rng = [0] if o == 0 else range(1, min(2 * o - 1, n_pts_after_max or 2 * o) + 1)
            for npa in rng:
                tops = get_topologies_at_order(o, npa) if o else get_topologies_at_order(0)
                if not tops:
                    continue
                gd, k = _lib.pack_group(_lib.QIW_GROUP_BOLD, o, npa, tops)
                bold.append(gd)
                keep.append(k)
                self.max_D = max(self.max_D, 2 * o)
        bare_arr = (_lib.GroupDesc * max(1, len(bare)))(*bare)
        bold_arr = (_lib.GroupDesc * max(1, len(bold)))(*bold)
        taus = np.ascontiguousarray(grid.taus, dtype=np.float64)
        P0 = _lib.pack_ppgf(expansion.P)
        pd = packed.desc()
        steps = grid.n_tau - 2 if n_steps is None else min(grid.n_tau - 2, n_steps)
        sd = _lib.SolveDesc(C.pointer(pd), taus.ctypes.data, P0.ctypes.data, len(bare), len(bold),
                            bare_arr, bold_arr, N_samples, steps, 0)
        sid = C.c_int32()
        self._check(self.lib.qiw_batch_add(self.h, C.byref(sd), C.byref(sid)))
        self._keep.append((keep, bare_arr, bold_arr, taus, P0, pd))
        self.expansions.append(expansion)
        return sid.value

    def run(self, precision: int = _lib.QIW_PREC_FP64, graph: bool = True, autotune: bool = True) -> BatchResult:
        D = max(1, self.max_D)
        m = np.ascontiguousarray(direction_numbers(D), dtype=np.uint32)
        flags = (_lib.QIW_BATCH_GRAPH if graph else 0) | (_lib.QIW_BATCH_AUTOTUNE if autotune else 0)
        self._check(self.lib.qiw_batch_run(self.h, precision, flags, m.ctypes.data, D))
        st = _lib.BatchStats()
        self._check(self.lib.qiw_batch_stats_get(self.h, C.byref(st)))
        return BatchResult(st.kernel_ms, st.flops, st.topology_samples, st.threads, st.grid, bool(st.persistent),
                           st.graph_nodes, st.n_plans, int(st.n_tiles_bold), list(st.tune_ms))

    def P_table(self, sid: int) -> np.ndarray:
        """P of solve sid after the last run (complex), in the element order of _lib.pack_ppgf."""
        exp = self.expansions[sid]
        out = np.zeros(2 * sum(P_s.data.size for P_s in exp.P))
        self._check(self.lib.qiw_batch_get_P(self.h, sid, out.ctypes.data))
        return out.view(np.complex128)

    def store_P(self, sid: int):
        """Writes the solve's P back into its expansion (what inchworm! leaves in expansion.P)."""
        exp = self.expansions[sid]
        flat = self.P_table(sid)
        o = 0
        for P_s in exp.P:
            n_tau, d, _ = P_s.data.shape
            blk = flat[o:o + n_tau * d * d].reshape(n_tau, d, d)   # [tau][l][k], k fastest
            P_s.data[...] = np.transpose(blk, (0, 2, 1))
            o += n_tau * d * d


def solve_cost(n_tau: int, max_order: int, N_samples: int) -> float:
    """Relative cost of one solve for sharding: steps x samples x bold topologies per step
    (sum over orders k <= max_order of (2k - 1)!! topologies, each counted once per n_pts_after
    group it falls in is close enough for balancing)."""
    tops = sum(math.prod(range(2 * k - 1, 0, -2)) if k > 0 else 1 for k in range(max_order + 1))
    return float(max(n_tau - 1, 1)) * N_samples * tops


def shard_solves(costs: Sequence[float], rank: int, size: int) -> List[int]:
    """Indices of the solves rank `rank` of `size` runs: independent solves need no exchange, so
    they are dealt out whole (longest first, each to the rank with the least cost so far; ties to
    the lowest rank).  Every rank computes the same assignment from the same costs."""
    if size < 1 or not 0 <= rank < size:
        raise ValueError("rank must lie in 0..size-1")
    load = [0.0] * size
    mine: List[int] = []
    for i in sorted(range(len(costs)), key=lambda j: (-costs[j], j)):
        r = min(range(size), key=lambda q: (load[q], q))
        load[r] += costs[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def inchworm_batch(expansions: Sequence, orders: Union[Sequence[int], Sequence[Sequence[int]]],
                   orders_bare: Union[Sequence[int], Sequence[Sequence[int]]],
                   N_samples: Union[int, Sequence[int]], n_pts_after_max: Optional[int] = None,
                   precision: int = _lib.QIW_PREC_FP64, graph: bool = True, autotune: bool = True,
                   device: int = 0, batch: Optional[Batch] = None) -> BatchResult:
    """inchworm! for every expansion (orders, orders_bare and N_samples per solve or shared);
    each expansion.P holds its solve's bold propagator afterwards."""
    n = len(expansions)
    per = lambda x, scalar: [x] * n if scalar else list(x)
    orders_l = per(orders, len(orders) == 0 or np.isscalar(orders[0]))
    bare_l = per(orders_bare, len(orders_bare) == 0 or np.isscalar(orders_bare[0]))
    N_l = per(N_samples, np.isscalar(N_samples))
    b = batch or Batch(device)
    if not b.expansions:
        for exp, o, ob, N in zip(expansions, orders_l, bare_l, N_l):
            b.add(exp, o, ob, N, n_pts_after_max)
    res = b.run(precision, graph, autotune)
    for sid in range(n):
        b.store_P(sid)
    return res
