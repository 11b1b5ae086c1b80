"""ctypes binding of the C ABI declared in include/qiw.h (the Python stand-in for the Julia
`ccall` wrappers)."""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

QIW_OK = 0
QIW_ERR_ARG = 1
QIW_ERR_CUDA = 2
QIW_ERR_UNSUPPORTED = 3
QIW_ERR_OFFDIAG = 4
QIW_ERR_DEVICE = 5
QIW_ERR_MEMORY = 6

QIW_PROP_LINEAR = 0
QIW_PROP_CUBIC = 1

QIW_GROUP_BOLD = 0
QIW_GROUP_BARE = 1
QIW_GROUP_CORRELATOR = 2
QIW_GROUP_SIGMA = 3

QIW_PREC_FP64 = 0
QIW_PREC_FP32 = 1
QIW_PREC_FP32_TC = 2
QIW_TRANSFORM_DEFAULT = 0
QIW_TRANSFORM_SORT = 1
QIW_TRANSFORM_EXPMODEL = 2

EXPORTS = ["qiw_ctx_create", "qiw_ctx_destroy", "qiw_last_error", "qiw_problem_set", "qiw_ppgf_set",
           "qiw_group_create", "qiw_group_stats_get", "qiw_integrate", "qiw_last_kernel_ms",
           "qiw_measure_fma_peak", "qiw_integrate_noalloc", "qiw_warp_create", "qiw_warp_set_mix", "qiw_warp_n_params",
           "qiw_warp_get_params", "qiw_warp_set_params", "qiw_warp_grad", "qiw_warp_train", "qiw_warp_map",
           "qiw_integrate_warped", "qiw_integrate_samples", "qiw_batch_create", "qiw_batch_destroy",
           "qiw_batch_last_error", "qiw_batch_add", "qiw_batch_run", "qiw_batch_get_P", "qiw_batch_stats_get",
           "qiw_plan_cache_info", "qiw_plan_cache_clear", "qiw_sobol_points", "qiw_warp_train_batch",
           "qiw_integrate_samples_batch", "qiw_integrate_sample_norms"]

QIW_BATCH_GRAPH = 1
QIW_BATCH_AUTOTUNE = 2


class ProblemDesc(C.Structure):
    _fields_ = [("n_sectors", C.c_int32), ("sector_dims", C.c_void_p), ("beta", C.c_double),
                ("n_tau", C.c_int32), ("atomic_energies", C.c_void_p), ("n_ops", C.c_int32),
                ("op_n_blocks", C.c_void_p), ("op_blocks", C.c_void_p), ("op_value_offset", C.c_void_p),
                ("op_values", C.c_void_p), ("identity_op", C.c_int32), ("n_pairs", C.c_int32),
                ("pair_ops", C.c_void_p), ("pair_prop_kind", C.c_void_p), ("pair_prop_data", C.c_void_p)]


class GroupDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("order", C.c_int32), ("n_pts_after", C.c_int32),
                ("corr_A_op", C.c_int32), ("corr_B_op", C.c_int32), ("n_topologies", C.c_int32),
                ("top_pairs", C.c_void_p), ("top_parity", C.c_void_p)]


class GroupStats(C.Structure):
    _fields_ = [("n_nodes_dag", C.c_int64), ("n_instructions", C.c_int64), ("arena_elements", C.c_int64),
                ("flops_per_sample", C.c_double), ("tree_flops_per_sample", C.c_double),
                ("n_leaves_tree", C.c_int64)]


class WorkDesc(C.Structure):
    _fields_ = [("group", C.c_int32), ("transform", C.c_int32), ("t_i", C.c_double), ("t_w", C.c_double),
                ("t_f", C.c_double), ("first_index", C.c_uint64), ("n_samples", C.c_uint64),
                ("n_total", C.c_uint64), ("sobol_m", C.c_void_p), ("sobol_x0", C.c_void_p)]


_lib = None


class SolveDesc(C.Structure):
    _fields_ = [("problem", C.POINTER(ProblemDesc)), ("taus", C.c_void_p), ("P_init", C.c_void_p),
                ("n_bare", C.c_int32), ("n_bold", C.c_int32), ("bare", C.POINTER(GroupDesc)),
                ("bold", C.POINTER(GroupDesc)), ("n_samples", C.c_uint64), ("n_steps", C.c_int32),
                ("reserved", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("flops", C.c_double), ("topology_samples", C.c_double),
                ("threads", C.c_int32), ("grid", C.c_int32), ("persistent", C.c_int32),
                ("n_steps_max", C.c_int32), ("graph_nodes", C.c_int32), ("n_plans", C.c_int32),
                ("n_tiles_bold", C.c_int64), ("n_tiles_bare", C.c_int64), ("tune_ms", C.c_double * 6)]


def load(path: Optional[str] = None) -> C.CDLL:
    """Load (building first if needed) libqiw.so; raises if the extension is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None:
        path = _build.build()
    lib = C.CDLL(path)
    lib.qiw_ctx_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    lib.qiw_ctx_destroy.argtypes = [C.c_void_p]
    lib.qiw_ctx_destroy.restype = None
    lib.qiw_last_error.argtypes = [C.c_void_p]
    lib.qiw_last_error.restype = C.c_char_p
    lib.qiw_problem_set.argtypes = [C.c_void_p, C.POINTER(ProblemDesc)]
    lib.qiw_ppgf_set.argtypes = [C.c_void_p, C.c_void_p]
    lib.qiw_group_create.argtypes = [C.c_void_p, C.POINTER(GroupDesc), C.POINTER(C.c_int32)]
    lib.qiw_group_stats_get.argtypes = [C.c_void_p, C.c_int32, C.POINTER(GroupStats)]
    lib.qiw_plan_cache_info.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.qiw_plan_cache_clear.argtypes = []
    lib.qiw_integrate.argtypes = [C.c_void_p, C.c_int32, C.POINTER(WorkDesc), C.c_int32, C.c_void_p]
    lib.qiw_last_kernel_ms.argtypes = [C.c_void_p]
    lib.qiw_last_kernel_ms.restype = C.c_double
    lib.qiw_measure_fma_peak.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]
    lib.qiw_sobol_points.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64,
                                     C.c_void_p]
    lib.qiw_integrate_noalloc.argtypes = [C.c_void_p, C.c_int32, C.POINTER(WorkDesc), C.c_int32, C.c_void_p]
    lib.qiw_warp_create.argtypes = [C.c_void_p, C.c_int32, C.c_uint64, C.POINTER(C.c_int32)]
    lib.qiw_warp_set_mix.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    lib.qiw_warp_n_params.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]
    lib.qiw_warp_get_params.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
    lib.qiw_warp_set_params.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
    lib.qiw_warp_grad.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                  C.POINTER(C.c_double)]
    lib.qiw_warp_train.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                                   C.c_double, C.POINTER(C.c_double)]
    lib.qiw_warp_map.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p]
    lib.qiw_integrate_warped.argtypes = [C.c_void_p, C.c_int32, C.POINTER(WorkDesc), C.c_void_p, C.c_int32,
                                         C.c_void_p]
    lib.qiw_integrate_samples.argtypes = [C.c_void_p, C.POINTER(WorkDesc), C.c_int32, C.c_void_p, C.c_void_p]
    lib.qiw_integrate_samples_batch.argtypes = [C.c_void_p, C.c_int32, C.POINTER(WorkDesc), C.c_int32, C.c_void_p,
                                                C.c_void_p]
    lib.qiw_integrate_sample_norms.argtypes = [C.c_void_p, C.c_int32, C.POINTER(WorkDesc), C.c_int32, C.c_void_p,
                                               C.c_void_p]
    lib.qiw_warp_train_batch.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int32, C.c_int32, C.c_double, C.c_void_p]
    lib.qiw_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    lib.qiw_batch_destroy.argtypes = [C.c_void_p]
    lib.qiw_batch_destroy.restype = None
    lib.qiw_batch_last_error.argtypes = [C.c_void_p]
    lib.qiw_batch_last_error.restype = C.c_char_p
    lib.qiw_batch_add.argtypes = [C.c_void_p, C.POINTER(SolveDesc), C.POINTER(C.c_int32)]
    lib.qiw_batch_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32]
    lib.qiw_batch_get_P.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
    lib.qiw_batch_stats_get.argtypes = [C.c_void_p, C.POINTER(BatchStats)]
    _lib = lib
    return lib


class QiwError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"qiw error {code}: {msg}")
        self.code = code


# --------------------------------------------------------------------------- packing

class PackedProblem:
    """Flattens an Expansion into the arrays of qiw_problem_desc (operator list:
    identity, then (operator_i, operator_f) per pair, then (A, B) per correlator pair)."""

    def __init__(self, exp):
        from .gf import SplineInterpolatedGF
        ed = exp.ed
        self.S = ed.n_sectors
        self.dims = np.array(ed.dims, dtype=np.int32)
        ops = [exp.identity_mat]
        self.identity_op = 0
        pair_ops = []
        for (oi, of) in exp.pair_operator_mat:
            pair_ops += [len(ops), len(ops) + 1]
            ops += [oi, of]
        self.corr_ops = []
        for (A, B) in exp.corr_operators_mat:
            self.corr_ops.append((len(ops), len(ops) + 1))
            ops += [A, B]
        self.n_ops = len(ops)
        nb, blocks, offs, vals = [], [], [], []
        pos = 0
        for sbm in ops:
            nb.append(len(sbm))
            for s_i in sorted(sbm):
                s_f, m = sbm[s_i]
                blocks += [s_i, s_f]
                offs.append(pos)
                col = np.asarray(m, dtype=np.complex128).ravel(order="F")
                vals.append(col)
                pos += col.size
        self.op_n_blocks = np.array(nb, dtype=np.int32)
        self.op_blocks = np.array(blocks or [0], dtype=np.int32)
        self.op_value_offset = np.array(offs or [0], dtype=np.int64)
        v = np.concatenate(vals) if vals else np.zeros(1, np.complex128)
        self.op_values = np.ascontiguousarray(np.stack([v.real, v.imag], axis=-1).ravel())
        self.pair_ops = np.array(pair_ops or [0], dtype=np.int32)
        kinds, data = [], []
        for pair in exp.pairs:
            g = pair.propagator
            spline = isinstance(g, SplineInterpolatedGF)
            kinds.append(1 if spline else 0)
            y = (g.GF if spline else g).data[:, 0, 0]
            data.append(np.stack([y.real, y.imag], axis=-1).ravel())
        self.pair_prop_kind = np.array(kinds or [0], dtype=np.int32)
        self.pair_prop_data = np.ascontiguousarray(np.concatenate(data) if data else np.zeros(2))
        self.E = np.ascontiguousarray(np.concatenate([p.E for p in exp.P0]))
        self.beta = exp.grid.beta
        self.n_tau = exp.grid.n_tau
        self.n_pairs = len(exp.pairs)

    def desc(self) -> ProblemDesc:
        p = lambda a: a.ctypes.data
        return ProblemDesc(self.S, p(self.dims), self.beta, self.n_tau, p(self.E), self.n_ops,
                           p(self.op_n_blocks), p(self.op_blocks), p(self.op_value_offset), p(self.op_values),
                           self.identity_op, self.n_pairs, p(self.pair_ops), p(self.pair_prop_kind),
                           p(self.pair_prop_data))


def pack_ppgf(P) -> np.ndarray:
    """expansion.P -> concatenated d x d x n_tau column-major complex blocks (Julia layout)."""
    parts = []
    for P_s in P:
        data = P_s.data  # [n_tau][d][d]
        jl = np.transpose(data, (0, 2, 1))  # [n_tau][l][k]: k fastest == column-major (k,l) per tau
        parts.append(np.ascontiguousarray(jl).ravel())
    v = np.concatenate(parts)
    return np.ascontiguousarray(np.stack([v.real, v.imag], axis=-1).ravel())


def pack_group(kind: int, order: int, n_pts_after: int, tops, corr=None):
    """Topologies (qiw.diagrammatics.Topology or (pairs, parity)) -> GroupDesc + keep-alive."""
    pairs, par = [], []
    for t in tops:
        if hasattr(t, "pairs"):
            pp, pr = t.pairs, t.parity
        else:
            pp, pr = t
        for (a, b) in pp:
            pairs += [a, b]
        par.append(pr)
    tp = np.array(pairs or [0], dtype=np.int32)
    pa = np.array(par or [1], dtype=np.int32)
    A, B = corr if corr is not None else (-1, -1)
    d = GroupDesc(kind, order, n_pts_after, A, B, len(par), tp.ctypes.data, pa.ctypes.data)
    return d, (tp, pa)
