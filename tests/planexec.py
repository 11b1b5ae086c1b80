"""Test helper: runs a planned group program on the CPU with numpy (vectorised over samples).

It mirrors the instruction semantics of the CUDA kernel (csrc/qiw_kernels.cu) so the host
planner's DAG can be checked against the CPU oracle without a GPU.  It is only a checker:
the product path is the CUDA kernel, and nothing outside tests/ imports this module.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from qiw import _lib, build as qbuild
from qiw.sobol import ScrambledSobolSeq

INSTR = np.dtype([("op", "u1"), ("rows", "u1"), ("inner", "u1"), ("cols", "u1"), ("acc", "u1"),
                  ("flags", "u1"), ("pad", "u1", 2), ("dst", "<i4"), ("src", "<i4"), ("a", "<i4"), ("w", "<i4"), ("c", "<f8")])
PMJOB = np.dtype([("iv", "<i2"), ("s", "<i2"), ("off", "<i4")])
WJOB = np.dtype([("head", "<i2"), ("tail", "<i2"), ("pair", "<i2"), ("pad", "<i2"), ("off", "<i4")])

_plib = None


def plan_lib():
    global _plib
    if _plib is None:
        _plib = C.CDLL(qbuild.build_plan_host())
        _plib.qiwp_plan.restype = C.c_int
        _plib.qiwp_plan.argtypes = [C.POINTER(_lib.ProblemDesc), C.POINTER(_lib.GroupDesc), C.c_int64,
                                    C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    return _plib


class HostPlan:
    def __init__(self, packed: "_lib.PackedProblem", kind, order, n_pts_after, tops, corr=None,
                 arena_budget=8192):
        pd = packed.desc()
        gd, self._keep = _lib.pack_group(kind, order, n_pts_after, tops, corr)
        cap = [4096, 256, 256]
        while True:
            ins = np.zeros(cap[0], INSTR)
            pm = np.zeros(cap[1], PMJOB)
            wj = np.zeros(cap[2], WJOB)
            counts = np.zeros(3, np.int64)
            meta = np.zeros(64, np.int32)
            stats = np.zeros(5, np.float64)
            err = C.create_string_buffer(512)
            rc = plan_lib().qiwp_plan(C.byref(pd), C.byref(gd), C.c_int64(arena_budget),
                                      ins.ctypes.data, C.c_int64(cap[0]), pm.ctypes.data, C.c_int64(cap[1]),
                                      wj.ctypes.data, C.c_int64(cap[2]), counts.ctypes.data, meta.ctypes.data,
                                      stats.ctypes.data, err, 512)
            if rc == _lib.QIW_ERR_MEMORY and np.any(counts > np.array(cap)):
                cap = [int(max(a, b)) for a, b in zip(cap, counts)]
                continue
            if rc:
                raise _lib.QiwError(rc, err.value.decode())
            break
        self.ins, self.pm, self.wj = ins[:counts[0]], pm[:counts[1]], wj[:counts[2]]
        m = meta
        self.kind, self.order, self.n_nodes, self.D = int(m[0]), int(m[1]), int(m[2]), int(m[3])
        self.d_before, self.d_after, self.use_bold = int(m[4]), int(m[5]), int(m[6])
        self.arena, self.res_size, self.n_fixed = int(m[7]), int(m[8]), int(m[9])
        self.fixed_pos = [int(x) for x in m[10:10 + self.n_fixed]]
        self.fixed_time = [int(x) for x in m[14:14 + self.n_fixed]]
        self.var_pos = [int(x) for x in m[18:18 + self.D]]
        self.flops, self.tree_flops, self.tree_leaves, self.dag_nodes, self.batches = stats


def _lin(table, inv_h, dt):
    n = table.shape[0]
    x = dt * inv_h
    i = np.clip(np.floor(x).astype(np.int64), 0, n - 2)
    f = x - i
    return i, f


def execute(plan: HostPlan, exp, packed, P_tables, t_i, t_w, t_f, N, first=0, m=None, x0=None):
    """Returns the group's result blocks (list of complex d x d), like qiw_integrate."""
    S = packed.S
    dims = packed.dims
    h = exp.grid.step
    inv_h = 1.0 / h
    opv = packed.op_values[0::2]
    Ns = 1 if plan.D == 0 else N
    tm = np.zeros((plan.n_nodes, Ns))
    sel = [t_i, t_w, t_f]
    for p_, ts in zip(plan.fixed_pos, plan.fixed_time):
        tm[p_] = sel[ts]
    D = plan.D
    if D > 0:
        if m is None:
            from qiw.sobol import direction_numbers
            m = direction_numbers(D)
            x0 = np.zeros(D, np.uint32)
        u = np.zeros((D, Ns))
        for k in range(Ns):
            u[:, k] = np.ldexp(ScrambledSobolSeq.point_uint(m, x0, first + k).astype(np.float64), -32)
        if plan.kind in (1, 3):   # Root: bare and self-energy groups
            acc = np.power(u[0], 1.0 / D)
            u[0] = acc
            for i in range(2, D + 1):
                acc = acc * np.power(u[i - 1], 1.0 / (D - i + 1))
                u[i - 1] = acc
            u = t_i + u * (t_f - t_i)
        else:
            dg, dl = plan.d_after, plan.d_before
            acc = np.power(u[0], 1.0 / dg)
            u[0] = acc
            for i in range(2, dg + 1):
                acc = acc * np.power(u[i - 1], 1.0 / (dg - i + 1))
                u[i - 1] = acc
            u[:dg] = u[:dg] * (t_f - t_w) + t_w
            if dl > 0:
                acc = np.power(u[dg], 1.0 / dl)
                u[dg] = acc
                for i in range(dg + 2, D + 1):
                    acc = acc * np.power(u[i - 1], 1.0 / (D - i + 1))
                    u[i - 1] = acc
                u[dg:] = u[dg:] * (t_w - t_i) + t_i
        for j in range(D):
            tm[plan.var_pos[j]] = u[j]
    R = run_program(plan, exp, packed, P_tables, tm)
    tot = R.sum(axis=1)
    if D > 0:
        if plan.kind in (1, 3):
            J = math.prod([(t_f - t_i) / i for i in range(1, D + 1)])
        else:
            J = math.prod([(t_w - t_i) / i for i in range(1, plan.d_before + 1)] or [1.0]) * \
                math.prod([(t_f - t_w) / i for i in range(1, plan.d_after + 1)] or [1.0])
        scale = J / N
    else:
        scale = 1.0
    if plan.kind == 3:   # self-energy groups: +i * parity (2k - 2 integrated times)
        scale = -scale
    out = -1j * scale * tot
    blocks, o = [], 0
    for d in dims:
        blocks.append(out[o:o + d * d].reshape(d, d, order="F"))
        o += d * d
    return blocks



def run_program(plan: HostPlan, exp, packed, P_tables, tm: np.ndarray) -> np.ndarray:
    """The group's program at explicit node times tm[n_nodes][Ns]: per-sample real-phase sums
    R[res_size][Ns] (qiw_integrate returns -i * J/N * parity-signed sum over samples)."""
    Ns = tm.shape[1]
    dims = packed.dims
    h = exp.grid.step
    inv_h = 1.0 / h
    opv = packed.op_values[0::2]
    eoff = np.concatenate([[0], np.cumsum(dims)[:-1]])
    A = np.zeros((plan.arena, Ns))
    for job in plan.pm:
        iv, s, off = int(job["iv"]), int(job["s"]), int(job["off"])
        dt = np.maximum(tm[iv + 1] - tm[iv], 0.0)
        d = int(dims[s])
        if plan.use_bold:
            T = P_tables[s]  # [n_tau][d*d] column-major, i*P real
            i, f = _lin(T, inv_h, dt)
            lo, hi = T[i], T[i + 1]
            A[off:off + d * d] = (lo + f[:, None] * (hi - lo)).T
        else:
            E = packed.E[eoff[s]:eoff[s] + d]
            A[off:off + d] = np.exp(-np.outer(E, dt))
    for job in plan.wj:
        hd, tl, p, off = int(job["head"]), int(job["tail"]), int(job["pair"]), int(job["off"])
        dt = np.maximum(tm[tl] - tm[hd], 0.0)
        y = -packed.pair_prop_data[2 * p * exp.grid.n_tau + 1:2 * (p + 1) * exp.grid.n_tau:2]
        i, f = _lin(y, inv_h, dt)
        if packed.pair_prop_kind[p] == 0:
            A[off] = y[i] + f * (y[i + 1] - y[i])
        else:
            from qiw.gf import natural_cubic_second_derivatives
            M = natural_cubic_second_derivatives(y, h)
            s_ = 1 - f
            A[off] = s_ * y[i] + f * y[i + 1] + h * h / 6 * ((s_ ** 3 - s_) * M[i] + (f ** 3 - f) * M[i + 1])
    R = np.zeros((plan.res_size, Ns))
    for I in plan.ins:
        op, rows, inner, cols = int(I["op"]), int(I["rows"]), int(I["inner"]), int(I["cols"])
        dst, src, a, w, c, accf = int(I["dst"]), int(I["src"]), int(I["a"]), int(I["w"]), float(I["c"]), int(I["acc"])
        if op == 1:
            if inner:
                blk = np.zeros((rows * rows, Ns))
                for r in range(rows):
                    blk[r * rows + r] = c * A[a + r]
            else:
                blk = c * A[a:a + rows * rows]
            A[dst:dst + rows * rows] = blk
        elif op == 2:
            A[dst:dst + rows * cols] = c * opv[a:a + rows * cols][:, None]
        elif op == 3:
            Pm = A[a:a + rows * rows].reshape(rows, rows, Ns)       # [k][r]
            X = A[src:src + rows * cols].reshape(cols, rows, Ns)   # [j][k]
            Y = np.einsum("krn,jkn->jrn", Pm, X)
            A[dst:dst + rows * cols] = Y.reshape(rows * cols, Ns)
        elif op == 4:
            X = A[src:src + rows * cols].reshape(cols, rows, Ns)
            A[dst:dst + rows * cols] = (A[a:a + rows][None] * X).reshape(rows * cols, Ns)
        elif op == 5:
            O = opv[a:a + rows * inner].reshape(inner, rows)        # [k][r]
            X = A[src:src + inner * cols].reshape(cols, inner, Ns)
            Y = np.einsum("kr,jkn->jrn", O, X).reshape(rows * cols, Ns)
            coef = c * (A[w] if w >= 0 else 1.0)
            A[dst:dst + rows * cols] = (A[dst:dst + rows * cols] if accf else 0.0) + coef * Y
        elif op == 6:
            coef = c * (A[w] if w >= 0 else 1.0)
            A[dst:dst + rows * cols] = (A[dst:dst + rows * cols] if accf else 0.0) + coef * A[src:src + rows * cols]
        elif op == 7:
            R[a:a + rows * cols] += A[src:src + rows * cols]
        elif op == 9:   # 1x1 P multiply fused into its AXPY
            coef = c * (A[w] if w >= 0 else 1.0)
            A[dst] = (A[dst] if accf else 0.0) + coef * (A[a] * A[src])
        elif op == 8:
            A[dst:dst + rows * rows] = 0.0
            for r in range(rows):
                A[dst + r * rows + r] = c
        else:
            raise ValueError(f"bad opcode {op}")
    return R


def p_tables(exp):
    """i*P tables per sector in the device layout: [n_tau][d*d] column-major (real part)."""
    out = []
    for P_s in exp.P:
        data = P_s.data
        iP = -data.imag
        out.append(np.ascontiguousarray(np.transpose(iP, (0, 2, 1)).reshape(data.shape[0], -1)))
    return out
