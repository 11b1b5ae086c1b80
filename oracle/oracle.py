"""CPU oracle driver -- TEST INFRASTRUCTURE ONLY (tests, smoke check, CPU-baseline leg).

Wraps the C restatement in `qiw_oracle.c` and restates, independently of the product's
host code, the parts of the reference around it:
  * topology generation and filtering          src/diagrammatics.jl:288-337
  * TopologyEvaluator fixed-node layouts        src/inchworm.jl:148-166, 261-269, 834-850
  * inchworm_step / inchworm_step_bare          src/inchworm.jl:123-304
  * inchworm! loop, set_ppgf!, normalize!       src/inchworm.jl:332-498, src/ppgf.jl:474-695
  * correlator_2p                               src/inchworm.jl:805-1052
  * IncrementalSpline extend!                    src/utility.jl:136-140
It consumes the problem data (ED blocks, atomic propagators, hybridisation tables) built by
`qiw.expansion`, which are inputs, not part of the path under test.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from typing import Callable, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqiw_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, no FP contraction so x86 and Arm agree bit for bit)."""
    src = os.path.join(HERE, "qiw_oracle.c")
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "qiw_oracle.h"))):
        cmd = ["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               "-o", LIB_PATH + ".tmp", src, "-lm"]
        subprocess.check_call(cmd, cwd=HERE)
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class _ScalarGF(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_tau", C.c_int), ("h", C.c_double),
                ("data", C.c_void_p), ("aux", C.c_void_p)]


class _PPGF(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_tau", C.c_int), ("n_valid", C.c_int),
                ("data", C.c_void_p), ("der", C.c_void_p)]


class _Problem(C.Structure):
    _fields_ = [("n_sectors", C.c_int), ("dims", C.c_void_p), ("sector_offset", C.c_void_p),
                ("beta", C.c_double), ("h", C.c_double), ("atomic_energies", C.c_void_p),
                ("P", C.c_void_p), ("n_ops", C.c_int), ("op_target", C.c_void_p),
                ("op_offset", C.c_void_p), ("op_values", C.c_void_p), ("identity_op", C.c_int),
                ("n_pairs", C.c_int), ("pair_op_i", C.c_void_p), ("pair_op_f", C.c_void_p),
                ("pair_prop", C.c_void_p), ("props", C.c_void_p)]


class _Group(C.Structure):
    _fields_ = [("order", C.c_int), ("use_bold", C.c_int), ("transform", C.c_int),
                ("d_before", C.c_int), ("d_after", C.c_int),
                ("t_i", C.c_double), ("t_w", C.c_double), ("t_f", C.c_double),
                ("n_fixed", C.c_int), ("fixed_pos", C.c_void_p), ("fixed_kind", C.c_void_p),
                ("fixed_op", C.c_void_p), ("fixed_time", C.c_void_p),
                ("n_top", C.c_int), ("top_pairs", C.c_void_p), ("top_parity", C.c_void_p),
                ("decay", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.qiwo_integrate.restype = C.c_int
        _lib.qiwo_integrate.argtypes = [C.POINTER(_Problem), C.POINTER(_Group), C.c_void_p, C.c_void_p,
                                        C.c_int64, C.c_int, C.c_void_p]
        _lib.qiwo_sobol_directions.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        _lib.qiwo_sobol_points.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
        _lib.qiwo_sobol_point_u32.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
        _lib.qiwo_natural_spline_M.argtypes = [C.c_int, C.c_double, C.c_void_p, C.c_void_p]
        _lib.qiwo_integrate_range.restype = C.c_int
        _lib.qiwo_integrate_range.argtypes = [C.POINTER(_Problem), C.POINTER(_Group), C.c_void_p, C.c_void_p,
                                              C.c_int64, C.c_int64, C.c_int64, C.c_void_p]
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------- Sobol

def sobol_directions(D: int) -> np.ndarray:
    import scipy
    path = os.path.join(os.path.dirname(scipy.__file__), "stats", "_sobol_direction_numbers.npz")
    with np.load(path) as f:
        poly = np.ascontiguousarray(f["poly"][:max(D, 1)].astype(np.int64))
        vinit = np.ascontiguousarray(f["vinit"][:max(D, 1)].astype(np.int64))
    m = np.zeros((max(D, 1), 32), dtype=np.uint32)
    lib().qiwo_sobol_directions(D, _ptr(poly), _ptr(vinit), vinit.shape[1], _ptr(m))
    return m[:D]


def sobol_points(m: np.ndarray, x0: Optional[np.ndarray], skip: int, n: int) -> np.ndarray:
    D = m.shape[0]
    m = np.ascontiguousarray(m, dtype=np.uint32)
    x0 = np.zeros(D, np.uint32) if x0 is None else np.ascontiguousarray(x0, dtype=np.uint32)
    out = np.zeros((n, D))
    lib().qiwo_sobol_points(D, _ptr(m), _ptr(x0), skip, n, _ptr(out))
    return out


def sobol_point_u32(m: np.ndarray, x0: Optional[np.ndarray], n: int) -> np.ndarray:
    """Point n (0-based) as UInt32 by the Gray-code closed form of next!'s recurrence."""
    D = m.shape[0]
    m = np.ascontiguousarray(m, dtype=np.uint32)
    x0 = np.zeros(D, np.uint32) if x0 is None else np.ascontiguousarray(x0, dtype=np.uint32)
    out = np.zeros(D, np.uint32)
    if lib().qiwo_sobol_point_u32(D, _ptr(m), _ptr(x0), n, _ptr(out)):
        raise ValueError("Sobol index beyond 2^32 - 1")
    return out


# --------------------------------------------------------------------------- topologies

def topologies(order: int, k: Optional[int] = None, with_external_arc: bool = False):
    out = []

    def rec(pairs, parity, unp):
        if not unp:
            out.append((tuple(pairs), parity))
            return
        for i in range(2, len(unp) + 1):
            rest = unp[1:i - 1] + unp[i:]
            rec(pairs + [(unp[0], unp[i - 1])], parity * (-1) ** i, rest)

    rec([], 1, list(range(1, 2 * order + 1)))
    if k is None:
        return out

    def cross(p, q):
        a1, b1 = sorted(p)
        a2, b2 = sorted(q)
        return a1 < a2 < b1 < b2 or a2 < a1 < b2 < b1

    def dk(top):
        con = [p for p in top if min(p) <= k < max(p)]
        dis = [p for p in top if not (min(p) <= k < max(p))]
        stack = list(con)
        while stack:
            pc = stack.pop()
            for i in range(len(dis) - 1, -1, -1):
                if cross(pc, dis[i]):
                    stack.append(dis.pop(i))
        return not dis

    out = [(t, p) for (t, p) in out if dk(t)]
    if with_external_arc:
        out = [(t, (-1) ** k * p) for (t, p) in out]
    return out


# --------------------------------------------------------------------------- problem

class OracleProblem:
    """Evaluator inputs packed for the C oracle; P is owned (and updated) here."""

    def __init__(self, exp):
        from qiw.gf import SplineInterpolatedGF
        ed = exp.ed
        self.exp = exp
        self.grid = exp.grid
        self.S = ed.n_sectors
        self.dims = np.array(ed.dims, dtype=np.int32)
        self.off = np.concatenate([[0], np.cumsum(self.dims)[:-1]]).astype(np.int32)
        self.E = np.ascontiguousarray(np.concatenate([p.E for p in exp.P0]))
        # operator list: 0 identity, then (op_i, op_f) per pair, then correlator (A, B) pairs
        ops = [exp.identity_mat]
        self.pair_op_i, self.pair_op_f = [], []
        for (oi, of) in exp.pair_operator_mat:
            self.pair_op_i.append(len(ops)); ops.append(oi)
            self.pair_op_f.append(len(ops)); ops.append(of)
        self.corr_ops = []
        for (A, B) in exp.corr_operators_mat:
            self.corr_ops.append((len(ops), len(ops) + 1))
            ops += [A, B]
        S = self.S
        tgt = -np.ones(len(ops) * S, dtype=np.int32)
        offs = np.zeros(len(ops) * S, dtype=np.int64)
        vals = []
        pos = 0
        for o, sbm in enumerate(ops):
            for s, (sf, blk) in sbm.items():
                tgt[o * S + s] = sf
                offs[o * S + s] = pos
                b = np.ascontiguousarray(blk, dtype=np.complex128)
                vals.append(b.ravel())
                pos += b.size
        self.op_target, self.op_offset = tgt, offs
        self.op_values = np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1, np.complex128))
        self.n_ops = len(ops)
        # scalar propagators
        self.props = (_ScalarGF * max(1, len(exp.pairs)))()
        self._keep = []
        h = self.grid.step
        for p, pair in enumerate(exp.pairs):
            g = pair.propagator
            spline = isinstance(g, SplineInterpolatedGF)
            data = np.ascontiguousarray((g.GF if spline else g).data[:, 0, 0], dtype=np.complex128)
            M = np.zeros_like(data)
            if spline:
                lib().qiwo_natural_spline_M(data.size, h, _ptr(data), _ptr(M))
            self._keep += [data, M]
            self.props[p] = _ScalarGF(1 if spline else 0, data.size, h, data.ctypes.data, M.ctypes.data)
        self.pair_prop = np.arange(len(exp.pairs), dtype=np.int32)
        self.pair_op_i = np.array(self.pair_op_i, dtype=np.int32)
        self.pair_op_f = np.array(self.pair_op_f, dtype=np.int32)
        # bold P state (independent copy)
        self.spline_P = bool(exp.interpolate_ppgf)
        self.P_data = [np.ascontiguousarray(P_s.data.copy()) for P_s in exp.P]
        n_tau = self.grid.n_tau
        if self.spline_P:
            from qiw.ppgf import initial_ppgf_derivative
            dP = initial_ppgf_derivative(ed, self.grid.beta)
            self.P_der = [np.zeros_like(d) for d in self.P_data]
            for s in range(S):
                self.P_der[s][0] = dP[s] * h
            self.n_valid = 1
        else:
            self.P_der = [np.zeros(1, np.complex128) for _ in range(S)]
            self.n_valid = n_tau

    # -- P maintenance (restated from src/ppgf.jl, src/utility.jl) --------------
    def set_ppgf(self, j_f: int, blocks: List[np.ndarray]):
        for s in range(self.S):
            if self.spline_P:
                assert self.n_valid == j_f
                self.P_data[s][j_f] = blocks[s]
                self.P_der[s][j_f] = 2 * (self.P_data[s][j_f] - self.P_data[s][j_f - 1]) - self.P_der[s][j_f - 1]
            else:
                self.P_data[s][j_f] = blocks[s]
        if self.spline_P:
            self.n_valid = j_f + 1

    def _normalize(self, lam: float):
        """normalize!(P_s, lambda); for the spline-wrapped P the first segment's derivative
        is rebuilt as der_data[1]/h - 1im*lambda*data[1] (src/ppgf.jl:689), which only
        feeds the spline bookkeeping: the evaluator reads P by linear interpolation of the
        grid data."""
        taus = self.grid.taus
        h = self.grid.step
        for s in range(self.S):
            if self.spline_P:
                n = self.n_valid
                self.P_data[s][:n] *= np.exp(-taus[:n] * lam)[:, None, None]
                d0 = self.P_der[s][0] / h - 1j * lam * self.P_data[s][0]
                self.P_der[s][0] = d0 * h
                for j in range(1, n):
                    self.P_der[s][j] = 2 * (self.P_data[s][j] - self.P_data[s][j - 1]) - self.P_der[s][j - 1]
            else:
                self.P_data[s] *= np.exp(-taus * lam)[:, None, None]

    def normalize_tau(self, j: int):
        tau = self.grid.tau(j)
        pmax = max(float(np.max(-np.imag(np.diag(self.P_data[s][j])))) for s in range(self.S))
        self._normalize(math.log(pmax) / tau)

    def normalize_beta(self):
        Z = self.partition_function()
        lam = np.log(Z) / self.grid.beta
        self._normalize(float(np.real(lam)) if np.imag(lam) == 0 else lam)

    def partition_function(self) -> complex:
        return complex(sum(1j * np.trace(self.P_data[s][-1]) for s in range(self.S)))

    # -- integration ----------------------------------------------------------
    def _problem(self):
        S = self.S
        Ps = (_PPGF * S)()
        for s in range(S):
            # The evaluator reads the bold P by linear interpolation of its grid data, also
            # when P carries incremental-spline interpolants (`kd.interpolate!` at
            # src/topology_eval.jl:368 works on the wrapped grid GF).
            Ps[s] = _PPGF(0, self.grid.n_tau, self.n_valid,
                          self.P_data[s].ctypes.data, self.P_der[s].ctypes.data)
        pb = _Problem(S, self.dims.ctypes.data, self.off.ctypes.data, self.grid.beta, self.grid.step,
                      self.E.ctypes.data, C.cast(Ps, C.c_void_p), self.n_ops,
                      self.op_target.ctypes.data, self.op_offset.ctypes.data, self.op_values.ctypes.data,
                      0, len(self.exp.pairs), self.pair_op_i.ctypes.data, self.pair_op_f.ctypes.data,
                      self.pair_prop.ctypes.data, C.cast(self.props, C.c_void_p))
        return pb, Ps

    def integrate(self, kind: str, order: int, n_pts_after: int, tops, t_i: float, t_w: float,
                  t_f: float, N: int, n_ranks: int = 1, m=None, x0=None, corr: Optional[int] = None,
                  sample_range=None, transform: str = "root", decay: float = 0.0):
        """One group: kind 'bold', 'bare', 'corr' or 'sigma'; returns per-sector diagonal blocks.
        Bare groups take transform 'root' (default), 'sort' or 'expmodel' (decay rate `decay`)."""
        n_pair_fixed = 0
        if kind == "bare":
            fixed = [(0, 2, 0, t_i), (2 * order + 1, 2, 0, t_f)]
            transform, d_before, d_after, use_bold = {"root": 0, "sort": 2, "expmodel": 3}[transform], 0, 0, 0
        elif kind == "sigma":
            # self-energy diagrams of diff_inchworm_step! (src/inchworm.jl:560-566): PairNodes
            # fixed at t_i and t_f, the 2k - 2 other vertices integrated over [t_i, t_f] (Root)
            fixed = [(0, 1, 0, t_i), (2 * order - 1, 1, 0, t_f)]
            transform, d_before, d_after, use_bold = 0, 0, 0, 1
            n_pair_fixed = 2
        else:
            d_after = n_pts_after
            d_before = 2 * order - n_pts_after
            if kind == "bold":
                fixed = [(0, 2, 0, t_i), (d_before + 1, 3, 0, t_w), (2 * order + 2, 2, 0, t_f)]
            else:
                A, B = self.corr_ops[corr]
                fixed = [(0, 4, B, t_i), (d_before + 1, 4, A, t_w), (2 * order + 2, 2, 0, t_f)]
            transform, use_bold = 1, 1
        fp = np.array([f[0] for f in fixed], np.int32)
        fk = np.array([f[1] for f in fixed], np.int32)
        fo = np.array([f[2] for f in fixed], np.int32)
        ft = np.array([f[3] for f in fixed], np.float64)
        tp = np.array([[v for p in t for v in p] for (t, _) in tops] or [[0]], dtype=np.int32)
        par = np.array([p for (_, p) in tops] or [1], dtype=np.int32)
        gr = _Group(order, use_bold, transform, d_before, d_after, t_i, t_w, t_f, len(fixed),
                    fp.ctypes.data, fk.ctypes.data, fo.ctypes.data, ft.ctypes.data, len(tops),
                    tp.ctypes.data, par.ctypes.data, decay)
        D = 2 * order - n_pair_fixed
        if m is None:
            m = sobol_directions(D) if D > 0 else np.zeros((1, 32), np.uint32)
        m = np.ascontiguousarray(m, dtype=np.uint32)
        x0 = np.zeros(max(D, 1), np.uint32) if x0 is None else np.ascontiguousarray(x0, dtype=np.uint32)
        out = np.zeros(int(np.sum(self.dims ** 2)), dtype=np.complex128)
        pb, _keep = self._problem()
        if sample_range is None:
            rc = lib().qiwo_integrate(C.byref(pb), C.byref(gr), _ptr(m), _ptr(x0), N, n_ranks, _ptr(out))
        else:
            first, count = sample_range
            rc = lib().qiwo_integrate_range(C.byref(pb), C.byref(gr), _ptr(m), _ptr(x0), first, count, N, _ptr(out))
        if rc == 2:
            raise AssertionError("A block off-diagonal contribution to a pseudo-particle propagator detected")
        if rc:
            raise RuntimeError(f"oracle error {rc}")
        blocks, o = [], 0
        for d in self.dims:
            blocks.append(out[o:o + d * d].reshape(d, d))
            o += d * d
        return blocks


# --------------------------------------------------------------------------- drivers

def inchworm(exp, orders, orders_bare, N_samples: int, n_pts_after_max: Optional[int] = None,
             n_ranks: int = 1, n_steps: Optional[int] = None):
    """inchworm! restated; returns the OracleProblem holding the final (un-normalised) P."""
    pb = OracleProblem(exp)
    grid = exp.grid
    S = pb.S
    # bare step tau_0 -> tau_1
    total = [np.zeros((d, d), np.complex128) for d in pb.dims]
    for order in orders_bare:
        tops = topologies(order)
        blk = pb.integrate("bare", order, 0, tops, grid.tau(0), 0.0, grid.tau(1), N_samples, n_ranks)
        total = [a + b for a, b in zip(total, blk)]
    pb.set_ppgf(1, total)
    groups = []
    for order in orders:
        rng = [0] if order == 0 else range(1, min(2 * order - 1, n_pts_after_max or 10 ** 9) + 1)
        for npa in rng:
            tops = topologies(order, npa)
            if tops:
                groups.append((order, npa, tops))
    last = grid.n_tau - 1 if n_steps is None else min(grid.n_tau - 1, 1 + n_steps)
    for n in range(1, last):
        t_i, t_w, t_f = grid.tau(0), grid.tau(n), grid.tau(n + 1)
        total = [np.zeros((d, d), np.complex128) for d in pb.dims]
        for (order, npa, tops) in groups:
            blk = pb.integrate("bold", order, npa, tops, t_i, t_w, t_f, N_samples, n_ranks)
            total = [a + b for a, b in zip(total, blk)]
        pb.set_ppgf(n + 1, total)
        pb.normalize_tau(n + 1)
    return pb


def diff_inchworm(exp, orders, N_samples: int, n_ranks: int = 1, conv_factor: complex = -1j, rand=None):
    """diff_inchworm! restated (src/inchworm.jl:529-786); returns (OracleProblem, Sigma tables),
    and with `rand` = (new_seq, N_seqs, target_std) also the per-step std of Sigma summed over
    orders (one packed vector per step); new_seq(D) makes (and draws) the next D-dimensional
    scrambled sequence (m, x0), the role of ScrambledSobolSeq(D; scramble_rng).

    Per step n (tau_f_prev = tau_n, tau_f = tau_{n+1}): Sigma(tau_n) = sum over orders k >= 1 of
    the self-energy diagrams (topologies with n_pts_after = 1, PairNodes at tau_0 and tau_n);
    conv = integral over [tau_0, tau_n] of Sigma(tau_n - tau) P(tau), trapezoid rule on the grid
    (Keldysh's integrate; its contour measure on the imaginary branch is `conv_factor` * h);
    P(tau_{n+1}) = P(tau_n) + h (conv - H P(tau_n)) with H_s = diag(E_s + lambda) (Euler,
    Delta tau = 1im * step = h).  No normalisation.  With spline-interpolated P the stored
    Sigma lags one grid point, as the reference's incremental-spline container does.

    Randomized (src/inchworm.jl:566-597): order 1 is evaluated exactly (no draws, std 0); order
    k >= 2 draws 2k-dimensional scrambled sequences one at a time (mean_std_from_randomization
    below) and the Root transform of the 2k - 2 integrated times reads the first 2k - 2
    coordinates of each."""
    pb = OracleProblem(exp)
    grid = exp.grid
    step_std = []
    S = pb.S
    h = grid.step
    groups = []
    for order in orders:
        if order == 0:
            continue
        tops = topologies(order, 1)
        if tops:
            groups.append((order, tops))
    H = [np.diag(P0.E).astype(np.complex128) for P0 in exp.P0]
    sigma = [np.zeros_like(d) for d in pb.P_data]
    for n in range(0, grid.n_tau - 1):
        t_i, t_prev = grid.tau(0), grid.tau(n)
        P_prev = [pb.P_data[s][n].copy() for s in range(S)]
        total = [np.zeros((d, d), np.complex128) for d in pb.dims]
        std_n = np.zeros(int(np.sum(pb.dims ** 2)))
        for (order, tops) in groups:
            if rand is None or order == 1:
                blk = pb.integrate("sigma", order, 1, tops, t_i, 0.0, t_prev, N_samples, n_ranks)
            else:
                new_seq, n_seqs, target = rand
                D = 2 * order - 2
                f = lambda m, x0, order=order, tops=tops: np.concatenate([b.ravel() for b in pb.integrate(
                    "sigma", order, 1, tops, t_i, 0.0, t_prev, N_samples, n_ranks, m=m[:D], x0=x0[:D])])
                mean, std = mean_std_from_randomization(f, lambda order=order: new_seq(2 * order), n_seqs, target)
                std_n = std_n + std.real
                blk, o = [], 0
                for d in pb.dims:
                    blk.append(mean[o:o + d * d].reshape(d, d))
                    o += d * d
            total = [a + b for a, b in zip(total, blk)]
        step_std.append(std_n)
        # set_ppgf!(Sigma, tau_i, tau_n, .): with spline-interpolated P, Sigma = zero(P) is an
        # incremental spline whose interpolant already holds the tau_0 point, so extend! stores
        # the value one grid point later (src/ppgf.jl:474-482, src/spline_gf.jl:333-336, 377-386)
        j_store = n + 1 if pb.spline_P else n
        if j_store < grid.n_tau:
            for s in range(S):
                sigma[s][j_store] = total[s]
        new = []
        for s in range(S):
            conv = np.zeros_like(P_prev[s])
            for j in range(0, n + 1):
                w = 0.5 if (j == 0 or j == n) else 1.0
                if n == 0:
                    w = 0.0
                conv = conv + w * (sigma[s][n - j] @ pb.P_data[s][j])
            conv = conv_factor * h * conv
            rhs = conv - H[s] @ P_prev[s]
            new.append(P_prev[s] + h * rhs)
        pb.set_ppgf(n + 1, new)
    return (pb, sigma) if rand is None else (pb, sigma, step_std)


def correlator_2p(pb: OracleProblem, orders, N_samples: int, n_ranks: int = 1,
                  taus: Optional[Sequence[int]] = None) -> List[np.ndarray]:
    """correlator_2p restated (src/inchworm.jl:918-1052); P must be final."""
    grid = pb.grid
    groups = []
    for order in orders:
        rng = [0] if order == 0 else range(1, 2 * order)
        for npa in rng:
            tops = topologies(order, npa, with_external_arc=True)
            if tops:
                groups.append((order, npa, tops))
    Z = pb.partition_function()
    out = []
    idx = list(range(grid.n_tau)) if taus is None else list(taus)
    for c in range(len(pb.corr_ops)):
        g = np.zeros(len(idx), dtype=np.complex128)
        for q, j in enumerate(idx):
            if j == 0:
                use = [grp for grp in groups[:1] if grp[0] == 0]
            else:
                use = groups
            val = 0j
            for (order, npa, tops) in use:
                blk = pb.integrate("corr", order, npa, tops, grid.tau(0), grid.tau(j), grid.tau(grid.n_tau - 1),
                                   N_samples, n_ranks, corr=c)
                val += sum(np.trace(b) for b in blk)
            g[q] = val / Z
        out.append(g)
    return out


def mean_std_from_randomization(f: Callable, new_seq: Callable, N_seqs: int, target_std: float):
    """mean_std_from_randomization restated (src/randomization.jl:86-100).

    new_seq() plays the sequence constructor seq_type(D; scramble_rng): every call makes (and,
    scrambled, draws) the next sequence (m, x0); f(m, x0) is the quantity of one sequence.  The
    loop stops after sequence s > 1 once norm(std(samples), Inf) <= target_std; std is Julia's
    corrected std (NaN for one sample)."""
    samples = []
    for s in range(1, N_seqs + 1):
        m, x0 = new_seq()
        samples.append(np.atleast_1d(np.asarray(f(m, x0), dtype=np.complex128)).ravel())
        if s > 1 and np.max(np.std(np.array(samples), axis=0, ddof=1)) <= target_std:
            break
    a = np.array(samples)
    return a.mean(axis=0), (a.std(axis=0, ddof=1) if len(a) > 1 else np.full(a.shape[1], np.nan))
