"""Python host wrapper of one libqiw context (the role of the Julia `QInchwormGPU` ccall
layer): uploads an Expansion, plans topology groups and runs qMC integrals on the GPU."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .ed import SectorBlockMatrix
from .sobol import direction_numbers


@dataclass
class Work:
    group: int
    t_i: float
    t_w: float
    t_f: float
    first_index: int = 0
    n_samples: int = 0
    n_total: int = 0
    sobol_m: Optional[np.ndarray] = None
    sobol_x0: Optional[np.ndarray] = None
    transform: int = 0             # _lib.QIW_TRANSFORM_* (bare groups; EXPMODEL takes its decay rate from t_w)


class Device:
    """One qiw context on one CUDA device.  Raises if the CUDA extension or a GPU is missing."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.qiw_ctx_create(C.byref(h), device)
        if rc != _lib.QIW_OK:
            raise _lib.QiwError(rc, "qiw_ctx_create failed (no CUDA device?)")
        self.h = h
        self.packed: Optional[_lib.PackedProblem] = None
        self.group_info: Dict[int, Tuple[int, int, int]] = {}
        self._sobol_cache: Dict[int, np.ndarray] = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.qiw_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != _lib.QIW_OK:
            raise _lib.QiwError(rc, self.lib.qiw_last_error(self.h).decode())

    # -- problem ----------------------------------------------------------------
    def set_problem(self, exp) -> _lib.PackedProblem:
        self.packed = _lib.PackedProblem(exp)
        d = self.packed.desc()
        self._check(self.lib.qiw_problem_set(self.h, C.byref(d)))
        self.group_info.clear()
        return self.packed

    def set_ppgf(self, P) -> None:
        buf = _lib.pack_ppgf(P)
        self._check(self.lib.qiw_ppgf_set(self.h, buf.ctypes.data))

    def create_group(self, kind: int, order: int, n_pts_after: int, tops, corr: Optional[int] = None) -> int:
        ops = self.packed.corr_ops[corr] if corr is not None else None
        gd, keep = _lib.pack_group(kind, order, n_pts_after, tops, ops)
        gid = C.c_int32()
        self._check(self.lib.qiw_group_create(self.h, C.byref(gd), C.byref(gid)))
        self.group_info[gid.value] = (kind, order, n_pts_after)
        return gid.value

    def group_stats(self, gid: int) -> _lib.GroupStats:
        st = _lib.GroupStats()
        self._check(self.lib.qiw_group_stats_get(self.h, gid, C.byref(st)))
        return st

    def plan_cache_info(self) -> dict:
        """Entries, hits and host bytes of the process's plan cache (qiw_plan_cache_info)."""
        e, h, b = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.qiw_plan_cache_info(C.byref(e), C.byref(h), C.byref(b)))
        return {"entries": e.value, "hits": h.value, "bytes": b.value}

    def plan_cache_clear(self) -> None:
        self._check(self.lib.qiw_plan_cache_clear())

    def sobol(self, D: int) -> np.ndarray:
        if D not in self._sobol_cache:
            self._sobol_cache[D] = np.ascontiguousarray(direction_numbers(D), dtype=np.uint32)
        return self._sobol_cache[D]

    # -- integration --------------------------------------------------------------
    def _descs(self, works):
        descs = (_lib.WorkDesc * len(works))()
        keep = []
        for i, w in enumerate(works):
            kind, order, _ = self.group_info.get(w.group, (0, 0, 0))
            D = 2 * order - (2 if kind == _lib.QIW_GROUP_SIGMA else 0)   # integrated times
            m = w.sobol_m if w.sobol_m is not None else (self.sobol(D) if D else np.zeros((1, 32), np.uint32))
            x0 = w.sobol_x0 if w.sobol_x0 is not None else np.zeros(max(D, 1), np.uint32)
            m = np.ascontiguousarray(m, dtype=np.uint32)
            x0 = np.ascontiguousarray(x0, dtype=np.uint32)
            keep += [m, x0]
            descs[i] = _lib.WorkDesc(w.group, w.transform, w.t_i, w.t_w, w.t_f, w.first_index, w.n_samples,
                                     w.n_total or w.n_samples, m.ctypes.data, x0.ctypes.data)
        return descs, keep

    def _unpack(self, out, n):
        dims = self.packed.dims
        rs = int(np.sum(dims ** 2))
        res = []
        z = out[0::2] + 1j * out[1::2]
        for i in range(n):
            blocks, o = [], i * rs
            for d in dims:
                blocks.append(z[o:o + d * d].reshape(d, d, order="F").copy())
                o += d * d
            res.append(blocks)
        return res

    def integrate(self, works: Sequence[Work], precision: int = _lib.QIW_PREC_FP64,
                  warps: Optional[Sequence[int]] = None) -> List[List[np.ndarray]]:
        """Runs all work items in one launch; returns per item the list of sector blocks.
        `warps[i]` >= 0 evaluates item i on the points of that learned warp."""
        descs, keep = self._descs(works)
        dims = self.packed.dims
        rs = int(np.sum(dims ** 2))
        out = np.zeros(2 * rs * len(works))
        if warps is None:
            self._check(self.lib.qiw_integrate(self.h, len(works), descs, precision, out.ctypes.data))
        else:
            ids = np.ascontiguousarray(warps, dtype=np.int32)
            self._check(self.lib.qiw_integrate_warped(self.h, len(works), descs, ids.ctypes.data, precision,
                                                      out.ctypes.data))
        return self._unpack(out, len(works))

    def integrate_packed(self, works: Sequence[Work], precision: int = _lib.QIW_PREC_FP64) -> np.ndarray:
        """integrate() without unpacking: [n_work][sum d_s^2] complex, per work item the sector
        blocks in sector order, each column-major."""
        descs, keep = self._descs(works)
        rs = int(np.sum(self.packed.dims ** 2))
        out = np.zeros(2 * rs * len(works))
        self._check(self.lib.qiw_integrate(self.h, len(works), descs, precision, out.ctypes.data))
        return (out[0::2] + 1j * out[1::2]).reshape(len(works), rs)

    def integrate_samples(self, work: Work, precision: int = _lib.QIW_PREC_FP64):
        """One work item; returns (blocks, per-sample values [n_samples][sum d^2])."""
        descs, keep = self._descs([work])
        rs = int(np.sum(self.packed.dims ** 2))
        out = np.zeros(2 * rs)
        samples = np.zeros((work.n_samples, rs))
        self._check(self.lib.qiw_integrate_samples(self.h, descs, precision, out.ctypes.data, samples.ctypes.data))
        return self._unpack(out, 1)[0], samples

    def integrate_samples_batch(self, works: Sequence[Work], precision: int = _lib.QIW_PREC_FP64):
        """integrate_samples of several work items in one launch: (blocks per item, per-sample
        values per item [n_samples_i][sum d^2])."""
        descs, keep = self._descs(works)
        rs = int(np.sum(self.packed.dims ** 2))
        out = np.zeros(2 * rs * len(works))
        samples = np.zeros((sum(w.n_samples for w in works), rs))
        self._check(self.lib.qiw_integrate_samples_batch(self.h, len(works), descs, precision, out.ctypes.data,
                                                         samples.ctypes.data))
        cut = np.cumsum([0] + [w.n_samples for w in works])
        return self._unpack(out, len(works)), [samples[a:b] for a, b in zip(cut[:-1], cut[1:])]

    # -- learned warps --------------------------------------------------------------
    def warp_create(self, D: int, seed: int = 0, uniform_mix: Optional[float] = None) -> int:
        wid = C.c_int32()
        self._check(self.lib.qiw_warp_create(self.h, D, seed, C.byref(wid)))
        if uniform_mix is not None:
            self._check(self.lib.qiw_warp_set_mix(self.h, wid.value, uniform_mix))
        return wid.value

    def warp_params(self, wid: int) -> np.ndarray:
        n = C.c_int64()
        self._check(self.lib.qiw_warp_n_params(self.h, wid, C.byref(n)))
        p = np.zeros(n.value)
        self._check(self.lib.qiw_warp_get_params(self.h, wid, p.ctypes.data))
        return p

    def warp_set_params(self, wid: int, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self._check(self.lib.qiw_warp_set_params(self.h, wid, p.ctypes.data))

    def warp_grad(self, wid: int, x: np.ndarray, w: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        g = np.zeros_like(self.warp_params(wid))
        loss = C.c_double()
        self._check(self.lib.qiw_warp_grad(self.h, wid, x.ctypes.data, w.ctypes.data, len(w), g.ctypes.data,
                                           C.byref(loss)))
        return g, loss.value

    def warp_train(self, wid: int, x: np.ndarray, w: np.ndarray, steps: int = 400, batch: int = 4096,
                   lr: float = 3e-3) -> float:
        x = np.ascontiguousarray(x, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        loss = C.c_double()
        self._check(self.lib.qiw_warp_train(self.h, wid, x.ctypes.data, w.ctypes.data, len(w), steps, batch, lr,
                                            C.byref(loss)))
        return loss.value

    def integrate_sample_norms(self, works: Sequence[Work], precision: int = _lib.QIW_PREC_FP64):
        """integrate_samples_batch returning only each sample's value norm ||f_i||: (blocks per
        item, norms per item [n_samples_i])."""
        descs, keep = self._descs(works)
        rs = int(np.sum(self.packed.dims ** 2))
        out = np.zeros(2 * rs * len(works))
        norms = np.zeros(sum(w.n_samples for w in works))
        self._check(self.lib.qiw_integrate_sample_norms(self.h, len(works), descs, precision, out.ctypes.data,
                                                        norms.ctypes.data))
        cut = np.cumsum([0] + [w.n_samples for w in works])
        return self._unpack(out, len(works)), [norms[a:b] for a, b in zip(cut[:-1], cut[1:])]

    def warp_train_batch(self, wids: Sequence[int], xs: Sequence[np.ndarray], ws: Sequence[np.ndarray],
                         steps: int = 400, batch: int = 4096, lr: float = 3e-3) -> np.ndarray:
        """warp_train of several distinct warps at once (trained concurrently on the device);
        returns their final losses."""
        n = len(wids)
        xs = [np.ascontiguousarray(x, dtype=np.float64) for x in xs]
        ws = [np.ascontiguousarray(w, dtype=np.float64) for w in ws]
        ids = np.ascontiguousarray(wids, dtype=np.int32)
        xp = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        wp = (C.c_void_p * n)(*[w.ctypes.data for w in ws])
        cnt = np.ascontiguousarray([len(w) for w in ws], dtype=np.int64)
        loss = np.zeros(n)
        self._check(self.lib.qiw_warp_train_batch(self.h, n, ids.ctypes.data, C.cast(xp, C.c_void_p),
                                                  C.cast(wp, C.c_void_p), cnt.ctypes.data, steps, batch, lr,
                                                  loss.ctypes.data))
        return loss

    def warp_map(self, wid: int, D: int, first: int, n: int, m=None, x0=None) -> np.ndarray:
        m = np.ascontiguousarray(self.sobol(D) if m is None else m, dtype=np.uint32)
        x0 = np.ascontiguousarray(np.zeros(D, np.uint32) if x0 is None else x0, dtype=np.uint32)
        pts = np.zeros((n, D + 1))
        self._check(self.lib.qiw_warp_map(self.h, wid, m.ctypes.data, x0.ctypes.data, first, n, pts.ctypes.data))
        return pts

    def sobol_points(self, m: np.ndarray, x0: Optional[np.ndarray], first: int, n: int) -> np.ndarray:
        """The kernels' Sobol integers (qiw_sobol_points): uint32 array [n][D] of points
        first .. first + n - 1 for direction numbers m [D][32] and shift x0 [D]."""
        m = np.ascontiguousarray(m, dtype=np.uint32)
        D = m.shape[0]
        x0 = np.ascontiguousarray(np.zeros(D, np.uint32) if x0 is None else x0, dtype=np.uint32)
        out = np.zeros((n, D), np.uint32)
        self._check(self.lib.qiw_sobol_points(self.h, D, m.ctypes.data, x0.ctypes.data, first, n, out.ctypes.data))
        return out

    def fma_peak_tflops(self, precision: int = _lib.QIW_PREC_FP64) -> float:
        v = C.c_double()
        self._check(self.lib.qiw_measure_fma_peak(self.h, precision, C.byref(v)))
        return v.value

    def last_kernel_ms(self) -> float:
        return float(self.lib.qiw_last_kernel_ms(self.h))


def blocks_to_sbm(blocks: List[np.ndarray]) -> SectorBlockMatrix:
    return SectorBlockMatrix({s: (s, b) for s, b in enumerate(blocks)})
