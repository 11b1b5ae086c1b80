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

    def sobol(self, D: int) -> np.ndarray:
        if D not in self._sobol_cache:
            self._sobol_cache[D] = np.ascontiguousarray(direction_numbers(D), dtype=np.uint32)
        return self._sobol_cache[D]

    # -- integration --------------------------------------------------------------
    def integrate(self, works: Sequence[Work], precision: int = _lib.QIW_PREC_FP64) -> List[List[np.ndarray]]:
        """Runs all work items in one launch; returns per item the list of sector blocks."""
        descs = (_lib.WorkDesc * len(works))()
        keep = []
        for i, w in enumerate(works):
            order = self.group_info.get(w.group, (0, 0, 0))[1]
            D = 2 * order
            m = w.sobol_m if w.sobol_m is not None else (self.sobol(D) if D else np.zeros((1, 32), np.uint32))
            x0 = w.sobol_x0 if w.sobol_x0 is not None else np.zeros(max(D, 1), np.uint32)
            m = np.ascontiguousarray(m, dtype=np.uint32)
            x0 = np.ascontiguousarray(x0, dtype=np.uint32)
            keep += [m, x0]
            descs[i] = _lib.WorkDesc(w.group, 0, w.t_i, w.t_w, w.t_f, w.first_index, w.n_samples,
                                     w.n_total or w.n_samples, m.ctypes.data, x0.ctypes.data)
        dims = self.packed.dims
        rs = int(np.sum(dims ** 2))
        out = np.zeros(2 * rs * len(works))
        self._check(self.lib.qiw_integrate(self.h, len(works), descs, precision, out.ctypes.data))
        res = []
        z = out[0::2] + 1j * out[1::2]
        for i in range(len(works)):
            blocks, o = [], i * rs
            for d in dims:
                blocks.append(z[o:o + d * d].reshape(d, d, order="F").copy())
                o += d * d
            res.append(blocks)
        return res

    def fma_peak_tflops(self, precision: int = _lib.QIW_PREC_FP64) -> float:
        v = C.c_double()
        self._check(self.lib.qiw_measure_fma_peak(self.h, precision, C.byref(v)))
        return v.value

    def last_kernel_ms(self) -> float:
        return float(self.lib.qiw_last_kernel_ms(self.h))


def blocks_to_sbm(blocks: List[np.ndarray]) -> SectorBlockMatrix:
    return SectorBlockMatrix({s: (s, b) for s, b in enumerate(blocks)})
